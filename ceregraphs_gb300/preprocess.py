"""Host-side graph preparation: the GB300 replacement of preprocess_bool.py.

The reference splits A into a P x P grid of hypersparse per-PE CSC blocks with
u16 indices (bfs/implementation/preprocess_bool.py:29-229).  One GB300 holds
the whole graph, so this module only produces the two arrays pairs the device
keeps resident, with the reference's sort invariants (preprocess_bool.py:67-72,
run_graph500.py:165-187: sorted CSR, sorted CSC):

* ``in_off/in_idx``   CSR of A: row r lists the sources c of edges c -> r
* ``out_off/out_idx`` CSC of A: column c lists the targets of c

For a symmetric A both are the same arrays and only one copy goes to the GPU.
Offsets are int64 (scale 26 has ~2.1e9 entries), indices int32.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
from scipy import sparse


@dataclass
class GraphArrays:
  n: int
  nnz: int
  in_off: np.ndarray
  in_idx: np.ndarray
  out_off: np.ndarray | None
  out_idx: np.ndarray | None
  symmetric: bool

  def scipy_csr(self):
    """A as a scipy CSR matrix (row = dst, col = src)."""
    return sparse.csr_matrix((np.ones(self.nnz, dtype=np.float32), self.in_idx, self.in_off),
                             shape=(self.n, self.n))

  def out_lists(self):
    if self.symmetric:
      return self.in_off, self.in_idx
    return self.out_off, self.out_idx


def is_symmetric(A_csr):
  """run_graph500.py:179: A == A^T structurally."""
  A = sparse.csr_matrix(A_csr)
  return (A != A.T).nnz == 0


def preprocess(A, symmetric=None):
  """Build the resident arrays from the reference's A (row = dst, col = src)."""
  A = sparse.csr_matrix(A)
  n0, n1 = A.shape
  if n0 != n1:
    raise ValueError("BFS needs a square adjacency matrix")
  A.sum_duplicates()
  A.sort_indices()
  if symmetric is None:
    symmetric = is_symmetric(A)
  in_off = A.indptr.astype(np.int64)
  in_idx = A.indices.astype(np.int32)
  if symmetric:
    return GraphArrays(n0, int(A.nnz), in_off, in_idx, None, None, True)
  C = A.tocsc()
  C.sort_indices()
  return GraphArrays(n0, int(A.nnz), in_off, in_idx, C.indptr.astype(np.int64),
                     C.indices.astype(np.int32), False)


def from_edges(n, src, dst, symmetrize=False, drop_self_loops=False):
  """Build GraphArrays from an edge list src -> dst (entries A[dst, src]),
  merging duplicates.  ``symmetrize`` stores both directions."""
  src = np.asarray(src, dtype=np.int64)
  dst = np.asarray(dst, dtype=np.int64)
  if symmetrize:
    src, dst = np.concatenate([src, dst]), np.concatenate([dst, src])
  if drop_self_loops:
    keep = src != dst
    src, dst = src[keep], dst[keep]
  key = dst * n + src
  key.sort()
  if len(key):
    key = key[np.concatenate(([True], key[1:] != key[:-1]))]
  rows = key // n
  cols = (key % n).astype(np.int32)
  in_off = np.zeros(n + 1, dtype=np.int64)
  np.cumsum(np.bincount(rows, minlength=n), out=in_off[1:])
  A = sparse.csr_matrix((np.ones(len(cols), dtype=np.float32), cols, in_off), shape=(n, n))
  return preprocess(A, symmetric=True if symmetrize else None)
