"""Synthetic graph inputs.

* ``rmat``     -- the reference's R-MAT recipe (datasets/gen_rmat.py:15-44),
                  bit-identical: same ``default_rng(seed)`` stream, consumed level
                  by level, same quadrant rule, then symmetrised, self-loops
                  dropped and duplicates merged, no relabelling.  Draws are taken
                  in bounded chunks so memory stays at two uint32 arrays of m.
* ``er_directed`` -- directed Erdos-Renyi G(n, m = n * mean_degree) with
                  self-loops and duplicates removed (no counterpart in the
                  reference; construction stated in the docstring).
* ``grid2d``   -- the 4-neighbour side x side grid (no counterpart in the
                  reference).
All return preprocess.GraphArrays with A[dst, src] = 1 for an edge src -> dst.
"""
from __future__ import annotations

import numpy as np

from .preprocess import GraphArrays, from_edges

RMAT_A, RMAT_B, RMAT_C, RMAT_D = 0.57, 0.19, 0.19, 0.05


def rmat_edge_endpoints(scale, edgefactor, seed, A=RMAT_A, B=RMAT_B, C=RMAT_C,
                        chunk=1 << 23):
  """The raw R-MAT edge endpoints (u, v), before symmetrisation: m =
  2^scale * edgefactor pairs.  Level l of edge e uses the (l*m + e)-th double
  of default_rng(seed), exactly as gen_rmat.py draws rng.random(m) per level."""
  n = 1 << scale
  m = n * edgefactor
  dt = np.uint32 if scale <= 31 else np.uint64
  u = np.zeros(m, dtype=dt)
  v = np.zeros(m, dtype=dt)
  rng = np.random.default_rng(seed)
  ab, abc = A + B, A + B + C
  for level in range(scale):
    shift = scale - 1 - level
    for e0 in range(0, m, chunk):
      e1 = min(m, e0 + chunk)
      r = rng.random(e1 - e0)
      u[e0:e1] |= (r >= ab).astype(dt) << dt(shift)
      v[e0:e1] |= (((r >= A) & (r < ab)) | (r >= abc)).astype(dt) << dt(shift)
  return u, v


def rmat(scale, edgefactor, seed, A=RMAT_A, B=RMAT_B, C=RMAT_C) -> GraphArrays:
  """Symmetric, loop-free, deduplicated R-MAT graph (gen_rmat.py:15-44)."""
  n = 1 << scale
  u, v = rmat_edge_endpoints(scale, edgefactor, seed, A, B, C)
  return from_edges(n, u, v, symmetrize=True, drop_self_loops=True)


def er_directed(log2_n, mean_degree, seed) -> GraphArrays:
  """Directed G(n, m): m = n * mean_degree ordered pairs (src, dst) drawn
  uniformly from default_rng(seed) as ``rng.integers(0, n, size=(2, m))``
  (row 0 = src, row 1 = dst); self-loops and duplicate pairs are removed."""
  n = 1 << log2_n
  m = n * mean_degree
  rng = np.random.default_rng(seed)
  sd = rng.integers(0, n, size=(2, m), dtype=np.int64)
  return from_edges(n, sd[0], sd[1], symmetrize=False, drop_self_loops=True)


def grid2d(side) -> GraphArrays:
  """side x side 4-neighbour grid; vertex id = row * side + col; undirected
  (both directions stored).  Diameter 2 * (side - 1)."""
  n = side * side
  ids = np.arange(n, dtype=np.int64).reshape(side, side)
  src = np.concatenate([ids[:, :-1].ravel(), ids[:-1, :].ravel()])
  dst = np.concatenate([ids[:, 1:].ravel(), ids[1:, :].ravel()])
  return from_edges(n, src, dst, symmetrize=True)
