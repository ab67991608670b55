"""ORACLE -- test infrastructure, not product code.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module, and only as the checker.  The ceregraphs_gb300 package never
imports it, and its CUDA path has no route through it.

This is a CPU restatement of CereGraphs' host-side BFS path, one function per
reference routine (file:line cited on each):

* ``rmat``                  datasets/gen_rmat.py:15-44
* ``pick_sources``          bfs/scripts/run_graph500.py:106-127
* ``harmonic_mean``         bfs/scripts/run_graph500.py:130-134
* ``compute_m``             bfs/implementation/bfs_timing.py:379-398
* ``extract_parent_result`` bfs/implementation/device_io.py:157-178
* ``derive_visited``        bfs/implementation/device_io.py:181-205
* ``invalid_parents``       bfs/plots/bfs_tree_plot.py:140-152
* ``scipy_bfs``             run_graph500.py:383-395 / run_bfs.py:517-527 (the
                            reference's own CPU BFS: scipy breadth_first_order
                            on A^T)
* ``bfs``                   the C restatement in bfs_oracle.c of the device
                            kernel bool_pe.csl (levels + lowest-index parents)
* ``min_parents``           the lowest-global-index parent rule of
                            bfs/README.md:208-224, computed from levels with
                            ``np.minimum.at`` (independent of bfs_oracle.c)
* ``graph500_validate``     the five Graph500 tree checks that
                            docs/GRAPH500_BENCHMARK.md:18-21 cites

Matrix convention everywhere: A[r, c] != 0 is an edge c -> r (row = dst,
col = src; docs/GRAPH500_BENCHMARK.md:126-128, graph_loader.py:76-90).

Parity is pinned by tests/golden/, whose fixtures were produced by importing
the reference's own modules (tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np
from scipy import sparse

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB = os.path.join(_BUILD, "liboracle.so")

PARENT_NONE_GLOBAL = 0xFFFFFFFF  # device_io.py:157


# --------------------------------------------------------------------------
# inputs
# --------------------------------------------------------------------------
def rmat(scale, edgefactor, seed, A=0.57, B=0.19, C=0.19, D=0.05):
  """R-MAT graph as a symmetric, loop-free, deduplicated scipy CSR matrix.

  Restates datasets/gen_rmat.py:15-44: ``scale`` levels, each drawing one
  uniform double per edge from ``np.random.default_rng(seed)``; quadrant
  (0,1) sets the column bit, (1,0) the row bit, (1,1) both.  Then both
  directions are stored, self-loops dropped and duplicates merged.  No vertex
  relabelling, so vertex 0 is the hub.
  """
  del D  # implied by A + B + C, as in the reference
  rng = np.random.default_rng(seed)
  n = 1 << scale
  m = n * edgefactor
  u = np.zeros(m, dtype=np.int64)
  v = np.zeros(m, dtype=np.int64)
  ab, abc = A + B, A + B + C
  for level in range(scale):
    r = rng.random(m)
    bit = 1 << (scale - 1 - level)
    u += np.where(r >= ab, bit, 0)
    v += np.where(((r >= A) & (r < ab)) | (r >= abc), bit, 0)
  rows = np.concatenate([u, v])
  cols = np.concatenate([v, u])
  keep = rows != cols
  rows, cols = rows[keep], cols[keep]
  key = np.unique(rows * n + cols)
  indptr = np.zeros(n + 1, dtype=np.int64)
  np.add.at(indptr, key // n + 1, 1)
  np.cumsum(indptr, out=indptr)
  return sparse.csr_matrix((np.ones(len(key)), (key % n).astype(np.int32), indptr),
                           shape=(n, n))


def pick_sources(A_csc, n, num_searches, seed):
  """Roots with out-degree >= 1 not counting self-loops, sampled without
  replacement by ``default_rng(seed).choice`` (run_graph500.py:106-127).
  Out-degree is the column count of A (row = dst, col = src)."""
  A_csc = sparse.csc_matrix(A_csc)
  outdeg = np.diff(A_csc.indptr) - (A_csc.diagonal() != 0).astype(np.int64)
  candidates = np.nonzero(outdeg > 0)[0]
  num = min(num_searches, len(candidates))
  rng = np.random.default_rng(seed)
  return rng.choice(candidates, size=num, replace=False).tolist()


def harmonic_mean(values):
  """run_graph500.py:130-134: over the finite, positive values only."""
  values = [v for v in values if v > 0 and np.isfinite(v)]
  if not values:
    return float("nan")
  return len(values) / sum(1.0 / v for v in values)


def compute_m(A_csr, visited, is_symmetric):
  """Edges traversed by one search (bfs_timing.py:379-398)."""
  coo = sparse.coo_matrix(A_csr)
  visited = np.asarray(visited, dtype=bool)
  if is_symmetric:
    return int(np.sum(visited[coo.row] & (coo.col <= coo.row)))
  return int(np.sum(visited[coo.col]))


def extract_parent_result(parent_u32, n):
  """Sentinel 0xFFFFFFFF -> -1 (device_io.py:157-178)."""
  p = np.asarray(parent_u32).astype(np.int64)[:n]
  return np.where(p == PARENT_NONE_GLOBAL, -1, p)


def derive_visited(parent, source):
  """visited = parent >= 0, plus the source (device_io.py:181-205)."""
  visited = np.asarray(parent) >= 0
  visited[source] = True
  return visited


def invalid_parents(parent, visited, A_csr, source):
  """Vertices whose parent is not a visited vertex joined by a real edge
  A[v, u] (bfs_tree_plot.py:140-152), vectorised."""
  A_csr = sparse.csr_matrix(A_csr)
  parent = np.asarray(parent, dtype=np.int64)
  visited = np.asarray(visited, dtype=bool)
  n = len(parent)
  idx = np.arange(n)
  cand = visited & (idx != source)
  bad = cand & ((parent < 0) | (parent >= n))
  ok = cand & ~bad
  vv, uu = idx[ok], parent[ok]
  has_edge = np.asarray(A_csr[vv, uu]).reshape(-1) != 0
  bad_ok = ~visited[uu] | ~has_edge
  bad[vv[bad_ok]] = True
  return np.nonzero(bad)[0].tolist()


def scipy_bfs(A_csr, source):
  """The reference's own host BFS: breadth_first_order on A^T
  (run_bfs.py:517-527).  Returns (levels, scipy_parent, visited), with levels
  derived from the predecessor array in BFS order."""
  from scipy.sparse.csgraph import breadth_first_order
  A_fwd = sparse.csr_matrix(A_csr).transpose().tocsr()
  order, pred = breadth_first_order(A_fwd, source, directed=True, return_predecessors=True)
  n = A_fwd.shape[0]
  levels = np.full(n, -1, dtype=np.int32)
  levels[source] = 0
  pred = pred.astype(np.int64)
  for v in order[1:]:
    levels[v] = levels[pred[v]] + 1
  parent = np.where(pred < 0, -1, pred)
  parent[source] = source
  visited = levels >= 0
  return levels, parent, visited


def min_parents(A_csr, levels, source):
  """Lowest-index parent (bfs/README.md:208-224): for every edge c -> r with
  level[c] == level[r] - 1, parent[r] = min c.  Independent of bfs_oracle.c."""
  coo = sparse.coo_matrix(A_csr)
  r, c = coo.row.astype(np.int64), coo.col.astype(np.int64)
  levels = np.asarray(levels, dtype=np.int64)
  sel = (levels[r] >= 1) & (levels[c] == levels[r] - 1)
  big = np.iinfo(np.int64).max
  parent = np.full(len(levels), big, dtype=np.int64)
  np.minimum.at(parent, r[sel], c[sel])
  parent[parent == big] = -1
  parent[source] = source
  return parent.astype(np.int32)


def fifo_parents(in_off, in_idx, levels, source):
  """Parents by the rule of the reference's own host BFS, scipy
  breadth_first_order on A^T (run_graph500.py:383-395, run_bfs.py:517-527):
  it pops its queue in order and hands each not-yet-seen out-neighbour (in
  ascending id order) the popped vertex as predecessor.  So the parent of a
  vertex at level L+1 is its level-L in-neighbour of smallest queue rank, and
  level L+1 is queued in order of (rank of the parent, vertex id).  Restated
  level by level from the levels alone, without scipy.  in_off/in_idx: the
  in-lists (row r of A: the sources of the edges into r)."""
  n = len(levels)
  levels = np.asarray(levels, dtype=np.int64)
  in_off = np.asarray(in_off, dtype=np.int64)
  dst = np.repeat(np.arange(n, dtype=np.int64), np.diff(in_off))
  src = np.asarray(in_idx, dtype=np.int64)
  parent = np.full(n, -1, dtype=np.int64)
  rank = np.full(n, -1, dtype=np.int64)
  parent[source] = source
  rank[source] = 0
  big = np.iinfo(np.int64).max
  for L in range(int(levels.max())):
    sel = (levels[dst] == L + 1) & (levels[src] == L)
    best = np.full(n, big, dtype=np.int64)
    np.minimum.at(best, dst[sel], rank[src[sel]] * n + src[sel])
    vs = np.nonzero(levels == L + 1)[0]
    if not len(vs):
      break
    parent[vs] = best[vs] % n
    prank = best[vs] // n
    order = np.lexsort((vs, prank))
    rank[vs[order]] = np.arange(len(vs))
  return parent.astype(np.int32)


def graph500_validate(A_csr, source, levels, parent):
  """The five Graph500 tree checks, stated in our own words:

  1. parent forms a tree rooted at ``source`` (no cycles, root is its own parent);
  2. each tree edge joins vertices whose levels differ by exactly one;
  3. every input edge joins vertices whose levels differ by at most one, or
     has both endpoints unreached;
  4. the tree spans exactly the vertices reachable from ``source``;
  5. every (parent, child) pair is an edge of the input graph.

  Returns a list of failure strings (empty == valid).
  """
  A = sparse.csr_matrix(A_csr)
  n = A.shape[0]
  levels = np.asarray(levels, dtype=np.int64)
  parent = np.asarray(parent, dtype=np.int64)
  errs = []
  reached = parent >= 0
  if parent[source] != source or levels[source] != 0:
    errs.append("1: root is not its own parent at level 0")
  # 1. pointer doubling: every reached vertex's 2^k-th ancestor must become
  #    the root once 2^k >= n (the root is its own parent, so it is absorbing)
  cur = np.where(reached)[0]
  p = np.where((parent >= 0) & (parent < n), parent, -1)
  for _ in range(int(np.ceil(np.log2(max(n, 2)))) + 1):
    p = np.where(p >= 0, p[np.clip(p, 0, n - 1)], -1)
  if np.any(p[cur] != source):
    errs.append("1: parent pointers do not all lead to the root (cycle or break)")
  # 2. tree edges span one level
  ch = np.where(reached & (np.arange(n) != source))[0]
  if np.any(parent[ch] >= n):
    errs.append("1: a parent is out of range")
    ch = ch[parent[ch] < n]
  if np.any(levels[parent[ch]] != levels[ch] - 1):
    errs.append("2: a tree edge does not join consecutive levels")
  # 3. graph edges (c -> r) span at most one level among reached vertices;
  #    an edge from a reached vertex must reach its target
  coo = A.tocoo()
  r, c = coo.row, coo.col
  lr, lc = levels[r], levels[c]
  both = (lr >= 0) & (lc >= 0)
  if np.any(both & (lr - lc > 1)):
    errs.append("3: an edge skips a level")
  if np.any((lc >= 0) & (lr < 0)):
    errs.append("3: an edge leaves the reached set")
  # 4. spans the reachable set
  ref_levels, _, _ = scipy_bfs(A, source)
  if np.any((ref_levels >= 0) != reached):
    errs.append("4: reached set differs from the reachable set")
  if np.any((levels >= 0) != reached):
    errs.append("4: levels and parents disagree on reached vertices")
  # 5. tree edges are graph edges (parent -> child, i.e. A[child, parent])
  if len(ch):
    if np.any(np.asarray(A[ch, parent[ch]]).reshape(-1) == 0):
      errs.append("5: a tree edge is not an input edge")
  return errs


CHECKS = ("root", "tree", "edges", "span", "tree_edge", "lowest")


def validation_counts(in_off, in_idx, root, levels, parents):
  """The per-check tallies of the device validator, restated in numpy:
  {check: (failures, lowest failing vertex or -1)}.

  The checks are graph500_validate's (above) written per vertex, plus the
  lowest-index parent rule of bfs/README.md:208-224: root (parent[root] ==
  root at level 0), tree (a reached v != root has a parent in range one level
  up), edges (per stored entry u -> v: u reached implies v reached no deeper
  than level[u] + 1 -- counted per entry), span (levels and parents agree on
  the reached set), tree_edge (parent[v] -> v is an input edge,
  bfs_tree_plot.py:140-152) and lowest (parent[v] is the lowest in-neighbour
  one level up).  tree_edge and lowest are only asked of vertices that pass
  tree.
  """
  in_off = np.asarray(in_off, dtype=np.int64)
  in_idx = np.asarray(in_idx, dtype=np.int64)
  lv = np.asarray(levels, dtype=np.int64)
  pa = np.asarray(parents, dtype=np.int64)
  n = len(in_off) - 1
  v = np.arange(n)
  rows = np.repeat(v, np.diff(in_off))
  out = {}

  def put(name, bad_mask):
    idx = np.nonzero(bad_mask)[0]
    out[name] = (int(len(idx)), int(idx[0]) if len(idx) else -1)

  put("span", (lv >= 0) != (pa >= 0))
  put("root", (v == root) & ((pa != root) | (lv != 0)))
  cand = (v != root) & (pa >= 0)
  in_range = cand & (pa < n)
  lp = np.where(in_range, lv[np.clip(pa, 0, n - 1)], -2)
  tree_bad = (cand & ((pa >= n) | (lv < 1) | (lp != lv - 1))) | ((v != root) & (pa < -1))
  put("tree", tree_bad)
  ok = cand & ~tree_bad
  keys = rows * n + in_idx                      # sorted: rows ascending, in-lists sorted
  want = v * n + np.where(ok, pa, 0)
  pos = np.searchsorted(keys, want)
  has = (pos < len(keys)) & (keys[np.minimum(pos, len(keys) - 1)] == want) if len(keys) else \
      np.zeros(n, dtype=bool)
  put("tree_edge", ok & ~has)
  lu = lv[in_idx]
  hit = lu == lv[rows] - 1
  low = np.full(n, -1, dtype=np.int64)
  big = np.iinfo(np.int64).max
  first = np.full(n, big, dtype=np.int64)
  np.minimum.at(first, rows[hit], in_idx[hit])
  low = np.where(first == big, -1, first)
  put("lowest", ok & (low != pa))
  lr = lv[rows]
  ebad = (lu >= 0) & ((lr < 0) | (lr > lu + 1))
  cnt = int(ebad.sum())
  out["edges"] = (cnt, int(rows[ebad].min()) if cnt else -1)
  return out


# --------------------------------------------------------------------------
# the C restatement
# --------------------------------------------------------------------------
def build(quiet=True):
  """Compile bfs_oracle.c into oracle/_build/liboracle.so with gcc."""
  os.makedirs(_BUILD, exist_ok=True)
  src = os.path.join(_HERE, "bfs_oracle.c")
  if os.path.exists(_LIB) and os.path.getmtime(_LIB) >= os.path.getmtime(src):
    return _LIB
  tmp = _LIB + f".{os.getpid()}.tmp"
  subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-o", tmp, src], check=True,
                 capture_output=quiet)
  os.replace(tmp, _LIB)
  return _LIB


_lib = None


def _load():
  global _lib
  if _lib is None:
    lib = ctypes.CDLL(build())
    p64, p32 = ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32)
    lib.oracle_bfs.argtypes = [ctypes.c_int64, p64, p32, p64, p32, ctypes.c_int64, p32, p32]
    lib.oracle_bfs.restype = ctypes.c_int64
    lib.oracle_count_m.argtypes = [ctypes.c_int64, p64, p32, p32, ctypes.c_int]
    lib.oracle_count_m.restype = ctypes.c_int64
    lib.oracle_msbfs.argtypes = [ctypes.c_int64, p64, p32, p64, p32, p64, ctypes.c_int64,
                                 p32, p32]
    lib.oracle_msbfs.restype = ctypes.c_int64
    _lib = lib
  return _lib


def _p(a, t):
  return a.ctypes.data_as(ctypes.POINTER(t))


def _adj(off, idx):
  return (np.ascontiguousarray(off, dtype=np.int64), np.ascontiguousarray(idx, dtype=np.int32))


def bfs(out_off, out_idx, in_off, in_idx, root):
  """C oracle BFS.  out_* = CSC of A (out-lists), in_* = CSR of A (in-lists,
  ascending).  Returns (levels, parents, rounds)."""
  lib = _load()
  out_off, out_idx = _adj(out_off, out_idx)
  in_off, in_idx = _adj(in_off, in_idx)
  n = len(out_off) - 1
  levels = np.empty(n, dtype=np.int32)
  parents = np.empty(n, dtype=np.int32)
  rounds = lib.oracle_bfs(n, _p(out_off, ctypes.c_int64), _p(out_idx, ctypes.c_int32),
                          _p(in_off, ctypes.c_int64), _p(in_idx, ctypes.c_int32), int(root),
                          _p(levels, ctypes.c_int32), _p(parents, ctypes.c_int32))
  if rounds < 0:
    raise ValueError(f"oracle_bfs failed ({rounds})")
  return levels, parents, int(rounds)


def bfs_csr(A_csr, root):
  """Oracle BFS straight from the reference's A (row = dst, col = src)."""
  A = sparse.csr_matrix(A_csr)
  A.sort_indices()
  At = A.tocsc()
  At.sort_indices()
  return bfs(At.indptr, At.indices, A.indptr, A.indices, root)


def count_m(in_off, in_idx, levels, symmetric):
  """C restatement of compute_m (bfs_timing.py:379-398) over the CSR of A."""
  lib = _load()
  in_off, in_idx = _adj(in_off, in_idx)
  levels = np.ascontiguousarray(levels, dtype=np.int32)
  return int(lib.oracle_count_m(len(in_off) - 1, _p(in_off, ctypes.c_int64),
                                _p(in_idx, ctypes.c_int32), _p(levels, ctypes.c_int32),
                                1 if symmetric else 0))
