"""Synthetic graph inputs.

* ``rmat``        -- the reference's R-MAT recipe (datasets/gen_rmat.py:15-44),
                     bit-identical: same ``default_rng(seed)`` stream, consumed
                     level by level, same quadrant rule, then symmetrised,
                     self-loops dropped and duplicates merged, no relabelling.
                     ``rmat`` runs on the host in bounded chunks;
                     ``rmat_device`` draws the same stream on the GPU
                     (cg_rmat_edges, PCG64 jump-ahead) and builds the CSR there.
* ``er_directed`` -- directed Erdos-Renyi G(n, m = n * mean_degree): src of edge
                     e is floor(r_e * n) for the e-th double r_e of
                     ``default_rng(seed)``, dst uses doubles m .. 2m-1; self-loops
                     and duplicates removed (no counterpart in the reference).
* ``grid2d``      -- the 4-neighbour side x side grid (no counterpart in the
                     reference), built straight into CSR.
Host forms return preprocess.GraphArrays (A[dst, src] = 1 for edge src -> dst);
device forms return (engine.Graph, GraphArrays).
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

from .preprocess import GraphArrays, from_edges

RMAT_A, RMAT_B, RMAT_C, RMAT_D = 0.57, 0.19, 0.19, 0.05
_M64 = (1 << 64) - 1


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
  """Directed G(n, m): see the module docstring for the exact draw."""
  n = 1 << log2_n
  m = n * mean_degree
  rng = np.random.default_rng(seed)
  src = (rng.random(m) * n).astype(np.int64)
  dst = (rng.random(m) * n).astype(np.int64)
  return from_edges(n, src, dst, symmetrize=False, drop_self_loops=True)


def grid2d(side) -> GraphArrays:
  """side x side 4-neighbour grid; vertex id = row * side + col; undirected
  (both directions stored, ascending per row).  Diameter 2 * (side - 1)."""
  n = side * side
  ids = np.arange(n, dtype=np.int64)
  r, c = ids // side, ids % side
  # neighbours in ascending id order: up, left, right, down
  cand = np.stack([ids - side, ids - 1, ids + 1, ids + side], axis=1)
  ok = np.stack([r > 0, c > 0, c < side - 1, r < side - 1], axis=1)
  deg = ok.sum(axis=1)
  off = np.zeros(n + 1, dtype=np.int64)
  np.cumsum(deg, out=off[1:])
  idx = cand[ok].astype(np.int32)
  return GraphArrays(n, int(off[-1]), off, idx, None, None, True)


# --------------------------------------------------------------------------
# device construction
# --------------------------------------------------------------------------
def pcg64_state(seed):
  """{state_hi, state_lo, inc_hi, inc_lo} of the PCG64 that default_rng(seed)
  starts from (numpy seeds it through SeedSequence)."""
  st = np.random.PCG64(seed).state["state"]
  s, inc = int(st["state"]), int(st["inc"])
  return np.array([s >> 64, s & _M64, inc >> 64, inc & _M64], dtype=np.uint64)


def rmat_thresholds(A=RMAT_A, B=RMAT_B, C=RMAT_C):
  """ceil(t * 2^53) for t = A, A+B, A+B+C (the float sums gen_rmat.py forms):
  a double r = k * 2^-53 satisfies r >= t exactly when k >= that integer."""
  ab, abc = A + B, A + B + C
  return np.array([math.ceil(Fraction(t) * (1 << 53)) for t in (A, ab, abc)], dtype=np.uint64)


def _graph_from_device_edges(n, m, d_src, d_dst, flags, export=True):
  import ctypes
  import torch
  from . import _lib
  from .engine import Graph
  torch.cuda.synchronize()
  h = ctypes.c_void_p()
  _lib.check(_lib.load().cg_graph_from_edges(n, m, ctypes.c_void_p(d_src.data_ptr()),
                                             ctypes.c_void_p(d_dst.data_ptr()), flags,
                                             ctypes.byref(h)), "cg_graph_from_edges")
  g = Graph.from_handle(h)
  arrays = g.export() if export else None
  return g, arrays


def rmat_device(scale, edgefactor, seed, A=RMAT_A, B=RMAT_B, C=RMAT_C, export=True):
  """rmat() drawn and built on the GPU; returns (Graph, GraphArrays or None)."""
  import ctypes
  import torch
  from . import _lib
  n = 1 << scale
  m = n * edgefactor
  u = torch.empty(m, dtype=torch.int32, device="cuda")
  v = torch.empty(m, dtype=torch.int32, device="cuda")
  st = pcg64_state(seed)
  th = rmat_thresholds(A, B, C)
  stream = torch.cuda.current_stream().cuda_stream
  _lib.check(_lib.load().cg_rmat_edges(scale, m, st.ctypes.data_as(ctypes.c_void_p),
                                       th.ctypes.data_as(ctypes.c_void_p),
                                       ctypes.c_void_p(u.data_ptr()),
                                       ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(stream)),
             "cg_rmat_edges")
  out = _graph_from_device_edges(n, m, u, v, 3, export)  # symmetrise + drop loops
  del u, v
  return out


def rmat_edges_device(scale, edgefactor, seed, A=RMAT_A, B=RMAT_B, C=RMAT_C):
  """The raw endpoints (u, v) as torch CUDA int32 tensors."""
  import ctypes
  import torch
  from . import _lib
  n = 1 << scale
  m = n * edgefactor
  u = torch.empty(m, dtype=torch.int32, device="cuda")
  v = torch.empty(m, dtype=torch.int32, device="cuda")
  st = pcg64_state(seed)
  th = rmat_thresholds(A, B, C)
  _lib.check(_lib.load().cg_rmat_edges(scale, m, st.ctypes.data_as(ctypes.c_void_p),
                                       th.ctypes.data_as(ctypes.c_void_p),
                                       ctypes.c_void_p(u.data_ptr()),
                                       ctypes.c_void_p(v.data_ptr()),
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
             "cg_rmat_edges")
  torch.cuda.synchronize()
  return u, v


def er_directed_device(log2_n, mean_degree, seed, export=True):
  """er_directed() drawn and built on the GPU."""
  import ctypes
  import torch
  from . import _lib
  n = 1 << log2_n
  m = n * mean_degree
  src = torch.empty(m, dtype=torch.int32, device="cuda")
  dst = torch.empty(m, dtype=torch.int32, device="cuda")
  st = pcg64_state(seed)
  lib = _lib.load()
  stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
  for first, t in ((0, src), (m, dst)):
    _lib.check(lib.cg_uniform_bits(st.ctypes.data_as(ctypes.c_void_p), first, m, log2_n,
                                   ctypes.c_void_p(t.data_ptr()), stream), "cg_uniform_bits")
  out = _graph_from_device_edges(n, m, src, dst, 2, export)  # drop loops, keep direction
  del src, dst
  return out
