"""cg_bfs_noalloc: the search for callers that cannot let this library
allocate device memory (runtimes that budget the GPU's memory themselves, or
loops that cannot take the synchronisation of a cudaMalloc).  It keeps its
state in a fixed __device__ array instead of allocations, so these tests call
it through the C ABI on graphs the caller holds in device memory, twice in a
row on the same array, and compare it with the handle API's cg_bfs (integer
results: equal bit for bit).

This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes on its own in a fresh process (the first
call on the device sets the array up).
"""
import ctypes

import numpy as np
import pytest

from ceregraphs_gb300 import _lib, generators, graph500
from ceregraphs_gb300.engine import Graph

pytestmark = pytest.mark.gpu

MAX_VERTICES = 1 << 21


def _dev(torch, arr):
  return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


def _noalloc(lib, torch, a, d_in, d_out, root):
  """One cg_bfs_noalloc call; returns (levels, parents, stats) on the host."""
  n = a.n
  d_lv = torch.full((n,), 123, dtype=torch.int32, device="cuda")
  d_pa = torch.full((n,), 123, dtype=torch.int32, device="cuda")
  torch.cuda.synchronize()
  st = _lib.CgStats()
  p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
  rc = lib.cg_bfs_noalloc(n, a.nnz, p(d_in[0]), p(d_in[1]), p(d_out[0]), p(d_out[1]), int(root),
                          p(d_lv), p(d_pa), ctypes.byref(st), None)
  assert rc == 0, (rc, lib.cg_last_error_string())
  return d_lv.cpu().numpy(), d_pa.cpu().numpy(), st.as_dict()


@pytest.mark.parametrize("kind", ["rmat16", "rmat21", "er_directed"])
def test_noalloc_matches_cg_bfs_on_two_calls_in_a_row(built_lib, kind):
  torch = pytest.importorskip("torch")
  if kind == "rmat16":
    a = generators.rmat(16, 16, 0)
  elif kind == "rmat21":
    a = generators.rmat(21, 16, 0)      # the bench workload, at the capacity limit
  else:
    a = generators.er_directed(14, 8, 4)
  assert a.n <= MAX_VERTICES
  roots = graph500.pick_sources(a, 2, 9)
  d_in = (_dev(torch, a.in_off), _dev(torch, a.in_idx))
  d_out = (None, None)
  if not a.symmetric:
    d_out = (_dev(torch, a.out_off), _dev(torch, a.out_idx))
  with Graph(a) as g:
    want = [g.bfs(r) for r in roots]
  for r, (wl, wp, wst) in zip(roots, want):       # two calls in a row
    lv, pa, st = _noalloc(built_lib, torch, a, d_in, d_out, r)
    assert st["status"] == 0
    assert np.array_equal(lv, wl), (kind, r)
    assert np.array_equal(pa, wp), (kind, r)
    assert st["rounds"] == wst["rounds"] and st["visited"] == wst["visited"]


def test_noalloc_rejects_graphs_beyond_its_capacity(built_lib):
  torch = pytest.importorskip("torch")
  n = MAX_VERTICES + 1
  off = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
  idx = torch.zeros(1, dtype=torch.int32, device="cuda")
  out = torch.zeros(n, dtype=torch.int32, device="cuda")
  rc = built_lib.cg_bfs_noalloc(n, 0, ctypes.c_void_p(off.data_ptr()),
                                ctypes.c_void_p(idx.data_ptr()), None, None, 0,
                                ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                None, None)
  assert rc == _lib.CG_ERR_INVALID_ARG
  assert b"capacity" in built_lib.cg_last_error_string()
