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
from ceregraphs_gb300 import preprocess
from ceregraphs_gb300.engine import Graph, PinnedBuffer

pytestmark = pytest.mark.gpu

MAX_VERTICES = 1 << 21


def _dev(torch, arr):
  return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


def _ptr(t):
  return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _noalloc(lib, torch, a, d_in, d_out, root, stats="pageable"):
  """One cg_bfs_noalloc call; returns (levels, parents, stats or None) on the
  host.  stats: "pageable" (the call waits), "pinned" (the statistics arrive
  with the stream) or None (not reported)."""
  n = a.n
  d_lv = torch.full((n,), 123, dtype=torch.int32, device="cuda")
  d_pa = torch.full((n,), 123, dtype=torch.int32, device="cuda")
  torch.cuda.synchronize()
  pin = None
  if stats == "pageable":
    st = _lib.CgStats()
    st_arg = ctypes.byref(st)
  elif stats == "pinned":
    pin = PinnedBuffer(ctypes.sizeof(_lib.CgStats), dtype=np.uint8)
    st = _lib.CgStats.from_address(pin.array.ctypes.data)
    st_arg = ctypes.pointer(st)
  else:
    st, st_arg = None, None
  rc = lib.cg_bfs_noalloc(n, a.nnz, _ptr(d_in[0]), _ptr(d_in[1]), _ptr(d_out[0]), _ptr(d_out[1]),
                          int(root), _ptr(d_lv), _ptr(d_pa), st_arg, None)
  assert rc == 0, (rc, lib.cg_last_error_string())
  torch.cuda.synchronize()   # NULL / page-locked stats: the call only queued the work
  out = (d_lv.cpu().numpy(), d_pa.cpu().numpy(), st.as_dict() if st is not None else None)
  if pin is not None:
    pin.free()
  return out


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


def _small_directed(n, deg, seed):
  """A directed random graph whose n is not a multiple of 32 (the last frontier
  bitmap word is partial)."""
  rng = np.random.default_rng(seed)
  m = n * deg
  return preprocess.from_edges(n, rng.integers(0, n, m), rng.integers(0, n, m),
                               drop_self_loops=True)


@pytest.mark.parametrize("stats", ["pageable", "pinned", None])
def test_noalloc_partial_last_word_and_stats_modes(built_lib, stats):
  """n = 1000 (a partial last bitmap word) with pull rounds, every way of
  reading the outcome; two calls in a row against cg_bfs."""
  torch = pytest.importorskip("torch")
  a = _small_directed(1000, 12, 7)
  assert a.n % 32 != 0 and not a.symmetric
  roots = graph500.pick_sources(a, 2, 3)
  d_in = (_dev(torch, a.in_off), _dev(torch, a.in_idx))
  d_out = (_dev(torch, a.out_off), _dev(torch, a.out_idx))
  with Graph(a) as g:
    want = [g.bfs(r) for r in roots]
  assert any(w[2]["pull_rounds"] > 0 for w in want)   # the pull path runs
  for r, (wl, wp, wst) in zip(roots, want):
    lv, pa, st = _noalloc(built_lib, torch, a, d_in, d_out, r, stats=stats)
    assert np.array_equal(lv, wl), r
    assert np.array_equal(pa, wp), r
    if st is not None:
      assert st["status"] == 0
      assert st["rounds"] == wst["rounds"] and st["pull_rounds"] == wst["pull_rounds"]
