"""Device-side construction: the GPU R-MAT / ER draws and the CSR build must
equal the host generators (and, through them, the reference generator)."""
import numpy as np
import pytest

from golden_data import golden, sha
from ceregraphs_gb300 import generators, preprocess

pytestmark = pytest.mark.gpu
G = golden()


@pytest.mark.parametrize("key", ["s8_e16_seed0", "s10_e16_seed0", "s12_e4_seed0",
                                 "s14_e16_seed3", "s16_e16_seed0"])
def test_device_rmat_matches_reference_hashes(built_lib, key):
  g0 = G["graphs"][key]
  g, a = generators.rmat_device(g0["scale"], g0["edgefactor"], g0["seed"])
  with g:
    assert a.symmetric and a.n == g0["n"] and a.nnz == g0["nnz"]
    assert sha(a.in_off) == g0["indptr_sha"]
    assert sha(a.in_idx) == g0["indices_sha"]


def test_device_rmat_endpoints_match_host_draws(built_lib):
  for scale, ef, seed in ((9, 8, 4), (11, 3, 7), (5, 1, 0)):
    u, v = generators.rmat_edges_device(scale, ef, seed)
    hu, hv = generators.rmat_edge_endpoints(scale, ef, seed)
    assert np.array_equal(u.cpu().numpy().view(np.uint32), hu)
    assert np.array_equal(v.cpu().numpy().view(np.uint32), hv)


def test_device_er_matches_host(built_lib):
  g, a = generators.er_directed_device(12, 8, 4)
  with g:
    h = generators.er_directed(12, 8, 4)
    assert not a.symmetric
    for x, y in ((a.in_off, h.in_off), (a.in_idx, h.in_idx), (a.out_off, h.out_off),
                 (a.out_idx, h.out_idx)):
      assert np.array_equal(x, y)


def test_graph_from_edges_with_duplicates_and_loops(built_lib, oracle_mod):
  import ctypes
  import torch
  from ceregraphs_gb300 import _lib
  from ceregraphs_gb300.engine import Graph
  rng = np.random.default_rng(3)
  n, m = 3000, 20000
  src = rng.integers(0, n, m).astype(np.int32)
  dst = rng.integers(0, n, m).astype(np.int32)
  src[:50] = dst[:50]                 # self-loops
  src[50:100], dst[50:100] = src[100:150], dst[100:150]   # duplicates
  for flags, sym, drop in ((0, False, False), (1, True, False), (2, False, True), (3, True, True)):
    ds = torch.from_numpy(src).cuda()
    dd = torch.from_numpy(dst).cuda()
    torch.cuda.synchronize()
    h = ctypes.c_void_p()
    _lib.check(_lib.load().cg_graph_from_edges(n, m, ctypes.c_void_p(ds.data_ptr()),
                                               ctypes.c_void_p(dd.data_ptr()), flags,
                                               ctypes.byref(h)), "from_edges")
    with Graph.from_handle(h) as g:
      a = g.export()
      want = preprocess.from_edges(n, src, dst, symmetrize=sym, drop_self_loops=drop)
      assert a.nnz == want.nnz
      assert np.array_equal(a.in_off, want.in_off) and np.array_equal(a.in_idx, want.in_idx)
      if not a.symmetric:
        wo, wi = want.out_lists()
        assert np.array_equal(a.out_off, wo) and np.array_equal(a.out_idx, wi)
      for r in (0, 17, 2999):
        lv, pa, _ = g.bfs(r)
        oo, oi = a.out_lists()
        rl, rp, _ = oracle_mod.bfs(oo, oi, a.in_off, a.in_idx, r)
        assert np.array_equal(lv, rl) and np.array_equal(pa, rp)
