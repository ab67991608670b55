"""Degree-aware reordering (cg_graph_reorder, the counterpart of the
reference's util/analyze.cpp balancing with --operm's vertex identity):
per-root searches on the reordered copy must equal the original graph's and
the oracle's bit for bit -- roots and outputs in original ids, lowest-index
parents -- and everything the copy does not support is refused."""
import ctypes

import numpy as np
import pytest

from golden_data import arrays, csr_from
from ceregraphs_gb300 import _lib, generators, graph500, preprocess
from ceregraphs_gb300.engine import Graph

pytestmark = pytest.mark.gpu

DIRS = [_lib.CG_DIR_AUTO, _lib.CG_DIR_TOPDOWN, _lib.CG_DIR_BOTTOMUP, _lib.CG_DIR_TAU]


def _graphs():
  ARR = arrays()
  yield "rmat16", generators.rmat(16, 16, 0)
  yield "er14-directed", generators.er_directed(14, 8, 4)
  yield "dir600-loops", preprocess.preprocess(csr_from(ARR["dir600_indptr"],
                                                       ARR["dir600_indices"], 600))
  yield "grid96", generators.grid2d(96)


@pytest.mark.parametrize("name,a", list(_graphs()), ids=lambda x: x if isinstance(x, str) else "")
def test_reordered_searches_equal_original_and_oracle(built_lib, oracle_mod, name, a):
  roots = graph500.pick_sources(a, 6, 11)
  out_off, out_idx = a.out_lists()
  with Graph(a) as g, g.reorder() as gr:
    for direction in DIRS:
      g.set_options(direction=direction)
      gr.set_options(direction=direction)
      for r in roots:
        wl, wp, ws = g.bfs(r)
        lv, pa, st = gr.bfs(r)
        assert st["status"] == 0
        assert np.array_equal(lv, wl) and np.array_equal(pa, wp), (name, direction, r)
        assert st["rounds"] == ws["rounds"] and st["visited"] == ws["visited"]
    rl, rp, _ = oracle_mod.bfs(out_off, out_idx, a.in_off, a.in_idx, roots[0])
    lv, pa, _ = gr.bfs(roots[0])
    assert np.array_equal(lv, rl) and np.array_equal(pa, rp)


def test_reordered_benchmark_graph_device_outputs_and_capture(built_lib, oracle_mod):
  torch = pytest.importorskip("torch")
  g, a = generators.rmat_device(21, 16, 0)
  roots = graph500.pick_sources(a, 64, 1)[:4]
  with g, g.reorder() as gr:
    d = [torch.empty(a.n, dtype=torch.int32, device="cuda") for _ in range(4)]
    torch.cuda.synchronize()
    exe = gr.capture(lambda: [gr.bfs_device(r, d[2 * (i % 2)], d[2 * (i % 2) + 1])
                              for i, r in enumerate(roots[:2])])
    exe.launch()
    gr.last_stats()
    exe.close()
    for i, r in enumerate(roots):
      gr.bfs_device(r, d[0], d[1])
      g.bfs_device(r, d[2], d[3])
      assert gr.last_stats()["status"] == 0 and g.last_stats()["status"] == 0
      assert torch.equal(d[0], d[2]) and torch.equal(d[1], d[3]), r
    rl, rp, _ = oracle_mod.bfs(a.in_off, a.in_idx, a.in_off, a.in_idx, roots[0])
    gr.bfs_device(roots[0], d[0], d[1])
    gr.last_stats()
    assert np.array_equal(d[0].cpu().numpy(), rl) and np.array_equal(d[1].cpu().numpy(), rp)


def test_reordered_copy_refuses_what_it_does_not_map(built_lib):
  torch = pytest.importorskip("torch")
  lib = built_lib
  a = generators.rmat(12, 16, 0)
  with Graph(a) as g, g.reorder() as gr:
    h = gr.handle
    d = torch.zeros((2, a.n), dtype=torch.int32, device="cuda")
    p = ctypes.c_void_p(d.data_ptr())
    roots = np.array([0, 1], dtype=np.int64)
    rp = roots.ctypes.data_as(ctypes.c_void_p)
    m = np.zeros(2, dtype=np.int64)
    assert lib.cg_msbfs_device(h, rp, 2, p, p) == _lib.CG_ERR_NOT_SUPPORTED
    assert lib.cg_msbfs(h, rp, 2, None, None, None) == _lib.CG_ERR_NOT_SUPPORTED
    assert lib.cg_count_edges(h, p, 1, m.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))) == \
        _lib.CG_ERR_NOT_SUPPORTED
    assert lib.cg_validate_device(h, rp, 1, p, p, (_lib.CgValidation * 1)()) == \
        _lib.CG_ERR_NOT_SUPPORTED
    pool = ctypes.c_void_p()
    assert lib.cg_pool_create(h, 1, ctypes.byref(pool)) == _lib.CG_ERR_NOT_SUPPORTED
    off = np.empty(a.n + 1, dtype=np.int64)
    assert lib.cg_graph_export(h, off.ctypes.data_as(ctypes.c_void_p), None, None, None) == \
        _lib.CG_ERR_NOT_SUPPORTED
    again = ctypes.c_void_p()
    assert lib.cg_graph_reorder(h, _lib.CG_ORDER_DEGREE, ctypes.byref(again)) == \
        _lib.CG_ERR_NOT_SUPPORTED
    gr.set_options(parent_rule=_lib.CG_PARENT_FIFO)
    with pytest.raises(_lib.CgError):
      gr.bfs(0)
    assert b"reordered" in lib.cg_last_error_string()
    # the original handle is untouched by its copy
    lv, pa, st = g.bfs(0)
    assert st["status"] == 0
