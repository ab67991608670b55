"""FIFO parent rule on the GPU (cg_options.parent_rule = CG_PARENT_FIFO): the
parents of scipy's breadth_first_order, the reference's own host search --
against the golden fixtures made from it, and against the oracle's
restatement of the rule on larger graphs, per-root and batched."""
import numpy as np
import pytest

from golden_data import arrays, csr_from, golden, sha
from ceregraphs_gb300 import _lib, generators, graph500, preprocess
from ceregraphs_gb300.engine import Graph

pytestmark = pytest.mark.gpu

G = golden()
ARR = arrays()


def _fifo_oracle(oracle_mod, a, roots):
  out_off, out_idx = a.out_lists()
  lv = np.empty((len(roots), a.n), dtype=np.int32)
  pa = np.empty_like(lv)
  for i, r in enumerate(roots):
    lv[i], _, _ = oracle_mod.bfs(out_off, out_idx, a.in_off, a.in_idx, r)
    pa[i] = oracle_mod.fifo_parents(a.in_off, a.in_idx, lv[i], r)
  return lv, pa


@pytest.mark.parametrize("direction", [_lib.CG_DIR_AUTO, _lib.CG_DIR_TOPDOWN,
                                       _lib.CG_DIR_BOTTOMUP])
def test_fifo_matches_scipy_golden(built_lib, direction):
  """Per-root and batched FIFO parents equal scipy's predecessors stored in
  the golden fixtures (R-MAT s10/s12, symmetric)."""
  for key in ("s10_e16_seed0", "s12_e16_seed0"):
    g0 = G["graphs"][key]
    a = generators.rmat(g0["scale"], g0["edgefactor"], g0["seed"])
    recs = G["searches"][key]
    roots = [rec["source"] for rec in recs]
    with Graph(a) as g:
      g.set_options(direction=direction, parent_rule=_lib.CG_PARENT_FIFO)
      for rec in recs:
        r = rec["source"]
        lv, pa, st = g.bfs(r)
        assert st["status"] == 0
        assert np.array_equal(lv, ARR[f"{key}_r{r}_levels"])
        assert np.array_equal(pa, ARR[f"{key}_r{r}_scipy_parents"]), (key, r)
        assert sha(pa) == rec["scipy_parents_sha"]
      for lw in (1, 2):
        g.set_options(lane_words=lw)
        lv, pa, st = g.msbfs(roots)
        assert st["status"] == 0
        for i, rec in enumerate(recs):
          assert sha(pa[i]) == rec["scipy_parents_sha"], (key, lw, rec["source"])


def test_fifo_directed_with_self_loops(built_lib):
  """The directed 600-vertex matrix with self-loops (rand600.mtx kind)."""
  a = preprocess.preprocess(csr_from(ARR["dir600_indptr"], ARR["dir600_indices"], 600))
  with Graph(a) as g:
    g.set_options(parent_rule=_lib.CG_PARENT_FIFO)
    for rec in G["searches"]["dir600"]:
      r = rec["source"]
      lv, pa, st = g.bfs(r)
      assert st["status"] == 0
      assert np.array_equal(pa, ARR[f"dir600_r{r}_scipy_parents"])


@pytest.mark.parametrize("lane_words", [1, 2])
def test_fifo_batched_vs_oracle(built_lib, oracle_mod, lane_words):
  """100 roots on R-MAT s13, a directed ER graph and a grid (deep levels)."""
  cases = [(generators.rmat(13, 16, 7), None),
           (generators.er_directed(12, 6, 9), [0, 1, 2, 500, 4095]),
           (generators.grid2d(40), [0, 39, 820, 1599])]
  for a, roots in cases:
    if roots is None:
      roots = graph500.pick_sources(a, 100, 4)
    rl, rp = _fifo_oracle(oracle_mod, a, roots)
    with Graph(a) as g:
      g.set_options(lane_words=lane_words, parent_rule=_lib.CG_PARENT_FIFO)
      lv, pa, st = g.msbfs(roots)
      assert st["status"] == 0
      assert np.array_equal(lv, rl) and np.array_equal(pa, rp)
      # the trees still pass the Graph500 checks; only the lowest-index rule fails
      import torch
      d_lv = torch.from_numpy(lv).cuda()
      d_pa = torch.from_numpy(pa).cuda()
      res = g.validate(roots, d_lv, d_pa)
      for r in res:
        assert all(r[c]["failures"] == 0 for c in ("root", "tree", "edges", "span", "tree_edge"))


def test_fifo_scipy_directly(built_lib, oracle_mod):
  """A few roots of R-MAT s14 checked against scipy itself."""
  a = generators.rmat(14, 16, 3)
  A = a.scipy_csr()
  roots = graph500.pick_sources(a, 6, 2)
  with Graph(a) as g:
    g.set_options(parent_rule=_lib.CG_PARENT_FIFO)
    for r in roots:
      lv, pa, _ = g.bfs(r)
      sl, sp, _ = oracle_mod.scipy_bfs(A, r)
      assert np.array_equal(lv, sl)
      assert np.array_equal(pa, sp.astype(np.int32))


def test_fifo_refused_inside_a_capture(built_lib):
  """The FIFO pass synchronises with the stream, so a capture refuses it and
  the handle stays usable."""
  torch = pytest.importorskip("torch")
  a = generators.rmat(10, 16, 0)
  with Graph(a) as g:
    d_lv = torch.empty(a.n, dtype=torch.int32, device="cuda")
    d_pa = torch.empty_like(d_lv)
    torch.cuda.synchronize()
    g.bfs_device(0, d_lv, d_pa)  # first use (state set up) outside the capture
    g.last_stats()
    g.set_options(parent_rule=_lib.CG_PARENT_FIFO)
    with pytest.raises(_lib.CgError) as ei:
      g.capture(lambda: g.bfs_device(0, d_lv, d_pa))
    assert ei.value.status == _lib.CG_ERR_NOT_SUPPORTED
    g.set_options(parent_rule=_lib.CG_PARENT_LOWEST)
    lv, pa, st = g.bfs(0)
    assert st["status"] == 0 and pa[0] == 0
