"""Batched (bit-lane) search parity on the GPU: every lane must equal the
single-root search of the oracle bit for bit."""
import numpy as np
import pytest

from golden_data import arrays, csr_from, golden
from ceregraphs_gb300 import _lib, generators, graph500, preprocess
from ceregraphs_gb300.engine import Graph

pytestmark = pytest.mark.gpu

G = golden()
ARR = arrays()
MS_DIRS = [_lib.CG_DIR_AUTO, _lib.CG_DIR_TOPDOWN, _lib.CG_DIR_BOTTOMUP]


def _oracle_all(oracle_mod, a, roots):
  out_off, out_idx = a.out_lists()
  lv = np.empty((len(roots), a.n), dtype=np.int32)
  pa = np.empty((len(roots), a.n), dtype=np.int32)
  rounds = 0
  for i, r in enumerate(roots):
    lv[i], pa[i], rr = oracle_mod.bfs(out_off, out_idx, a.in_off, a.in_idx, r)
    rounds = max(rounds, rr)
  return lv, pa, rounds


@pytest.mark.parametrize("lane_words", [1, 2])
@pytest.mark.parametrize("direction", MS_DIRS)
def test_msbfs_matches_golden(built_lib, lane_words, direction):
  key = "s12_e16_seed0"
  g0 = G["graphs"][key]
  a = generators.rmat(g0["scale"], g0["edgefactor"], g0["seed"])
  recs = G["searches"][key]
  roots = [rec["source"] for rec in recs]
  with Graph(a) as g:
    g.set_options(lane_words=lane_words, direction=direction)
    lv, pa, st = g.msbfs(roots)
    assert st["status"] == 0
    for i, rec in enumerate(recs):
      r = rec["source"]
      assert np.array_equal(lv[i], ARR[f"{key}_r{r}_levels"]), (i, r)
      assert np.array_equal(pa[i], ARR[f"{key}_r{r}_parents"]), (i, r)
    assert st["rounds"] == max(rec["rounds"] for rec in recs)


@pytest.mark.parametrize("lane_words", [1, 2])
def test_msbfs_64_roots_s16_vs_oracle(built_lib, oracle_mod, lane_words):
  a = generators.rmat(16, 16, 0)
  roots = graph500.pick_sources(a, 64, 1)
  rl, rp, rounds = _oracle_all(oracle_mod, a, roots)
  with Graph(a) as g:
    for direction in MS_DIRS:
      g.set_options(lane_words=lane_words, direction=direction)
      lv, pa, st = g.msbfs(roots)
      assert np.array_equal(lv, rl), direction
      assert np.array_equal(pa, rp), direction
      assert st["rounds"] == rounds


def test_msbfs_many_passes_and_duplicate_roots(built_lib, oracle_mod):
  a = generators.rmat(13, 16, 5)
  roots = graph500.pick_sources(a, 150, 2)
  roots[7] = roots[3]      # the same root in two lanes
  roots[100] = roots[3]    # and in another pass
  rl, rp, _ = _oracle_all(oracle_mod, a, roots)
  with Graph(a) as g:
    for lw in (1, 2):
      g.set_options(lane_words=lw)
      lv, pa, st = g.msbfs(roots)   # 150 lanes: 3 passes of 64, or 2 of 128
      assert np.array_equal(lv, rl) and np.array_equal(pa, rp), lw


def test_msbfs_directed_and_deep(built_lib, oracle_mod):
  D = csr_from(ARR["dir600_indptr"], ARR["dir600_indices"], 600)
  cases = [(preprocess.preprocess(D), [rec["source"] for rec in G["searches"]["dir600"]]),
           (generators.er_directed(13, 8, 4), [0, 1, 2, 3, 100, 8191]),
           (generators.grid2d(80), [0, 79, 80 * 40 + 40, 80 * 80 - 1])]
  for a, roots in cases:
    rl, rp, rounds = _oracle_all(oracle_mod, a, roots)
    with Graph(a) as g:
      for direction in MS_DIRS:
        for lw in (1, 2):
          g.set_options(direction=direction, lane_words=lw)
          lv, pa, st = g.msbfs(roots)
          assert np.array_equal(lv, rl) and np.array_equal(pa, rp), (direction, lw)
          assert st["rounds"] == rounds


def test_msbfs_device_capture_and_edge_counts(built_lib, oracle_mod):
  torch = pytest.importorskip("torch")
  a = generators.rmat(14, 16, 3)
  roots = graph500.pick_sources(a, 64, 3)
  rl, rp, _ = _oracle_all(oracle_mod, a, roots)
  with Graph(a) as g:
    d_lv = torch.empty((64, a.n), dtype=torch.int32, device="cuda")
    d_pa = torch.empty((64, a.n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    g.msbfs_device(roots, d_lv, d_pa)   # allocates lane state before capture
    g.last_stats()
    exe = g.capture(lambda: g.msbfs_device(roots, d_lv, d_pa))
    d_lv.fill_(7)
    d_pa.fill_(7)
    torch.cuda.synchronize()
    for _ in range(2):
      exe.launch()
      st = g.last_stats()
      assert st["status"] == 0
      assert np.array_equal(d_lv.cpu().numpy(), rl)
      assert np.array_equal(d_pa.cpu().numpy(), rp)
    exe.close()
    m = g.count_edges(d_lv, 64)
    ec = graph500.EdgeCounter(a)
    assert m.tolist() == [ec.m(rl[i] >= 0) for i in range(64)]


def test_per_root_capture(built_lib, oracle_mod):
  torch = pytest.importorskip("torch")
  a = generators.rmat(12, 16, 0)
  roots = [0, 5, 9]
  with Graph(a) as g:
    d_lv = torch.empty((3, a.n), dtype=torch.int32, device="cuda")
    d_pa = torch.empty((3, a.n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()

    def body():
      for i, r in enumerate(roots):
        g.bfs_device(r, d_lv[i], d_pa[i])
    exe = g.capture(body)
    exe.launch()
    g.last_stats()
    for i, r in enumerate(roots):
      l, p, _ = oracle_mod.bfs(a.in_off, a.in_idx, a.in_off, a.in_idx, r)
      assert np.array_equal(d_lv[i].cpu().numpy(), l)
      assert np.array_equal(d_pa[i].cpu().numpy(), p)
    exe.close()


@pytest.mark.parametrize("history", [-1, 0, 3, 6])
def test_msbfs_history_modes(built_lib, oracle_mod, history):
  """Outputs written during the rounds (history < 0), from the round history
  (0: as memory allows), and searches that outgrow a short history (3, 6:
  the gated direct launch takes over) -- all equal to the oracle."""
  cases = [(generators.rmat(13, 16, 7), None),
           (generators.er_directed(12, 6, 9), [0, 1, 2, 500, 4095]),
           (generators.grid2d(40), [0, 39, 820, 1599])]
  for a, roots in cases:
    if roots is None:
      roots = graph500.pick_sources(a, 100, 4)
    rl, rp, rounds = _oracle_all(oracle_mod, a, roots)
    with Graph(a) as g:
      for lw in (1, 2):
        g.set_options(ms_history=history, lane_words=lw)
        lv, pa, st = g.msbfs(roots)
        assert st["status"] == 0
        assert np.array_equal(lv, rl) and np.array_equal(pa, rp), (history, lw)
        assert st["rounds"] == rounds


def test_msbfs_history_overflow_in_a_captured_graph(built_lib, oracle_mod):
  """A captured batch whose search outgrows the history: the fallback launch
  is part of the graph and decides on the device."""
  torch = pytest.importorskip("torch")
  a = generators.grid2d(30)
  roots = [0, 29, 450, 899]
  rl, rp, _ = _oracle_all(oracle_mod, a, roots)
  b = generators.rmat(12, 16, 0)
  broots = graph500.pick_sources(b, 64, 2)
  bl, bp, _ = _oracle_all(oracle_mod, b, broots)
  for arr, rts, wl, wp in ((a, roots, rl, rp), (b, broots, bl, bp)):
    with Graph(arr) as g:
      g.set_options(ms_history=8)
      d_lv = torch.empty((len(rts), arr.n), dtype=torch.int32, device="cuda")
      d_pa = torch.empty_like(d_lv)
      torch.cuda.synchronize()
      g.msbfs_device(rts, d_lv, d_pa)
      g.last_stats()
      exe = g.capture(lambda: g.msbfs_device(rts, d_lv, d_pa))
      d_lv.fill_(7)
      d_pa.fill_(7)
      torch.cuda.synchronize()
      exe.launch()
      assert g.last_stats()["status"] == 0
      assert np.array_equal(d_lv.cpu().numpy(), wl) and np.array_equal(d_pa.cpu().numpy(), wp)
      exe.close()


@pytest.mark.parametrize("lane_words", [1, 2])
@pytest.mark.parametrize("direction", MS_DIRS)
def test_msbfs_more_parents_than_records(built_lib, oracle_mod, lane_words, direction):
  """Light vertices with more distinct parents across lanes than they have
  (source, lanes) records: 128 roots hang off 24 middle vertices, and two
  targets of in-degree 24 see a different parent in almost every lane, so
  their records run out and the fix-up pass writes the rest."""
  roots = list(range(128))
  mid = [128 + j for j in range(24)]
  t1, t2 = 152, 153
  src, dst = [], []
  for r in roots:
    src.append(r)
    dst.append(mid[r % 24])
  for m in mid:
    src += [m, m]
    dst += [t1, t2]
  src += [t1, 154, 155]
  dst += [154, 155, 156]
  a = preprocess.from_edges(157, np.array(src), np.array(dst), symmetrize=True)
  k = 64 * lane_words
  rl, rp, _ = _oracle_all(oracle_mod, a, roots[:k])
  with Graph(a) as g:
    g.set_options(lane_words=lane_words, direction=direction)
    lv, pa, st = g.msbfs(roots[:k])
    assert st["status"] == 0
    assert np.array_equal(lv, rl) and np.array_equal(pa, rp)


@pytest.mark.parametrize("graph", ["rmat16", "grid96"])
def test_msbfs_into_page_locked_host_buffers(built_lib, oracle_mod, graph):
  """Page-locked outputs: the batch's kernels write host memory directly (two
  passes of 64 lanes; the 96 x 96 grid is deeper than the round history, so its
  batch runs in the direct kernel).  Equal to the oracle bit for bit."""
  from ceregraphs_gb300.engine import PinnedBuffer
  a = generators.rmat(16, 16, 0) if graph == "rmat16" else generators.grid2d(96)
  roots = graph500.pick_sources(a, 80, 2)
  k = len(roots)
  rl, rp, rounds = _oracle_all(oracle_mod, a, roots)
  with Graph(a) as g:
    lv, pa = PinnedBuffer((k, a.n)), PinnedBuffer((k, a.n))
    lv.array[:] = 7
    pa.array[:] = 7
    _, _, st = g.msbfs(roots, lv.array, pa.array)
    assert st["status"] == 0
    assert np.array_equal(lv.array, rl)
    assert np.array_equal(pa.array, rp)
    lv.free()
    pa.free()
