"""Per-root search parity on the GPU, through the C ABI, against the oracle and
the reference-generated golden fixtures.  Integer work: bit-exact."""
import numpy as np
import pytest

from golden_data import arrays, csr_from, golden, sha
from ceregraphs_gb300 import _lib, generators, preprocess
from ceregraphs_gb300.engine import Graph

pytestmark = pytest.mark.gpu

G = golden()
ARR = arrays()
DIRS = [_lib.CG_DIR_AUTO, _lib.CG_DIR_TOPDOWN, _lib.CG_DIR_BOTTOMUP, _lib.CG_DIR_TAU]


@pytest.fixture(scope="module")
def lib(built_lib):
  return built_lib


def _oracle(oracle_mod, a, root):
  out_off, out_idx = a.out_lists()
  return oracle_mod.bfs(out_off, out_idx, a.in_off, a.in_idx, root)


def _graph(key):
  g = G["graphs"][key]
  return generators.rmat(g["scale"], g["edgefactor"], g["seed"])


@pytest.mark.parametrize("key", ["s10_e16_seed0", "s12_e16_seed0", "s12_e4_seed0"])
@pytest.mark.parametrize("direction", DIRS)
def test_bfs_matches_golden(lib, key, direction):
  a = _graph(key)
  with Graph(a) as g:
    g.set_options(direction=direction)
    for rec in G["searches"][key]:
      r = rec["source"]
      lv, pa, st = g.bfs(r)
      assert st["status"] == 0
      assert np.array_equal(lv, ARR[f"{key}_r{r}_levels"]), (key, r, direction)
      assert np.array_equal(pa, ARR[f"{key}_r{r}_parents"]), (key, r, direction)
      assert st["rounds"] == rec["rounds"]
      assert st["visited"] == rec["visited"]


def test_bfs_s16_golden_hashes(lib):
  a = _graph("s16_e16_seed0")
  with Graph(a) as g:
    for rec in G["searches"]["s16_e16_seed0"]:
      lv, pa, st = g.bfs(rec["source"])
      assert sha(lv) == rec["levels_sha"] and sha(pa) == rec["parents_sha"]
      assert st["rounds"] == rec["rounds"]


@pytest.mark.parametrize("direction", DIRS)
def test_bfs_directed_with_self_loops(lib, direction):
  D = csr_from(ARR["dir600_indptr"], ARR["dir600_indices"], 600)
  a = preprocess.preprocess(D)
  with Graph(a) as g:
    g.set_options(direction=direction)
    for rec in G["searches"]["dir600"]:
      r = rec["source"]
      lv, pa, st = g.bfs(r)
      assert np.array_equal(lv, ARR[f"dir600_r{r}_levels"])
      assert np.array_equal(pa, ARR[f"dir600_r{r}_parents"])


@pytest.mark.parametrize("direction", DIRS)
def test_bfs_s16_all_directions_vs_oracle(lib, oracle_mod, direction):
  a = generators.rmat(16, 16, 0)
  roots = [0, 1, 2, 65535, 12345, 40000]
  with Graph(a) as g:
    g.set_options(direction=direction)
    for r in roots:
      lv, pa, st = g.bfs(r)
      rl, rp, rounds = _oracle(oracle_mod, a, r)
      assert np.array_equal(lv, rl) and np.array_equal(pa, rp), (r, direction)
      assert st["rounds"] == rounds


def test_bfs_directed_er_vs_oracle(lib, oracle_mod):
  a = generators.er_directed(14, 8, 4)
  with Graph(a) as g:
    for direction in DIRS:
      g.set_options(direction=direction)
      for r in (0, 5, 777, 16383):
        lv, pa, st = g.bfs(r)
        rl, rp, rounds = _oracle(oracle_mod, a, r)
        assert np.array_equal(lv, rl) and np.array_equal(pa, rp), (r, direction)
        assert st["rounds"] == rounds


def test_bfs_deep_grid_vs_oracle(lib, oracle_mod):
  a = generators.grid2d(96)
  with Graph(a) as g:
    for direction in DIRS:
      g.set_options(direction=direction)
      for r in (0, 96 * 48 + 48):
        lv, pa, st = g.bfs(r)
        rl, rp, rounds = _oracle(oracle_mod, a, r)
        assert np.array_equal(lv, rl) and np.array_equal(pa, rp), (r, direction)
        assert st["rounds"] == rounds


def test_heavy_and_medium_frontier_vertices(lib, oracle_mod):
  # a hub of degree 20000 (grid-split), a few of degree 1000 (one warp each),
  # and light chains behind them
  n = 40000
  src = [0] * 20000 + [1] * 1000 + [2] * 1000
  dst = list(range(100, 20100)) + list(range(20100, 21100)) + list(range(21100, 22100))
  src += [100, 101, 20100, 21100]
  dst += [1, 2, 30000, 30001]
  src += list(range(30000, 39999))
  dst += list(range(30001, 40000))
  a = preprocess.from_edges(n, np.array(src), np.array(dst), symmetrize=True)
  with Graph(a) as g:
    for direction in DIRS:
      g.set_options(direction=direction)
      for r in (0, 1, 39999, 30000):
        lv, pa, st = g.bfs(r)
        rl, rp, rounds = _oracle(oracle_mod, a, r)
        assert np.array_equal(lv, rl) and np.array_equal(pa, rp), (r, direction)
        assert st["rounds"] == rounds


def test_edge_cases(lib, oracle_mod):
  # single vertex, no edges
  one = preprocess.from_edges(1, np.array([], dtype=np.int64), np.array([], dtype=np.int64))
  with Graph(one) as g:
    lv, pa, st = g.bfs(0)
    assert lv.tolist() == [0] and pa.tolist() == [0] and st["rounds"] == 1
  # no edges at all: every search is the root alone
  empty = preprocess.from_edges(100, np.array([], dtype=np.int64), np.array([], dtype=np.int64))
  with Graph(empty) as g:
    lv, pa, st = g.bfs(57)
    assert (lv >= 0).sum() == 1 and lv[57] == 0 and pa[57] == 57 and st["visited"] == 1
    with pytest.raises(_lib.CgError) as e:
      g.bfs(100)
    assert e.value.status == _lib.CG_ERR_INVALID_ARG
    with pytest.raises(_lib.CgError):
      g.bfs(-1)
  # isolated root in a real graph; n not a multiple of 32
  a = preprocess.from_edges(1000, np.arange(0, 998), np.arange(1, 999), symmetrize=True)
  with Graph(a) as g:
    lv, pa, st = g.bfs(999)
    assert st["rounds"] == 1 and (lv >= 0).sum() == 1
    lv, pa, st = g.bfs(0)
    rl, rp, rounds = _oracle(oracle_mod, a, 0)
    assert np.array_equal(lv, rl) and np.array_equal(pa, rp) and rounds == 999 == st["rounds"]


def test_level_cap_and_bounded_wait_report_errors(lib, oracle_mod):
  a = generators.grid2d(40)
  with Graph(a) as g:
    g.set_options(level_cap=5)
    with pytest.raises(_lib.CgError) as e:
      g.bfs(0)
    assert e.value.status == _lib.CG_ERR_LEVEL_CAP
    # a grid-wide wait that can never complete must end with a status, and
    # leave the context usable
    g.set_options(level_cap=0, test_unmatched_wait=1, wait_timeout_ms=50)
    with pytest.raises(_lib.CgError) as e:
      g.bfs(0)
    assert e.value.status == _lib.CG_ERR_TIMEOUT
    g.set_options(test_unmatched_wait=0, wait_timeout_ms=1000)
    lv, pa, st = g.bfs(0)
    rl, rp, _ = _oracle(oracle_mod, a, 0)
    assert np.array_equal(lv, rl) and np.array_equal(pa, rp)


def test_device_outputs_and_edge_count(lib, oracle_mod):
  torch = pytest.importorskip("torch")
  a = _graph("s12_e16_seed0")
  recs = G["searches"]["s12_e16_seed0"]
  k = len(recs)
  with Graph(a) as g:
    d_lv = torch.empty((k, a.n), dtype=torch.int32, device="cuda")
    d_pa = torch.empty((k, a.n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for i, rec in enumerate(recs):
      g.bfs_device(rec["source"], d_lv[i], d_pa[i])
    st = g.last_stats()
    assert st["status"] == 0
    m = g.count_edges(d_lv, k)
    lv = d_lv.cpu().numpy()
    for i, rec in enumerate(recs):
      assert np.array_equal(lv[i], ARR[f"s12_e16_seed0_r{rec['source']}_levels"])
      assert m[i] == rec["m"]
  D = csr_from(ARR["dir600_indptr"], ARR["dir600_indices"], 600)
  d = preprocess.preprocess(D)
  with Graph(d) as g:
    recs = G["searches"]["dir600"]
    d_lv = torch.empty((len(recs), 600), dtype=torch.int32, device="cuda")
    d_pa = torch.empty((len(recs), 600), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for i, rec in enumerate(recs):
      g.bfs_device(rec["source"], d_lv[i], d_pa[i])
    g.last_stats()
    m = g.count_edges(d_lv, len(recs))
    assert m.tolist() == [rec["m"] for rec in recs]


def test_pinned_readback_and_graph500_driver(lib, oracle_mod):
  from ceregraphs_gb300 import graph500
  a = _graph("s12_e16_seed0")
  roots = graph500.pick_sources(a, 16, 1)
  A = a.scipy_csr()

  def validate(root, levels, parents):
    return oracle_mod.graph500_validate(A, root, levels, parents) == []

  with Graph(a) as g:
    summary = graph500.run_graph500(g, a, roots, validate=validate)
  d = summary.as_dict()
  assert d["num_searches"] == 16 and d["num_correctness_fail"] == 0
  assert all(s.gteps > 0 for s in summary.searches)
