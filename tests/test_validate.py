"""Graph500 result validation on the device (cg_validate_device) against the
oracle's restatement of the same checks, on clean search results and on
results with mistakes planted on the host."""
import numpy as np
import pytest

from ceregraphs_gb300 import generators

CHECKS = ("root", "tree", "edges", "span", "tree_edge", "lowest")


def _plant(a, lv, pa, root, rng):
  """Copies of (levels, parents) with one mistake of each kind; returns a
  list of (name, levels, parents, checks expected to fail)."""
  n = a.n
  reached = np.nonzero((lv > 0))[0]
  out = []
  # a parent out of range
  l2, p2 = lv.copy(), pa.copy()
  v = reached[len(reached) // 2]
  p2[v] = n + 5
  out.append(("parent_out_of_range", l2, p2, {"tree"}))
  # a reached vertex whose parent is garbage below -1
  l2, p2 = lv.copy(), pa.copy()
  p2[reached[1]] = -7
  out.append(("parent_garbage", l2, p2, {"tree", "span"}))
  # the root's parent moved
  l2, p2 = lv.copy(), pa.copy()
  p2[root] = reached[0]
  out.append(("root_parent", l2, p2, {"root"}))
  # a reached vertex marked unreached in levels only
  l2, p2 = lv.copy(), pa.copy()
  l2[reached[3]] = -1
  out.append(("levels_disagree", l2, p2, {"span"}))
  # a parent one level up that is not the lowest one (valid Graph500 tree)
  in_off, in_idx = a.in_off, a.in_idx
  for v in reached[::7]:
    nb = in_idx[in_off[v]:in_off[v + 1]]
    up = nb[lv[nb] == lv[v] - 1]
    if len(up) >= 2:
      l2, p2 = lv.copy(), pa.copy()
      p2[v] = up[-1]
      out.append(("not_lowest", l2, p2, {"lowest"}))
      break
  # a parent one level up that is not an in-neighbour
  for v in reached[::5]:
    nb = set(in_idx[in_off[v]:in_off[v + 1]].tolist())
    cands = np.nonzero(lv == lv[v] - 1)[0]
    cands = [c for c in cands[:200].tolist() if c not in nb]
    if cands:
      l2, p2 = lv.copy(), pa.copy()
      p2[v] = cands[0]
      out.append(("not_an_edge", l2, p2, {"tree_edge", "lowest"}))
      break
  # a leaf pushed one level deeper than an in-neighbour allows
  l2, p2 = lv.copy(), pa.copy()
  v = int(np.argmax(lv))
  l2[v] += 2
  out.append(("level_skips", l2, p2, {"tree", "edges"}))
  return out


def test_oracle_counts_clean_and_planted(oracle_mod):
  a = generators.rmat(10, 8, 3)
  out_off, out_idx = a.out_lists()
  rng = np.random.default_rng(0)
  root = 1
  lv, pa, _ = oracle_mod.bfs(out_off, out_idx, a.in_off, a.in_idx, root)
  clean = oracle_mod.validation_counts(a.in_off, a.in_idx, root, lv, pa)
  assert all(clean[c] == (0, -1) for c in CHECKS), clean
  for name, l2, p2, expect in _plant(a, lv, pa, root, rng):
    got = oracle_mod.validation_counts(a.in_off, a.in_idx, root, l2, p2)
    failing = {c for c in CHECKS if got[c][0] > 0}
    assert expect <= failing, (name, got)
    # the Graph500 checks (not the lowest-index rule) agree on validity
    g500 = oracle_mod.graph500_validate(a.scipy_csr(), root, l2, p2)
    assert bool(g500) == bool(failing - {"lowest"}), (name, g500, got)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["rmat", "er_directed", "grid"])
def test_device_validator_matches_oracle(built_lib, oracle_mod, kind):
  import torch
  from ceregraphs_gb300.engine import Graph
  a = {"rmat": lambda: generators.rmat(13, 16, 5),
       "er_directed": lambda: generators.er_directed(12, 6, 9),
       "grid": lambda: generators.grid2d(50)}[kind]()
  rng = np.random.default_rng(1)
  roots = [0, 7, a.n // 2]
  with Graph(a) as g:
    k = len(roots)
    lv = torch.empty((k, a.n), dtype=torch.int32, device="cuda")
    pa = torch.empty_like(lv)
    torch.cuda.synchronize()
    g.msbfs_device(roots, lv, pa)
    g.last_stats()
    res = g.validate(roots, lv, pa)
    hl, hp = lv.cpu().numpy(), pa.cpu().numpy()
    for i, r in enumerate(roots):
      want = oracle_mod.validation_counts(a.in_off, a.in_idx, r, hl[i], hp[i])
      assert all(res[i][c]["failures"] == 0 for c in CHECKS), (r, res[i])
      assert all(want[c] == (0, -1) for c in CHECKS)
    # planted mistakes, several searches per call
    cases = _plant(a, hl[0], hp[0], roots[0], rng)
    L = torch.from_numpy(np.stack([c[1] for c in cases])).cuda()
    P = torch.from_numpy(np.stack([c[2] for c in cases])).cuda()
    res = g.validate([roots[0]] * len(cases), L, P)
    for (name, l2, p2, expect), got in zip(cases, res):
      want = oracle_mod.validation_counts(a.in_off, a.in_idx, roots[0], l2, p2)
      for c in CHECKS:
        assert (got[c]["failures"], got[c]["first"]) == want[c], (name, c, got, want)
      assert expect <= {c for c in CHECKS if want[c][0] > 0}, name


@pytest.mark.gpu
def test_device_validator_at_scale(built_lib):
  """Every one of 64 batched searches at scale 18 validates clean."""
  import torch
  from ceregraphs_gb300 import graph500
  from ceregraphs_gb300.engine import Graph
  a = generators.rmat(18, 16, 0)
  roots = graph500.pick_sources(a, 64, 1)
  with Graph(a) as g:
    lv = torch.empty((64, a.n), dtype=torch.int32, device="cuda")
    pa = torch.empty_like(lv)
    torch.cuda.synchronize()
    g.msbfs_device(roots, lv, pa)
    g.last_stats()
    res = g.validate(roots, lv, pa)
    assert all(r[c]["failures"] == 0 for r in res for c in CHECKS)


@pytest.mark.gpu
@pytest.mark.parametrize("lane_words", [1, 2])
def test_batched_trees_at_the_benchmark_scale(built_lib, lane_words):
  """The benchmark's graph (R-MAT s21 ef16 seed 0, drawn on the device) and
  its 64 Graph500 roots (seed 1), plus 64 more for 128 lanes: every batched
  search passes the Graph500 checks and the lowest-index rule on the device,
  a size-independent property where the oracle would take minutes."""
  import torch
  from ceregraphs_gb300 import graph500
  g, _ = generators.rmat_device(21, 16, 0, export=False)
  a = g.export()
  k = 64 * lane_words
  roots = graph500.pick_sources(a, k, 1)
  g.set_options(lane_words=lane_words)
  lv = torch.empty((k, a.n), dtype=torch.int32, device="cuda")
  pa = torch.empty_like(lv)
  torch.cuda.synchronize()
  g.msbfs_device(roots, lv, pa)
  assert g.last_stats()["status"] == 0
  res = g.validate(roots, lv, pa)
  assert all(r[c]["failures"] == 0 for r in res for c in CHECKS)
  g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["per-root", "batched"])
def test_driver_end_to_end(built_lib, tmp_path, mode):
  """The run_graph500 driver: R-MAT and a graph file, every search checked on
  the device, CSV rows written."""
  import csv
  from ceregraphs_gb300 import run_graph500
  out = tmp_path / "rows.csv"
  summ = tmp_path / "summary.csv"
  rc = run_graph500.main(["--rmat", "12", "16", "0", "--num-searches", "10", "--mode", mode,
                          "--csv", str(out), "--summary-csv", str(summ), "--quiet"])
  assert rc == 0
  rows = list(csv.DictReader(open(out)))
  assert len(rows) == 10 and all(r["correctness_ok"] == "True" for r in rows)
  assert all(float(r["gteps"]) > 0 for r in rows)
  mtx = tmp_path / "g.mtx"
  mtx.write_text("%%MatrixMarket matrix coordinate pattern general\n6 6 6\n"
                 "2 1\n3 2\n4 3\n5 4\n6 5\n1 6\n")
  rc = run_graph500.main(["--infile_mtx", str(mtx), "--sources", "0,3", "--mode", mode,
                          "--summary-csv", str(summ), "--quiet"])
  assert rc == 0
  s = list(csv.DictReader(open(summ)))
  assert len(s) == 2 and s[1]["num_correctness_fail"] == "0" and s[1]["matrix_symmetric"] == "False"


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["per-root", "batched"])
def test_driver_fifo_parents(built_lib, tmp_path, mode):
  """--parent-rule fifo: scipy's parents, every search still a valid
  Graph500 tree (the lowest-index rule is not judged)."""
  import csv
  from ceregraphs_gb300 import run_graph500
  out = tmp_path / "rows.csv"
  rc = run_graph500.main(["--rmat", "12", "16", "0", "--num-searches", "8", "--mode", mode,
                          "--parent-rule", "fifo", "--csv", str(out), "--quiet"])
  assert rc == 0
  rows = list(csv.DictReader(open(out)))
  assert len(rows) == 8 and all(r["correctness_ok"] == "True" for r in rows)
  assert all(r["parent_rule"] == "fifo" for r in rows)


@pytest.mark.gpu
def test_run_bfs_end_to_end(built_lib, tmp_path, oracle_mod):
  """The single-search driver on the device: one search, its tree checked,
  the tie-break count against scipy's rule, a CSV row."""
  import csv
  from ceregraphs_gb300 import run_bfs
  out = tmp_path / "bfs_timing.csv"
  for extra in ([], ["--directional"], ["--direction", "auto"]):
    rc = run_bfs.main(["--rmat", "12", "16", "0", "--source", "0", "--csv", str(out)] + extra)
    assert rc == 0
  rows = list(csv.DictReader(open(out)))
  assert len(rows) == 3 and all(r["correctness_ok"] == "True" for r in rows)
  a = generators.rmat(12, 16, 0)
  lv, pa, _ = oracle_mod.bfs(*a.out_lists(), a.in_off, a.in_idx, 0)
  fp = oracle_mod.fifo_parents(a.in_off, a.in_idx, lv, 0)
  want = int(np.sum((fp != pa) & (lv > 0)))
  assert all(int(r["scipy_parent_differs"]) == want for r in rows)
  assert [r["direction"] for r in rows] == ["topdown", "tau", "auto"]
