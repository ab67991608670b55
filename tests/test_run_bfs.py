"""The single-search driver (run_bfs) on the CPU: its flow -- options, round
report, edge count, GTEPS, tree checks, the scipy tie-break count, the CSV row
and the exit code -- with the graph handle's device calls answered by the
oracle (a fake of the handle, not of the driver)."""
import csv
import types

import numpy as np
import pytest

from ceregraphs_gb300 import _lib, generators, run_bfs, run_graph500

CHECKS = ("root", "tree", "edges", "span", "tree_edge", "lowest")


class FakeGraph:
  """Graph's bfs / validate / set_options / close, computed by the oracle."""

  def __init__(self, oracle_mod, a, plant=None):
    self.o, self.a, self.plant = oracle_mod, a, plant
    self.out_off, self.out_idx = a.out_lists()
    self.opts = {}
    self.closed = False

  def set_options(self, **kw):
    self.opts.update(kw)

  def bfs(self, root, levels=None, parents=None):
    lv, pa, rounds = self.o.bfs(self.out_off, self.out_idx, self.a.in_off, self.a.in_idx, root)
    if self.opts.get("parent_rule") == _lib.CG_PARENT_FIFO:
      pa = self.o.fifo_parents(self.a.in_off, self.a.in_idx, lv, root)
    elif self.plant is not None:
      pa = pa.copy()
      pa[self.plant] = self.plant  # a vertex as its own parent: no such edge
    if levels is not None:
      levels[:] = lv
    if parents is not None:
      parents[:] = pa
    st = {"rounds": rounds, "pull_rounds": 0, "switches": 0, "device_ms": 0.25,
          "round_ns": [2000] * rounds, "direction_history": [0] * rounds,
          "nf_history": [int(np.sum(lv == i + 1)) for i in range(rounds)]}
    return lv, pa, st

  def validate(self, roots, d_levels, d_parents):
    c = self.o.validation_counts(self.a.in_off, self.a.in_idx, roots[0],
                                 np.asarray(d_levels), np.asarray(d_parents))
    return [{k: {"failures": c[k][0], "first": c[k][1]} for k in CHECKS}]

  def close(self):
    self.closed = True


def _patch(monkeypatch, graph, a):
  monkeypatch.setattr(run_graph500, "kernel1", lambda args: (graph, a, 0.0, "fake.mtx"))
  monkeypatch.setattr(run_bfs, "host_buffers", lambda n: (
      types.SimpleNamespace(array=np.empty(n, np.int32)),
      types.SimpleNamespace(array=np.empty(n, np.int32))))
  monkeypatch.setattr(run_bfs, "device_copy", lambda x: x)


def test_run_bfs_row_and_counts(monkeypatch, tmp_path, oracle_mod):
  from ceregraphs_gb300.graph500 import EdgeCounter, pick_sources
  a = generators.rmat(10, 16, 0)
  root = pick_sources(a, 1, 3)[0]
  g = FakeGraph(oracle_mod, a)
  _patch(monkeypatch, g, a)
  out = tmp_path / "bfs_timing.csv"
  rc = run_bfs.main(["--rmat", "10", "16", "0", "--source", str(root), "--directional",
                     "--csv", str(out)])
  assert rc == 0 and g.closed
  assert g.opts["direction"] == _lib.CG_DIR_TAU
  assert g.opts["parent_rule"] == _lib.CG_PARENT_LOWEST  # restored after the FIFO search
  rows = list(csv.DictReader(open(out)))
  assert len(rows) == 1
  r = rows[0]
  lv, pa, rounds = oracle_mod.bfs(*a.out_lists(), a.in_off, a.in_idx, root)
  fp = oracle_mod.fifo_parents(a.in_off, a.in_idx, lv, root)
  assert r["correctness_ok"] == "True" and r["failed_checks"] == ""
  assert int(r["scipy_parent_differs"]) == int(np.sum((fp != pa) & (lv > 0)))
  assert int(r["m_edges_traversed"]) == EdgeCounter(a).m(lv >= 0)
  assert int(r["rounds_completed"]) == rounds and r["directions"] == "T" * min(rounds, 10)
  assert float(r["gteps_no_transfer"]) == pytest.approx(
      int(r["m_edges_traversed"]) / 0.25e-3 / 1e9)
  # a second run appends under the same header
  assert run_bfs.main(["--rmat", "10", "16", "0", "--source", str(root), "--directional",
                       "--csv", str(out), "--nocorrectness"]) == 0
  assert len(list(csv.DictReader(open(out)))) == 2


def test_run_bfs_reports_a_bad_tree(monkeypatch, oracle_mod):
  a = generators.rmat(9, 16, 1)
  lv, _, _ = oracle_mod.bfs(*a.out_lists(), a.in_off, a.in_idx, 0)
  bad = int(np.nonzero(lv == 2)[0][0])
  _patch(monkeypatch, FakeGraph(oracle_mod, a, plant=bad), a)
  assert run_bfs.main(["--rmat", "9", "16", "1", "--source", "0", "--notimings"]) == 1


def test_run_bfs_arguments():
  a = run_bfs.parse_args(["--rmat", "8", "16", "0"])
  assert a.direction == "topdown" and a.source == 0 and a.max_rounds == 10
  assert run_bfs.parse_args(["--infile_mtx", "g.mtx", "--directional"]).direction == "tau"
  assert run_bfs.parse_args(["--rmat", "8", "16", "0", "--direction", "auto"]).direction == "auto"
  with pytest.raises(SystemExit):
    run_bfs.parse_args(["--rmat", "8", "16", "0", "--directional", "--direction", "auto"])
  with pytest.raises(SystemExit):
    run_bfs.parse_args(["--source", "3"])   # a graph source is required
