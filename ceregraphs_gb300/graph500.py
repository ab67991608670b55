"""Graph500-style driver: the GB300 counterpart of bfs/scripts/run_graph500.py.

Kernel 1 (construction) is the one-time upload in ``Graph(...)``; Kernel 2 is
one search per root, each timed from the launch to the parents being in host
memory (the spec's rule that the reference follows, docs/GRAPH500_BENCHMARK.md
sections 1-2), and combined with the harmonic mean (run_graph500.py:130-134).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .bfs_timing import gteps, harmonic_mean
from .device_io import derive_visited_from_parent
from .preprocess import GraphArrays


def out_degree_no_loops(arrays: GraphArrays):
  """Out-degree per vertex minus one for a self-loop (run_graph500.py:119-122):
  column counts of A, i.e. the out-lists."""
  off, idx = arrays.out_lists()
  deg = np.diff(off)
  owner = np.repeat(np.arange(arrays.n, dtype=np.int64), deg)
  loops = np.bincount(owner[idx == owner], minlength=arrays.n)
  return deg - (loops > 0).astype(np.int64)


def pick_sources(arrays: GraphArrays, num_searches, seed):
  """Graph500 roots: degree >= 1 not counting self-loops, sampled without
  replacement with ``default_rng(seed).choice`` (run_graph500.py:106-127)."""
  candidates = np.nonzero(out_degree_no_loops(arrays) > 0)[0]
  num = min(num_searches, len(candidates))
  rng = np.random.default_rng(seed)
  return rng.choice(candidates, size=num, replace=False).tolist()


class EdgeCounter:
  """m of bfs_timing.py:379-398 as a per-vertex weight, so each search costs
  O(n): symmetric A -> w[r] = #{c in row r : c <= r}; directed A -> w[c] =
  column count of c.  m = sum of w over the visited vertices."""

  def __init__(self, arrays: GraphArrays):
    if arrays.symmetric:
      deg = np.diff(arrays.in_off)
      owner = np.repeat(np.arange(arrays.n, dtype=np.int64), deg)
      self.w = np.bincount(owner[arrays.in_idx <= owner], minlength=arrays.n).astype(np.int64)
      self.convention = "undirected_dedup"
    else:
      self.w = np.diff(arrays.out_off).astype(np.int64)
      self.convention = "directed_source_visited"

  def m(self, visited):
    return int(self.w[np.asarray(visited, dtype=bool)].sum())


@dataclass
class SearchRecord:
  source: int
  rounds: int
  visited: int
  m: int
  seconds: float
  gteps: float
  pull_rounds: int = 0
  correctness_ok: bool | None = None


@dataclass
class RunSummary:
  searches: list = field(default_factory=list)
  construction_seconds: float = 0.0

  @property
  def harmonic_mean_gteps(self):
    return harmonic_mean([s.gteps for s in self.searches])

  def as_dict(self):
    g = [s.gteps for s in self.searches if np.isfinite(s.gteps) and s.gteps > 0]
    return {"num_searches": len(self.searches),
            "num_correctness_fail": sum(1 for s in self.searches if s.correctness_ok is False),
            "construction_time_seconds": self.construction_seconds,
            "harmonic_mean_gteps": self.harmonic_mean_gteps,
            "min_gteps": min(g) if g else float("nan"),
            "median_gteps": float(np.median(g)) if g else float("nan"),
            "max_gteps": max(g) if g else float("nan")}


def run_graph500(graph, arrays: GraphArrays, roots, validate=None, pinned=True):
  """One search per root through the C ABI (cg_bfs: launch, every round on the
  device, parents and levels copied to host memory).  ``validate(root,
  levels, parents) -> bool`` is an optional per-search check."""
  from .engine import PinnedBuffer
  counter = EdgeCounter(arrays)
  if pinned:
    lv_buf, pa_buf = PinnedBuffer(arrays.n), PinnedBuffer(arrays.n)
    levels, parents = lv_buf.array, pa_buf.array
  else:
    levels = np.empty(arrays.n, dtype=np.int32)
    parents = np.empty(arrays.n, dtype=np.int32)
  summary = RunSummary()
  for root in roots:
    t0 = time.perf_counter()
    _, _, st = graph.bfs(int(root), levels, parents)
    t1 = time.perf_counter()
    visited = derive_visited_from_parent(arrays.n, parents, int(root))
    m = counter.m(visited)
    ok = None if validate is None else bool(validate(int(root), levels, parents))
    summary.searches.append(SearchRecord(int(root), st["rounds"], int(visited.sum()), m, t1 - t0,
                                         gteps(m, t1 - t0), st["pull_rounds"], ok))
  return summary
