"""Per-graph autotuner for the search knobs.

Results never depend on the knobs (levels and parents are bit-exact under any
direction policy, lane width or block size), so tuning is a pure timing
search: each candidate runs a few sample searches on the resident graph, timed
with CUDA events on the handle's stream, and the fastest wins.  Choices are
cached per graph fingerprint (n, nnz, symmetry and a hash of a sample of the
offsets) in a JSON file, so a graph is tuned once.

Knobs (cg_options): per-root -- alpha and beta of the push/pull switch
(Beamer's rule) and the block size of the persistent kernel; batched --
lane width (64 or 128 roots a pass), the pull threshold ms_alpha and the
block size.
"""
from __future__ import annotations

import hashlib
import itertools
import json
import os

import numpy as np

PER_ROOT_SPACE = {"alpha": [4.0, 8.0, 15.0, 30.0], "beta": [9.0, 18.0, 36.0],
                  "block_size": [256, 512]}
BATCHED_SPACE = {"lane_words": [1, 2], "ms_alpha": [1.0, 2.0, 4.0, 8.0, 16.0],
                 "block_size": [256, 512]}


def fingerprint(arrays):
  """Stable identity of a graph: sizes plus a hash of 4096 sampled offsets
  and indices."""
  h = hashlib.sha256()
  h.update(np.array([arrays.n, arrays.nnz, int(arrays.symmetric)], dtype=np.int64).tobytes())
  idx = np.linspace(0, arrays.n, num=min(arrays.n + 1, 4096), dtype=np.int64)
  h.update(np.asarray(arrays.in_off)[idx].tobytes())
  if arrays.nnz:
    j = np.linspace(0, arrays.nnz - 1, num=min(arrays.nnz, 4096), dtype=np.int64)
    h.update(np.asarray(arrays.in_idx)[j].tobytes())
  return h.hexdigest()[:24]


class Cache:
  def __init__(self, path=None):
    self.path = path or os.environ.get(
        "CEREGRAPHS_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache",
                                              "ceregraphs_gb300_tune.json"))
    self.data = {}
    try:
      with open(self.path, encoding="utf-8") as f:
        self.data = json.load(f)
    except (OSError, ValueError):
      self.data = {}

  def get(self, key):
    return self.data.get(key)

  def put(self, key, value):
    self.data[key] = value
    try:
      os.makedirs(os.path.dirname(self.path), exist_ok=True)
      tmp = self.path + f".{os.getpid()}.tmp"
      with open(tmp, "w", encoding="utf-8") as f:
        json.dump(self.data, f, indent=1, sort_keys=True)
      os.replace(tmp, self.path)
    except OSError:
      pass


def _time_per_root(graph, roots, d_lv, d_pa, reps):
  import torch
  stream = torch.cuda.ExternalStream(graph.stream)
  for r in roots[:2]:
    graph.bfs_device(int(r), d_lv, d_pa)
  graph.last_stats()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record(stream)
  for _ in range(reps):
    for r in roots:
      graph.bfs_device(int(r), d_lv, d_pa)
  e1.record(stream)
  torch.cuda.synchronize()
  st = graph.last_stats()
  if st["status"] != 0:
    return float("inf")
  return e0.elapsed_time(e1) / (reps * len(roots))


def _time_batched(graph, roots, d_lv, d_pa, reps):
  import torch
  stream = torch.cuda.ExternalStream(graph.stream)
  graph.msbfs_device(roots, d_lv, d_pa)
  graph.last_stats()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record(stream)
  for _ in range(reps):
    graph.msbfs_device(roots, d_lv, d_pa)
  e1.record(stream)
  torch.cuda.synchronize()
  st = graph.last_stats()
  if st["status"] != 0:
    return float("inf")
  return e0.elapsed_time(e1) / (reps * len(roots))


def tune(graph, arrays, roots, mode="per_root", space=None, reps=2, cache=None,
         max_candidates=None):
  """Time each candidate of `space` on `roots` and set the best on `graph`.
  Returns {"mode", "options", "ms_per_root", "candidates", "cached"}."""
  import torch
  space = dict(space or (PER_ROOT_SPACE if mode == "per_root" else BATCHED_SPACE))
  key = f"{fingerprint(arrays)}:{mode}"
  cache = cache if cache is not None else Cache()
  hit = cache.get(key)
  base = graph.options()
  if hit is not None:
    graph.set_options(base, **hit["options"])
    return dict(hit, cached=True)
  roots = [int(r) for r in roots]
  k = len(roots) if mode != "per_root" else 1
  d_lv = torch.empty((k, arrays.n), dtype=torch.int32, device="cuda")
  d_pa = torch.empty((k, arrays.n), dtype=torch.int32, device="cuda")
  torch.cuda.synchronize()
  names = sorted(space)
  combos = list(itertools.product(*(space[nm] for nm in names)))
  if max_candidates:
    combos = combos[:max_candidates]
  results = []
  for combo in combos:
    opts = dict(zip(names, combo))
    graph.set_options(base, **opts)
    if mode == "per_root":
      t = _time_per_root(graph, roots, d_lv[0], d_pa[0], reps)
    else:
      t = _time_batched(graph, roots, d_lv, d_pa, reps)
    results.append((t, opts))
  results.sort(key=lambda x: x[0])
  best_t, best = results[0]
  graph.set_options(base, **best)
  out = {"mode": mode, "options": best, "ms_per_root": best_t,
         "candidates": [{"ms_per_root": t, **o} for t, o in results]}
  cache.put(key, {k2: v for k2, v in out.items() if k2 != "candidates"})
  return dict(out, cached=False)
