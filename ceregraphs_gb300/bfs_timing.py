"""Search timing and the Graph500 TEPS metric (bfs/implementation/bfs_timing.py).

The reference converts wafer cycle counters at an assumed 875 MHz
(bfs_timing.py:60-62); here search times come from CUDA events or the host
clock, in seconds.  ``compute_m_and_gteps`` keeps the reference's edge-count
rule (bfs_timing.py:379-398):

* symmetric A: m = #{(r, c) in A : r visited and c <= r}  (undirected dedup)
* directed A:  m = #{(r, c) in A : c visited}             (edges out of visited)
"""
from __future__ import annotations

import numpy as np
from scipy import sparse


def compute_m(A_csr, visited, is_symmetric):
  coo = sparse.coo_matrix(A_csr)
  visited = np.asarray(visited, dtype=bool)
  if is_symmetric:
    return int(np.count_nonzero(visited[coo.row] & (coo.col <= coo.row)))
  return int(np.count_nonzero(visited[coo.col]))


def compute_m_and_gteps(A_csr, visited, is_symmetric, search_time_seconds):
  """Returns (m, m_convention, search_time_seconds, gteps)."""
  m = compute_m(A_csr, visited, is_symmetric)
  conv = "undirected_dedup" if is_symmetric else "directed_source_visited"
  gteps = m / search_time_seconds / 1e9 if search_time_seconds > 0 else float("nan")
  return m, conv, search_time_seconds, gteps


def gteps(m, seconds):
  return m / seconds / 1e9 if seconds > 0 else float("nan")


def harmonic_mean(values):
  """Harmonic mean over the finite positive values (run_graph500.py:130-134)."""
  vals = [float(v) for v in values if v > 0 and np.isfinite(v)]
  if not vals:
    return float("nan")
  return len(vals) / sum(1.0 / v for v in vals)
