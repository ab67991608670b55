"""Seed and readback conventions of the reference (bfs/implementation/device_io.py).

On the wafer a search is seeded by writing one bit into the diagonal PE that
owns the root (device_io.py:119-148) and read back from PE column MID with
0xFFFFFFFF marking "no parent" (device_io.py:157-178).  Here the root is a
launch argument and the parent array is written whole by the kernel, with the
same sentinel, so readback is one copy.
"""
from __future__ import annotations

import numpy as np

PARENT_NONE_GLOBAL = 0xFFFFFFFF  # device_io.py:157; reads as -1 through int32


def check_root(root, n):
  """The reference asserts 0 <= root < n (run_graph500.py:109-111)."""
  root = int(root)
  if not 0 <= root < n:
    raise ValueError(f"root {root} out of range [0, {n})")
  return root


def extract_parent_result(n, parent):
  """Parent array as int64 with the sentinel mapped to -1
  (device_io.py:160-178).  Accepts the device's int32 or uint32 view."""
  p = np.asarray(parent)[:n]
  if p.dtype == np.uint32:
    p = p.astype(np.int64)
    return np.where(p == PARENT_NONE_GLOBAL, -1, p)
  return p.astype(np.int64)


def derive_visited_from_parent(n, parent, source):
  """visited[v] = parent[v] >= 0, or v is the source (device_io.py:181-205)."""
  visited = np.asarray(parent)[:n] >= 0
  visited[source] = True
  return visited
