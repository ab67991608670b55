"""Multi-GPU mode: replicas.

Searches are independent units, so N GPUs each hold a full copy of the graph
and take a disjoint share of the roots (or of the multi-source lane batches);
no data crosses between GPUs during a search.  Results meet on the host:
``gather`` collects every rank's per-root records with torch.distributed
(any backend; the tests use gloo on CPU).
"""
from __future__ import annotations


def shard(items, rank, world):
  """Round-robin share of ``items`` for ``rank`` (order kept)."""
  if world <= 0 or not 0 <= rank < world:
    raise ValueError("bad rank/world")
  return list(items)[rank::world]


def lane_batches(roots, lanes):
  """Split roots into batches of at most ``lanes`` (64 or 128)."""
  roots = list(roots)
  return [roots[i:i + lanes] for i in range(0, len(roots), lanes)]


def gather(records, group=None):
  """All ranks' record lists, concatenated in rank order (every rank gets it)."""
  import torch.distributed as dist
  if not dist.is_available() or not dist.is_initialized():
    return list(records)
  out = [None] * dist.get_world_size(group)
  dist.all_gather_object(out, list(records), group=group)
  merged = []
  for part in out:
    merged.extend(part)
  return merged
