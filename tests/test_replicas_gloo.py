"""Replica mode's host logic across two processes (gloo, CPU): each rank
searches its share of the roots (with the oracle standing in for the GPU) and
the gathered records equal a single-process run."""
import os
import socket

import numpy as np
import pytest

from ceregraphs_gb300 import generators, graph500, replicas


def _free_port():
  with socket.socket() as s:
    s.bind(("127.0.0.1", 0))
    return s.getsockname()[1]


def _worker(rank, world, port, q):
  import sys
  sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
  import torch.distributed as dist
  from oracle import oracle
  os.environ["MASTER_ADDR"] = "127.0.0.1"
  os.environ["MASTER_PORT"] = str(port)
  dist.init_process_group("gloo", rank=rank, world_size=world)
  a = generators.rmat(10, 16, 0)
  roots = graph500.pick_sources(a, 16, 1)
  mine = replicas.shard(roots, rank, world)
  recs = []
  for r in mine:
    lv, pa, rounds = oracle.bfs(a.in_off, a.in_idx, a.in_off, a.in_idx, r)
    recs.append((r, rounds, int((lv >= 0).sum()), int(pa.sum())))
  allrecs = replicas.gather(recs)
  dist.barrier()
  dist.destroy_process_group()
  q.put((rank, allrecs))


def test_two_rank_replicas_match_single_process():
  import multiprocessing as mp
  ctx = mp.get_context("spawn")
  q = ctx.Queue()
  port = _free_port()
  procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
  for p in procs:
    p.start()
  got = dict(q.get(timeout=240) for _ in procs)
  for p in procs:
    p.join(timeout=60)
    assert p.exitcode == 0
  from oracle import oracle
  a = generators.rmat(10, 16, 0)
  roots = graph500.pick_sources(a, 16, 1)
  want = {}
  for r in roots:
    lv, pa, rounds = oracle.bfs(a.in_off, a.in_idx, a.in_off, a.in_idx, r)
    want[r] = (r, rounds, int((lv >= 0).sum()), int(pa.sum()))
  for rank in (0, 1):
    recs = got[rank]
    assert sorted(x[0] for x in recs) == sorted(roots)
    for rec in recs:
      assert tuple(rec) == want[rec[0]]


def test_shard_and_batches():
  assert replicas.shard(range(10), 1, 3) == [1, 4, 7]
  assert sum(len(replicas.shard(range(10), r, 3)) for r in range(3)) == 10
  b = replicas.lane_batches(range(130), 64)
  assert [len(x) for x in b] == [64, 64, 2]
  with pytest.raises(ValueError):
    replicas.shard([1], 2, 2)
