"""Continuous-batching BFS server over device-resident graphs.

Queries (graph, root) arrive over time.  Each graph has a pool (cg_pool_*):
up to 64 or 128 searches in flight as bit lanes of one resumable batched
launch.  Between steps the server admits waiting queries into free lanes --
they join the searches already running -- as long as the HBM budget covers
their outputs (levels + parents, 8 bytes per vertex), and hands back the
queries whose searches ended.  Latency = completion - arrival; throughput =
queries / wall time.  ``serial_baseline`` runs the same arrivals one query at a
time through cg_bfs, the reference's way (run_graph500.py:321-440).

No reference counterpart as a component: the reference runs one root per
launch from a host loop.
"""
from __future__ import annotations

import ctypes
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import check


class Pool:
  """A serving pool on one Graph (cg_pool)."""

  def __init__(self, graph, lane_words=1):
    self.graph = graph
    self._p = ctypes.c_void_p()
    check(_lib.load().cg_pool_create(graph.handle, int(lane_words), ctypes.byref(self._p)),
          "cg_pool_create")
    self.lanes = 64 * int(lane_words)
    self.next_round = 0

  def admit(self, root, d_levels, d_parents):
    """Put a query into a free lane; returns the lane, or None if none is free."""
    lane = ctypes.c_int32()
    rc = _lib.load().cg_pool_admit(self._p, int(root), ctypes.c_void_p(d_levels.data_ptr()),
                                   ctypes.c_void_p(d_parents.data_ptr()), ctypes.byref(lane))
    if rc == _lib.CG_ERR_ADMISSION:
      return None
    check(rc, "cg_pool_admit")
    return lane.value

  def step(self, max_rounds=0, stop_on_finish=True):
    """Advance every lane in flight; returns the lanes whose search ended."""
    done = (ctypes.c_uint64 * 2)()
    nr = ctypes.c_int32()
    check(_lib.load().cg_pool_step(self._p, int(max_rounds), 1 if stop_on_finish else 0, done,
                                   ctypes.byref(nr)), "cg_pool_step")
    self.next_round = nr.value
    out = []
    for w in range(2):
      bits = int(done[w])
      while bits:
        b = (bits & -bits).bit_length() - 1
        out.append(w * 64 + b)
        bits &= bits - 1
    return out

  def release(self, lane):
    check(_lib.load().cg_pool_release(self._p, int(lane)), "cg_pool_release")

  def busy(self):
    n, b = ctypes.c_int32(), ctypes.c_int32()
    check(_lib.load().cg_pool_info(self._p, ctypes.byref(n), ctypes.byref(b)), "cg_pool_info")
    return b.value

  def close(self):
    if self._p is not None and self._p.value:
      _lib.load().cg_pool_destroy(self._p)
    self._p = None

  def __del__(self):
    try:
      self.close()
    except Exception:
      pass


@dataclass
class Query:
  qid: int
  graph: str
  root: int
  t_arrival: float
  t_admit: float = float("nan")
  t_done: float = float("nan")
  lane: int = -1
  levels: object = None   # device tensors while in flight
  parents: object = None


@dataclass
class ServeReport:
  queries: list = field(default_factory=list)
  wall_s: float = 0.0
  steps: int = 0
  unserved: int = 0   # arrivals not started when the run's time limit ran out

  def latencies_ms(self):
    return np.array([(q.t_done - q.t_arrival) * 1e3 for q in self.queries])

  def summary(self):
    lat = self.latencies_ms()
    n = len(lat)
    return {"queries": n, "unserved": self.unserved, "wall_s": self.wall_s,
            "throughput_qps": n / self.wall_s if self.wall_s > 0 else float("nan"),
            "p50_ms": float(np.percentile(lat, 50)) if n else float("nan"),
            "p99_ms": float(np.percentile(lat, 99)) if n else float("nan"),
            "mean_ms": float(lat.mean()) if n else float("nan"), "steps": self.steps}


def poisson_arrivals(rate_qps, count, graph_roots, seed=6):
  """`count` queries: exponential inter-arrival times of mean 1/rate, graph
  uniform over the keys of graph_roots, root uniform over that graph's
  candidate roots.  Returns [(t, graph, root)] sorted by t."""
  rng = np.random.default_rng(seed)
  names = sorted(graph_roots)
  t = np.cumsum(rng.exponential(1.0 / rate_qps, size=count))
  gi = rng.integers(0, len(names), size=count)
  out = []
  for i in range(count):
    cands = graph_roots[names[gi[i]]]
    out.append((float(t[i]), names[gi[i]], int(cands[rng.integers(0, len(cands))])))
  return out


def check_budget(graphs, hbm_budget_bytes):
  """A budget must admit at least one query of every graph (its levels and
  parents, 8 bytes a vertex); otherwise that graph's queries would wait
  forever.  Raises ValueError naming the graph."""
  if hbm_budget_bytes is None:
    return
  for name, g in graphs.items():
    if 8 * g.n > hbm_budget_bytes:
      raise ValueError(f"HBM budget of {hbm_budget_bytes} bytes is below one query's "
                       f"outputs on graph {name!r} ({8 * g.n} bytes)")


class Server:
  """Continuous batching over one pool per resident graph: queries join the
  searches in flight as free lanes; a query that finds its graph's pool idle
  with no other query waiting runs as a per-root search instead.  With
  `batch_min`, a backlog of at least that many waiting queries stops joining
  the pool; once the pool is idle it starts them (up to its lanes) as one
  batched search with outputs written after the rounds -- a backlog's cheapest
  form -- while a shorter queue keeps joining searches in flight."""

  def __init__(self, graphs, lane_words=1, hbm_budget_bytes=None, max_rounds=0,
               on_done=None, solo_max=1, batch_min=None):
    import torch
    check_budget(graphs, hbm_budget_bytes)
    self.torch = torch
    self.graphs = graphs                      # name -> engine.Graph
    self.lane_words = lane_words
    # an idle pool with at most this many queries waiting runs them as per-root
    # searches (light load: a lone query does not pay for a lane sweep)
    self.solo_max = solo_max
    self.solo = 0
    self.batch_min = batch_min
    self.batched = 0                          # queries served by batched searches
    for g in graphs.values():
      g.set_options(lane_words=int(lane_words))
    self.pools = {k: Pool(g, lane_words) for k, g in graphs.items()}
    self.budget = hbm_budget_bytes
    self.in_use = 0
    self.max_rounds = max_rounds
    self.on_done = on_done                    # callback(query) before outputs are freed
    self._free = {k: [] for k in graphs}      # reusable output buffers per graph

  def _buffers(self, name):
    n = self.graphs[name].n
    if self._free[name]:
      return self._free[name].pop()
    return (self.torch.empty(n, dtype=self.torch.int32, device="cuda"),
            self.torch.empty(n, dtype=self.torch.int32, device="cuda"))

  def _bytes(self, name):
    return 8 * self.graphs[name].n

  def run(self, arrivals, realtime=True, time_limit=None):
    """Serve [(t, graph, root)].  With realtime the host clock paces the
    arrivals; otherwise every query is available at once (throughput mode).
    After `time_limit` seconds no query is admitted any more: those in flight
    finish, the rest count as unserved."""
    torch = self.torch
    torch.cuda.synchronize()
    waiting = {k: deque() for k in self.graphs}
    inflight = {k: {} for k in self.graphs}   # lane -> Query
    todo = deque(Query(i, g, r, t) for i, (t, g, r) in enumerate(arrivals))
    report = ServeReport()
    t0 = time.perf_counter()
    clock = (lambda: time.perf_counter() - t0) if realtime else (lambda: float("inf"))
    while todo or any(waiting[k] or inflight[k] for k in self.graphs):
      if time_limit is not None and time.perf_counter() - t0 > time_limit:
        report.unserved += len(todo) + sum(len(w) for w in waiting.values())
        todo.clear()
        for w in waiting.values():
          w.clear()
        if not any(inflight.values()):
          break
      now = clock()
      while todo and todo[0].t_arrival <= now:
        q = todo.popleft()
        if not realtime:
          q.t_arrival = time.perf_counter() - t0
        waiting[q.graph].append(q)
      for name, pool in self.pools.items():
        wq = waiting[name]
        if (self.batch_min and not inflight[name] and len(wq) >= self.batch_min and
            self._batch(name, pool, wq, report, t0)):
          continue
        if wq and not inflight[name] and len(wq) <= self.solo_max:
          g = self.graphs[name]
          while wq:
            q = wq.popleft()
            lv, pa = self._buffers(name)
            q.t_admit = time.perf_counter() - t0
            g.bfs_device(q.root, lv, pa)
            st = g.last_stats()
            if st["status"] != 0:
              raise RuntimeError(f"search failed: {st}")
            q.t_done = time.perf_counter() - t0
            q.levels, q.parents = lv, pa
            if self.on_done is not None:
              self.on_done(q)
            q.levels = q.parents = None
            self._free[name].append((lv, pa))
            report.queries.append(q)
            self.solo += 1
          continue
        while wq:
          if self.budget is not None and self.in_use + self._bytes(name) > self.budget:
            break
          if self.batch_min and len(wq) >= self.batch_min:
            break  # a backlog waits for the pool to drain, then runs as one batch
          q = wq[0]
          lv, pa = self._buffers(name)
          lane = pool.admit(q.root, lv, pa)
          if lane is None:
            self._free[name].append((lv, pa))
            break
          wq.popleft()
          q.lane, q.levels, q.parents = lane, lv, pa
          q.t_admit = time.perf_counter() - t0
          inflight[name][lane] = q
          self.in_use += self._bytes(name)
      stepped = False
      for name, pool in self.pools.items():
        if not inflight[name]:
          continue
        done = pool.step(self.max_rounds, stop_on_finish=True)
        report.steps += 1
        stepped = True
        tnow = time.perf_counter() - t0
        for lane in done:
          q = inflight[name].pop(lane)
          q.t_done = tnow
          if self.on_done is not None:
            self.on_done(q)
          pool.release(lane)
          self._free[name].append((q.levels, q.parents))
          q.levels = q.parents = None
          self.in_use -= self._bytes(name)
          report.queries.append(q)
      if not stepped and todo and realtime:
        wait = todo[0].t_arrival - clock()
        if wait > 0:
          time.sleep(min(wait, 0.001))
    report.wall_s = time.perf_counter() - t0
    report.queries.sort(key=lambda q: q.qid)
    return report

  def _batch(self, name, pool, wq, report, t0):
    """The waiting queries of an idle pool (up to its lanes, within the HBM
    budget) as one batched search, run to the end; False if none fits."""
    torch = self.torch
    g = self.graphs[name]
    take = min(len(wq), pool.lanes)
    if self.budget is not None:
      take = min(take, max(0, (self.budget - self.in_use) // self._bytes(name)))
    if take == 0:
      return False
    qs = [wq.popleft() for _ in range(take)]
    tnow = time.perf_counter() - t0
    for q in qs:
      q.t_admit = tnow
    nbytes = self._bytes(name) * take
    self.in_use += nbytes
    lv = torch.empty((take, g.n), dtype=torch.int32, device="cuda")
    pa = torch.empty((take, g.n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()          # the outputs exist before the graph's stream writes them
    g.msbfs_device([q.root for q in qs], lv, pa)
    st = g.last_stats()               # waits for the batch
    if st["status"] != 0:
      raise RuntimeError(f"batched search failed: {st}")
    tnow = time.perf_counter() - t0
    for i, q in enumerate(qs):
      q.t_done = tnow
      q.levels, q.parents = lv[i], pa[i]
      if self.on_done is not None:
        self.on_done(q)
      q.levels = q.parents = None
      report.queries.append(q)
    del lv, pa
    self.in_use -= nbytes
    self.batched += take
    report.steps += 1
    return True

  def close(self):
    for p in self.pools.values():
      p.close()


class BatchServer:
  """Dynamic batching: whenever a graph has no search in flight, the queries
  waiting for it start together -- one batched launch (64 or 128 bit lanes,
  outputs written once after the rounds) when at least ``batch_min`` wait,
  else one per-root search each (the lower latency at light load).  Queries
  that arrive meanwhile wait for the graph's next launch.  Launches go to the
  graphs' own streams but are chained by events, so at most one of these
  persistent, grid-synchronising kernels runs at a time (two of them sharing
  the GPU could each wait at a grid-wide barrier for blocks the other one
  keeps from being scheduled)."""

  def __init__(self, graphs, lane_words=1, hbm_budget_bytes=None, batch_min=4, on_done=None):
    import torch
    check_budget(graphs, hbm_budget_bytes)
    self.torch = torch
    self.graphs = graphs
    self.lanes = 64 * int(lane_words)
    for g in graphs.values():
      g.set_options(lane_words=int(lane_words))
    self.budget = hbm_budget_bytes
    self.batch_min = batch_min
    self.on_done = on_done
    self.in_use = 0
    self.launches = {"batched": 0, "per_root": 0}
    self._last = None                       # event of the latest launch, any graph

  def _launch(self, name, qs):
    torch = self.torch
    g = self.graphs[name]
    k = len(qs)
    lv = torch.empty((k, g.n), dtype=torch.int32, device="cuda")
    pa = torch.empty((k, g.n), dtype=torch.int32, device="cuda")
    stream = torch.cuda.ExternalStream(g.stream)
    # the outputs were allocated on torch's stream: the graph's stream waits for it
    ready = torch.cuda.Event()
    ready.record(torch.cuda.current_stream())
    stream.wait_event(ready)
    if self._last is not None:
      stream.wait_event(self._last)
    if k >= self.batch_min:
      g.msbfs_device([q.root for q in qs], lv, pa)
      self.launches["batched"] += 1
    else:
      for i, q in enumerate(qs):
        g.bfs_device(q.root, lv[i], pa[i])
      self.launches["per_root"] += k
    done = torch.cuda.Event()
    done.record(stream)
    self._last = done
    for i, q in enumerate(qs):
      q.levels, q.parents = lv[i], pa[i]
    return done

  def run(self, arrivals, realtime=True, time_limit=None):
    """As Server.run: after `time_limit` seconds nothing new is launched."""
    torch = self.torch
    torch.cuda.synchronize()
    waiting = {k: deque() for k in self.graphs}
    inflight = {}                           # graph -> (queries, event, bytes)
    todo = deque(Query(i, g, r, t) for i, (t, g, r) in enumerate(arrivals))
    report = ServeReport()
    t0 = time.perf_counter()
    clock = (lambda: time.perf_counter() - t0) if realtime else (lambda: float("inf"))
    while todo or inflight or any(waiting.values()):
      if time_limit is not None and time.perf_counter() - t0 > time_limit:
        report.unserved += len(todo) + sum(len(w) for w in waiting.values())
        todo.clear()
        for w in waiting.values():
          w.clear()
        if not inflight:
          break
      now = clock()
      while todo and todo[0].t_arrival <= now:
        q = todo.popleft()
        if not realtime:
          q.t_arrival = time.perf_counter() - t0
        waiting[q.graph].append(q)
      for name, wq in waiting.items():
        if not wq or name in inflight:
          continue
        n = self.graphs[name].n
        take = min(len(wq), self.lanes)
        if self.budget is not None:
          take = min(take, max(0, (self.budget - self.in_use) // (8 * n)))
        if take == 0:
          continue
        qs = [wq.popleft() for _ in range(take)]
        tnow = time.perf_counter() - t0
        for q in qs:
          q.t_admit = tnow
        nbytes = 8 * n * take
        self.in_use += nbytes
        inflight[name] = (qs, self._launch(name, qs), nbytes)
        report.steps += 1
      for name in list(inflight):
        qs, ev, nbytes = inflight[name]
        if not ev.query():
          continue
        tnow = time.perf_counter() - t0
        for q in qs:
          q.t_done = tnow
          if self.on_done is not None:
            self.on_done(q)
          q.levels = q.parents = None
          report.queries.append(q)
        self.in_use -= nbytes
        del inflight[name]
      if not inflight and todo and realtime:
        wait = todo[0].t_arrival - clock()
        if wait > 0:
          time.sleep(min(wait, 0.001))
    report.wall_s = time.perf_counter() - t0
    report.queries.sort(key=lambda q: q.qid)
    return report

  def close(self):
    pass


def serial_baseline(graphs, arrivals, realtime=True, on_done=None, time_limit=None):
  """The same arrivals served one query at a time (FIFO) through cg_bfs with
  device outputs (no batching); after `time_limit` seconds the rest are
  unserved."""
  import torch
  bufs = {k: (torch.empty(g.n, dtype=torch.int32, device="cuda"),
              torch.empty(g.n, dtype=torch.int32, device="cuda")) for k, g in graphs.items()}
  torch.cuda.synchronize()
  report = ServeReport()
  t0 = time.perf_counter()
  for i, (t, name, root) in enumerate(arrivals):
    now = time.perf_counter() - t0
    if time_limit is not None and now > time_limit:
      report.unserved = len(arrivals) - i
      break
    if realtime and t > now:
      time.sleep(t - now)
    q = Query(i, name, root, t if realtime else time.perf_counter() - t0)
    g = graphs[name]
    lv, pa = bufs[name]
    q.t_admit = time.perf_counter() - t0
    g.bfs_device(root, lv, pa)
    g.last_stats()
    q.t_done = time.perf_counter() - t0
    if on_done is not None:
      q.levels, q.parents = lv, pa
      on_done(q)
      q.levels = q.parents = None
    report.queries.append(q)
  report.wall_s = time.perf_counter() - t0
  return report
