"""Serving: continuous batching of queries into the lanes of a resumable
batched search.  Every query's result in the mix must equal the same query
run alone (integer results: bit-exact)."""
import numpy as np
import pytest

from ceregraphs_gb300 import generators, graph500, serving


def test_poisson_arrivals_are_deterministic_and_sorted():
  roots = {"a": [1, 2, 3], "b": [7, 8]}
  x = serving.poisson_arrivals(1000.0, 200, roots, seed=6)
  y = serving.poisson_arrivals(1000.0, 200, roots, seed=6)
  assert x == y
  ts = [t for t, _, _ in x]
  assert ts == sorted(ts) and ts[0] > 0
  assert {g for _, g, _ in x} == {"a", "b"}
  assert all(r in roots[g] for _, g, r in x)
  # mean inter-arrival close to 1 / rate
  assert abs(np.mean(np.diff(ts)) - 1e-3) < 3e-4


def test_report_summary():
  rep = serving.ServeReport()
  for i, lat in enumerate([1.0, 2.0, 3.0, 4.0]):
    q = serving.Query(i, "g", 0, 0.0)
    q.t_done = lat / 1e3
    rep.queries.append(q)
  rep.wall_s = 0.5
  s = rep.summary()
  assert s["queries"] == 4 and s["throughput_qps"] == 8.0
  assert s["p50_ms"] == pytest.approx(2.5)


def _alone(oracle_mod, a, root):
  out_off, out_idx = a.out_lists()
  lv, pa, _ = oracle_mod.bfs(out_off, out_idx, a.in_off, a.in_idx, root)
  return lv, pa


@pytest.mark.gpu
@pytest.mark.parametrize("lane_words", [1, 2])
def test_pool_lanes_join_mid_flight(built_lib, oracle_mod, lane_words):
  import torch
  from ceregraphs_gb300.engine import Graph
  a = generators.rmat(14, 16, 1)
  roots = graph500.pick_sources(a, 3 * 64 * lane_words, 4)
  want = {r: _alone(oracle_mod, a, r) for r in set(roots)}
  with Graph(a) as g:
    pool = serving.Pool(g, lane_words)
    bufs = {}
    todo = list(roots)
    inflight = {}
    finished = 0
    steps = 0
    while todo or inflight:
      # admit a few each step: later queries join searches already running
      for _ in range(5):
        if not todo:
          break
        lv = torch.empty(a.n, dtype=torch.int32, device="cuda")
        pa = torch.empty(a.n, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        lane = pool.admit(todo[0], lv, pa)
        if lane is None:
          break
        inflight[lane] = (todo.pop(0), lv, pa)
      for lane in pool.step(max_rounds=1, stop_on_finish=False):
        r, lv, pa = inflight.pop(lane)
        wl, wp = want[r]
        assert np.array_equal(lv.cpu().numpy(), wl), (r, lane)
        assert np.array_equal(pa.cpu().numpy(), wp), (r, lane)
        pool.release(lane)
        finished += 1
      steps += 1
      assert steps < 10000
    assert finished == len(roots)
    pool.close()


@pytest.mark.gpu
def test_pool_directed_and_deep(built_lib, oracle_mod):
  import torch
  from ceregraphs_gb300.engine import Graph
  for a, roots in ((generators.er_directed(12, 6, 9), [0, 3, 4000, 77, 1024]),
                   (generators.grid2d(40), [0, 39, 820, 1599])):
    with Graph(a) as g:
      pool = serving.Pool(g, 1)
      outs = {}

      def collect(done):
        for lane in done:
          r, lv, pa = outs.pop(lane)
          wl, wp = _alone(oracle_mod, a, r)
          assert np.array_equal(lv.cpu().numpy(), wl) and np.array_equal(pa.cpu().numpy(), wp)
          pool.release(lane)

      for r in roots:
        lv = torch.empty(a.n, dtype=torch.int32, device="cuda")
        pa = torch.empty(a.n, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        outs[pool.admit(r, lv, pa)] = (r, lv, pa)
        collect(pool.step(max_rounds=3, stop_on_finish=False))   # staggered starts
      for _ in range(100000):
        if not outs:
          break
        collect(pool.step(max_rounds=0, stop_on_finish=True))
      assert not outs
      pool.close()


@pytest.mark.gpu
@pytest.mark.parametrize("solo_max,batch_min", [(0, None), (1, None), (1, 4)])
def test_server_mix_equals_alone_under_hbm_budget(built_lib, solo_max, batch_min):
  """Queries served in the pool's mix (solo_max 0: every query through lanes;
  1: a lone query on an idle graph runs per-root; batch_min 4: an idle pool's
  backlog of 4 or more runs as one batched search) equal their searches alone."""
  import torch
  from ceregraphs_gb300.engine import Graph
  arrays = {"rmat13": generators.rmat(13, 16, 2), "rmat15": generators.rmat(15, 8, 3)}
  graphs = {k: Graph(a) for k, a in arrays.items()}
  roots = {k: graph500.pick_sources(a, 500, 5) for k, a in arrays.items()}
  arrivals = serving.poisson_arrivals(20000.0, 300, roots, seed=6)
  alone = {}
  for k, g in graphs.items():
    for r in {r for _, gg, r in arrivals if gg == k}:
      lv, pa, _ = g.bfs(r)
      alone[(k, r)] = (lv, pa)
  checked = []
  peak = [0]

  def on_done(q):
    lv = q.levels.cpu().numpy()
    pa = q.parents.cpu().numpy()
    wl, wp = alone[(q.graph, q.root)]
    checked.append(np.array_equal(lv, wl) and np.array_equal(pa, wp))

  budget = 40 * 8 * max(a.n for a in arrays.values())
  srv = serving.Server(graphs, lane_words=1, hbm_budget_bytes=budget, on_done=on_done,
                       solo_max=solo_max, batch_min=batch_min)
  orig = srv._buffers

  def tracked(name):
    peak[0] = max(peak[0], srv.in_use + srv._bytes(name))
    return orig(name)
  srv._buffers = tracked
  rep = srv.run(arrivals, realtime=True)
  srv.close()
  assert len(rep.queries) == 300 and all(checked) and len(checked) == 300
  assert (srv.batched > 0) == (batch_min is not None)
  assert srv.in_use == 0 and peak[0] <= budget + 8 * max(a.n for a in arrays.values())
  s = rep.summary()
  assert s["p99_ms"] >= s["p50_ms"] > 0
  base = serving.serial_baseline(graphs, arrivals, realtime=False)
  assert len(base.queries) == 300
  for g in graphs.values():
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("batch_min", [1, 4, 1000])
def test_batch_server_equals_alone(built_lib, batch_min):
  """Dynamic batching (batched launches for busy graphs, per-root searches for
  light queues): every query's result equals the same search run alone."""
  from ceregraphs_gb300.engine import Graph
  arrays = {"rmat13": generators.rmat(13, 16, 2), "grid": generators.grid2d(60)}
  graphs = {k: Graph(a) for k, a in arrays.items()}
  roots = {k: graph500.pick_sources(a, 300, 5) for k, a in arrays.items()}
  arrivals = serving.poisson_arrivals(50000.0, 400, roots, seed=6)
  alone = {}
  for k, g in graphs.items():
    for r in {r for _, gg, r in arrivals if gg == k}:
      lv, pa, _ = g.bfs(r)
      alone[(k, r)] = (lv, pa)
  checked = []

  def on_done(q):
    wl, wp = alone[(q.graph, q.root)]
    checked.append(np.array_equal(q.levels.cpu().numpy(), wl) and
                   np.array_equal(q.parents.cpu().numpy(), wp))

  budget = 100 * 8 * max(a.n for a in arrays.values())
  srv = serving.BatchServer(graphs, lane_words=1, hbm_budget_bytes=budget, batch_min=batch_min,
                            on_done=on_done)
  rep = srv.run(arrivals, realtime=True)
  assert len(rep.queries) == 400 and len(checked) == 400 and all(checked)
  assert srv.in_use == 0
  if batch_min == 1000:
    assert srv.launches["batched"] == 0
  s = rep.summary()
  assert s["p99_ms"] >= s["p50_ms"] > 0
  for g in graphs.values():
    g.close()


def test_budget_below_one_query_is_refused():
  """A graph whose single query does not fit the HBM budget would never be
  served: both servers refuse such a budget up front."""
  import types
  from ceregraphs_gb300 import serving
  graphs = {"small": types.SimpleNamespace(n=1000), "big": types.SimpleNamespace(n=10 ** 6)}
  serving.check_budget(graphs, None)
  serving.check_budget(graphs, 8 * 10 ** 6)
  with pytest.raises(ValueError, match="big"):
    serving.check_budget(graphs, 8 * 10 ** 6 - 1)
  with pytest.raises(ValueError):
    serving.BatchServer(graphs, hbm_budget_bytes=100)
  with pytest.raises(ValueError):
    serving.Server(graphs, hbm_budget_bytes=100)


@pytest.mark.gpu
def test_time_limit_stops_admission_and_counts_the_rest(built_lib):
  """Every mode stops taking queries once its time limit has passed: the
  queries it served plus those it reports unserved are all the arrivals, and
  those it served are complete."""
  from ceregraphs_gb300.engine import Graph
  a = generators.rmat(14, 16, 3)
  graphs = {"rmat14": Graph(a)}
  roots = {"rmat14": graph500.pick_sources(a, 200, 5)}
  arrivals = serving.poisson_arrivals(20000.0, 2000, roots, seed=6)
  runs = [serving.BatchServer(graphs, batch_min=4).run(arrivals, time_limit=0.02),
          serving.serial_baseline(graphs, arrivals, time_limit=0.02)]
  srv = serving.Server(graphs)
  runs.append(srv.run(arrivals, time_limit=0.02))
  srv.close()
  for rep in runs:
    s = rep.summary()
    assert s["queries"] + s["unserved"] == len(arrivals)
    assert s["unserved"] > 0
    assert all(q.t_done >= q.t_arrival for q in rep.queries)
  for g in graphs.values():
    g.close()


class _FakeGraph:
  """Host stand-in for engine.Graph: a search fills its outputs with its root."""

  def __init__(self, n):
    self.n = n
    self.handle = None

  def set_options(self, **kw):
    pass

  def bfs_device(self, root, lv, pa):
    lv.fill_(root)
    pa.fill_(root)

  def msbfs_device(self, roots, lv, pa):
    for i, r in enumerate(roots):
      lv[i].fill_(r)
      pa[i].fill_(r)

  def last_stats(self):
    return {"status": 0}


class _FakePool:
  """Host stand-in for serving.Pool: a lane's search ends two steps after its
  admission and then fills its outputs with its root."""

  def __init__(self, graph, lane_words=1):
    self.lanes = 64 * int(lane_words)
    self.live = {}
    self.admitted = 0

  def admit(self, root, lv, pa):
    free = [l for l in range(self.lanes) if l not in self.live]
    if not free:
      return None
    self.live[free[0]] = [root, lv, pa, 2]
    self.admitted += 1
    return free[0]

  def step(self, max_rounds=0, stop_on_finish=True):
    done = []
    for lane, rec in self.live.items():
      rec[3] -= 1
      if rec[3] == 0:
        rec[1].fill_(rec[0])
        rec[2].fill_(rec[0])
        done.append(lane)
    return done

  def release(self, lane):
    del self.live[lane]

  def close(self):
    pass


@pytest.mark.parametrize("count,solo_max,batch_min,expect", [
    (1, 1, 4, "solo"), (10, 1, 4, "batched"), (3, 0, 4, "pool"), (70, 0, None, "pool")])
def test_server_rules_on_the_host(monkeypatch, count, solo_max, batch_min, expect):
  """The continuous server's admission rules with host stand-ins for the
  pools and graphs (no GPU): a lone query on an idle graph runs per-root, a
  backlog of batch_min or more runs as one batched search once the pool is
  idle, a shorter queue joins the pool's lanes (more queries than lanes wait
  for lanes to free up); every query ends with its own root's outputs."""
  import types

  import torch
  monkeypatch.setattr(serving, "Pool", _FakePool)
  graphs = {"g": _FakeGraph(16)}
  seen = {}

  def on_done(q):
    seen[q.qid] = (int(q.levels[0]), int(q.parents[-1]), q.root)

  srv = serving.Server(graphs, on_done=on_done, solo_max=solo_max, batch_min=batch_min)
  srv.torch = types.SimpleNamespace(
      empty=lambda shape, dtype=None, device=None: torch.empty(shape, dtype=dtype),
      int32=torch.int32, cuda=types.SimpleNamespace(synchronize=lambda: None))
  monkeypatch.setattr(torch.cuda, "synchronize", lambda: None)
  arrivals = [(0.0, "g", 100 + i) for i in range(count)]
  rep = srv.run(arrivals, realtime=False)
  assert len(rep.queries) == count and srv.in_use == 0
  assert all(lv == pa == root for lv, pa, root in seen.values()) and len(seen) == count
  pool_admitted = srv.pools["g"].admitted
  assert (srv.solo, srv.batched, pool_admitted) == {
      "solo": (count, 0, 0), "batched": (0, count, 0), "pool": (0, 0, count)}[expect]
