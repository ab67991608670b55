"""Graph500-style BFS benchmark on one GB300 (or N replicas).

Workload (default): RMAT scale 23, edgefactor 16, A/B/C/D = .57/.19/.19/.05,
seed 2, symmetrised and deduplicated (the reference generator's recipe, drawn
on the GPU bit for bit); 64 roots drawn with the Graph500 rule (seed 3).  A
step = one direction-optimizing search per root.  Metric: harmonic-mean GTEPS
over the roots, m counted with the reference's undirected-dedup rule
(bfs_timing.py:379-398), identical in both arms.

* value: each search timed with CUDA events on the handle's stream, outputs
  (levels + parents) left in HBM.
* e2e: the same searches through the C ABI call cg_bfs with page-locked host
  buffers: launch + every round + parent array in host memory (the Graph500
  Kernel-2 rule, run_graph500.py:325-358), timed on the host clock.
* batched: the same roots as 64 bit lanes of one batched search replayed as a
  CUDA graph, compared with the per-root loop (GTEPS = sum of m / batch time).
* --impl reference: the reference's own host BFS (scipy breadth_first_order
  on A^T, run_graph500.py:383-395), one search at a time on one core.

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "per-root BFS GTEPS, harmonic mean over the Graph500 roots"

# DRAM bytes (read + write) per launch of bfs_persistent measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum, mean over the timed step's
# launches) for (scale, edgefactor, seed, root seed); roofline.traffic.
NCU_TRAFFIC_BYTES = {(21, 16, 0, 1): 80.5e6, (23, 16, 2, 3): 541.0e6}
FALLBACK_HBM_GBS = 6800.0


def parse():
  ap = argparse.ArgumentParser()
  ap.add_argument("--gpus", type=int, default=1)
  ap.add_argument("--steps", type=int, default=5)
  ap.add_argument("--warmup", type=int, default=3)
  ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
  ap.add_argument("--scale", type=int, default=23)
  ap.add_argument("--edgefactor", type=int, default=16)
  ap.add_argument("--seed", type=int, default=2)
  ap.add_argument("--roots", type=int, default=64)
  ap.add_argument("--root-seed", type=int, default=3)
  ap.add_argument("--direction", default="auto", choices=["auto", "topdown", "bottomup", "tau"])
  ap.add_argument("--cpu-seconds", type=float, default=15.0,
                  help="bound on the CPU-baseline sample")
  ap.add_argument("--no-cpu-baseline", action="store_true")
  ap.add_argument("--no-batched", action="store_true",
                  help="skip the multi-source (bit-lane) measurement")
  ap.add_argument("--no-reorder", action="store_true",
                  help="skip the per-root searches on the degree-ordered copy")
  ap.add_argument("--workload", default="graph500", choices=["graph500", "uneven", "serving"],
                  help="graph500: per-root + batched on one R-MAT graph (default); uneven: "
                       "256 roots in 128-lane batches over R-MAT s22 e32, directed ER 2^22 "
                       "and the 4096^2 grid, autotuned; serving: Poisson query sweep over "
                       "resident R-MAT s20/s22/s24/s26")
  ap.add_argument("--serving-scales", default="20,22,24,26")
  ap.add_argument("--serving-rates", default="100,1000,10000,100000")
  ap.add_argument("--serving-seconds", type=float, default=2.0,
                  help="arrival window per rate (each mode also stops admitting after "
                       "2 * window + 1 s)")
  return ap.parse_args()


def dist_env():
  rank = int(os.environ.get("RANK", "0"))
  world = int(os.environ.get("WORLD_SIZE", "1"))
  local = int(os.environ.get("LOCAL_RANK", "0"))
  return rank, world, local


def peaks():
  path = os.path.join(HERE, "MEASURED_PEAKS.json")
  try:
    with open(path, encoding="utf-8") as f:
      d = json.load(f)
    return float(d["hbm_gbs"]), "measured"
  except Exception:
    return FALLBACK_HBM_GBS, "fallback"


def roofline(achieved_gbs, traffic, kernel, formula):
  peak, kind = peaks()
  return {"bound": "hbm", "achieved": achieved_gbs, "peak": peak, "unit": "GB/s",
          "frac": achieved_gbs / peak, "traffic": traffic, "kernel": kernel,
          "peak_source": ("of measured (MEASURED_PEAKS.json hbm_gbs)" if kind == "measured"
                          else "of fallback 6.8 TB/s"),
          "algorithmic_bytes": formula}


class ClockSampler:
  """nvidia-smi clock/throttle samples during the timed region (read only)."""

  FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
            "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
            "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

  def __init__(self, gpu_index):
    self.gpu = gpu_index
    self.proc = None

  def start(self):
    try:
      self.proc = subprocess.Popen(
          ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
           "--format=csv,noheader,nounits", "-lms", "200"],
          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except Exception:
      self.proc = None
    return self

  def stop(self):
    if self.proc is None:
      return None
    self.proc.terminate()
    try:
      out, _ = self.proc.communicate(timeout=5)
    except Exception:
      self.proc.kill()
      out, _ = self.proc.communicate()
    self.proc = None
    sm, smax, reasons = [], 0.0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in out.strip().splitlines():
      parts = [p.strip() for p in line.split(",")]
      if len(parts) < 9:
        continue
      try:
        sm.append(float(parts[1]))
        smax = max(smax, float(parts[2]))
      except ValueError:
        continue
      for name, val in zip(names, parts[5:9]):
        if val.lower().startswith("active"):
          reasons.add(name)
    if not sm:
      return None
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
            "samples": len(sm)}


def make_graph(args):
  from ceregraphs_gb300 import generators
  t0 = time.perf_counter()
  a = generators.rmat(args.scale, args.edgefactor, args.seed)
  return a, time.perf_counter() - t0


def make_graph_device(args):
  """The same R-MAT graph drawn and built on the GPU (bit-identical to the
  host generator); returns (Graph, GraphArrays, seconds)."""
  import torch
  from ceregraphs_gb300 import generators
  torch.cuda.synchronize()
  t0 = time.perf_counter()
  g, a = generators.rmat_device(args.scale, args.edgefactor, args.seed)
  torch.cuda.synchronize()
  return g, a, time.perf_counter() - t0


def workload_config(args, n, nnz):
  """The workload, identical in both arms."""
  return {"workload": f"rmat{args.scale}-e{args.edgefactor}-seed{args.seed}, {args.roots} "
                      f"Graph500 roots (seed {args.root_seed}), one search per root",
          "scale": args.scale, "edgefactor": args.edgefactor, "n": int(n), "nnz": int(nnz),
          "roots": args.roots, "root_seed": args.root_seed,
          "l2": f"inputs larger than L2: CSR {(nnz * 4 + (n + 1) * 8) / 1e6:.0f} MB",
          "parallelism": f"replicas{args.gpus}"}


# --------------------------------------------------------------------------
# reference arm / CPU baseline: scipy breadth_first_order on A^T
# --------------------------------------------------------------------------
_REF = {}


def _ref_init(a):
  """A^T in CSR, built once outside any timing (the reference rebuilds it per
  search, run_graph500.py:384).  For a symmetric A it is A's own CSR."""
  from scipy import sparse
  A = sparse.csr_matrix((np.ones(a.nnz, dtype=np.int8), a.in_idx, a.in_off), shape=(a.n, a.n))
  _REF["At"] = A if a.symmetric else A.transpose().tocsr()


def _ref_search(root):
  from scipy.sparse.csgraph import breadth_first_order
  t0 = time.perf_counter()
  order, _ = breadth_first_order(_REF["At"], int(root), directed=True, return_predecessors=True)
  dt = time.perf_counter() - t0
  visited = np.zeros(_REF["At"].shape[0], dtype=bool)
  visited[order] = True
  return int(root), dt, visited


def cpu_reference_sample(a, roots, seconds_budget):
  """scipy BFS over roots one at a time (one core), stopping once the budget is
  spent; returns per-search (root, seconds, m)."""
  from ceregraphs_gb300.graph500 import EdgeCounter
  counter = EdgeCounter(a)
  _ref_init(a)
  out = []
  t_start = time.perf_counter()
  for r in roots:
    root, dt, visited = _ref_search(r)
    out.append((root, dt, counter.m(visited)))
    if time.perf_counter() - t_start > seconds_budget:
      break
  return out


def cpu_reference_all_cores(roots, processes):
  """One round of `processes` concurrent scipy searches (one per core, forked
  after _ref_init); returns (searches, wall seconds, per-search seconds)."""
  import multiprocessing as mp
  ctx = mp.get_context("fork")
  t0 = time.perf_counter()
  with ctx.Pool(processes) as pool:
    res = pool.map(_ref_search, roots[:processes])
  return res, time.perf_counter() - t0


def run_reference(args):
  """The reference's CPU path on this machine: scipy breadth_first_order on A^T,
  one search per step, one core (the search is single-threaded C)."""
  rank, _, _ = dist_env()
  if rank != 0:
    return 0
  from ceregraphs_gb300.bfs_timing import harmonic_mean
  from ceregraphs_gb300.graph500 import EdgeCounter, pick_sources
  a, gen_s = make_graph(args)
  roots = pick_sources(a, args.roots, args.root_seed)
  counter = EdgeCounter(a)
  _ref_init(a)
  for s in range(args.warmup):
    _ref_search(roots[s % len(roots)])
  samples = []
  t0 = time.perf_counter()
  for s in range(args.steps):
    root, dt, visited = _ref_search(roots[s % len(roots)])
    samples.append((root, dt, counter.m(visited)))
  wall = time.perf_counter() - t0
  value = harmonic_mean([m / dt / 1e9 for (_, dt, m) in samples])
  cores = os.cpu_count() or 1
  # all host cores at once (contended memory): aggregate throughput only
  par, par_wall = cpu_reference_all_cores(roots, min(cores, len(roots)))
  par_m = sum(counter.m(v) for (_, _, v) in par)
  line = {"metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": args.gpus,
          "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
          "data": "synthetic (R-MAT, the reference generator's recipe, bit-identical)",
          "impl": "reference", "config": workload_config(args, a.n, a.nnz),
          "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": 1, "kind": "reference",
                           "sample": f"{len(samples)} searches, one per step, one at a time: "
                                     "scipy.sparse.csgraph.breadth_first_order on A^T, the call "
                                     "of run_graph500.py:383-395 (single-threaded C); roots "
                                     "in Graph500 order, cycled"},
          "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0,
                  "d2h_bytes_per_step": 0},
          "construction_s": round(gen_s, 2),
          "all_cores": {"processes": len(par), "host_cores": cores,
                        "aggregate_gteps": par_m / par_wall / 1e9,
                        "per_search_hm_gteps_contended": harmonic_mean(
                            [counter.m(v) / dt / 1e9 for (_, dt, v) in par])}}
  print(json.dumps(line), flush=True)
  return 0


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------
def run_ours(args):
  import torch
  rank, world, local = dist_env()
  torch.cuda.set_device(local)
  dist = None
  if world > 1:
    import torch.distributed as dist
    dist.init_process_group("nccl", device_id=torch.device("cuda", local))

  from ceregraphs_gb300 import _lib, replicas
  from ceregraphs_gb300.bfs_timing import harmonic_mean
  from ceregraphs_gb300.engine import PinnedBuffer
  from ceregraphs_gb300.graph500 import EdgeCounter, pick_sources

  g, a, gen_s = make_graph_device(args)
  roots_all = pick_sources(a, args.roots, args.root_seed)
  # replicas: each GPU holds the whole graph and takes a disjoint share of roots
  roots = replicas.shard(roots_all, rank, world)
  dirmap = {"auto": _lib.CG_DIR_AUTO, "topdown": _lib.CG_DIR_TOPDOWN,
            "bottomup": _lib.CG_DIR_BOTTOMUP, "tau": _lib.CG_DIR_TAU}
  g.set_options(direction=dirmap[args.direction])

  n = a.n
  k = len(roots)
  d_lv = torch.empty((k, n), dtype=torch.int32, device="cuda")
  d_pa = torch.empty((k, n), dtype=torch.int32, device="cuda")
  torch.cuda.synchronize()
  stream = torch.cuda.ExternalStream(g.stream)

  # m per root (device count; checked against the host rule on smaller graphs)
  for i, r in enumerate(roots):
    g.bfs_device(r, d_lv[i], d_pa[i])
  st = g.last_stats()
  if st["status"] != 0:
    raise RuntimeError(f"search failed: {st}")
  m = g.count_edges(d_lv, k)
  if a.nnz <= 100_000_000:
    counter = EdgeCounter(a)
    lv_host = d_lv.cpu().numpy()
    m_host = np.array([counter.m(lv_host[i] >= 0) for i in range(k)])
    assert np.array_equal(m, m_host), "device and host edge counts differ"
  deg_t = torch.from_numpy(np.diff(a.out_lists()[0])).cuda()
  nnz_vis = np.array([int(((d_lv[i] >= 0).to(torch.int64) * deg_t).sum()) for i in range(k)])
  alg_bytes = 4 * nnz_vis + 8 * (n + 1) + 8 * n   # B_1 per search
  del deg_t

  def one_step(ev):
    for i, r in enumerate(roots):
      ev[i][0].record(stream)
      g.bfs_device(r, d_lv[i], d_pa[i])
      ev[i][1].record(stream)

  events = [[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
            for _ in range(k)]
  for _ in range(max(args.warmup, 3)):
    one_step(events)
  torch.cuda.synchronize()

  sampler = ClockSampler(local).start()
  time.sleep(0.3)
  if dist is not None:
    dist.barrier()
  torch.cuda.synchronize()
  per_root_ms = np.zeros(k)
  t_step0 = time.perf_counter()
  for _ in range(args.steps):
    one_step(events)
    torch.cuda.synchronize()
    per_root_ms += np.array([events[i][0].elapsed_time(events[i][1]) for i in range(k)])
  torch.cuda.synchronize()
  if dist is not None:
    dist.barrier()
  wall = time.perf_counter() - t_step0
  per_root_ms /= args.steps
  st = g.last_stats()
  if st["status"] != 0:
    raise RuntimeError(f"search failed: {st}")

  # e2e: C ABI with host (page-locked) parent buffers, host clock per search;
  # each root's time is the median over the steps (a host-side hiccup in one
  # step would otherwise dominate the harmonic mean)
  pin = PinnedBuffer(n)
  e2e_samples = np.zeros((args.steps, k))
  for r in roots[:4]:  # warm
    g.bfs(r, None, pin.array, want_levels=False)
  for step in range(args.steps):
    for i, r in enumerate(roots):
      t0 = time.perf_counter()
      _, _, st2 = g.bfs(r, None, pin.array, want_levels=False)
      e2e_samples[step, i] = time.perf_counter() - t0
      if st2["status"] != 0:
        raise RuntimeError(f"search failed: {st2}")
  e2e_s = np.median(e2e_samples, axis=0)
  pin.free()

  # degree-aware reordering (cg_graph_reorder): the same per-root searches on a
  # copy numbered by descending in-degree, outputs checked equal to the above
  reordered = None
  if not args.no_reorder:
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gr = g.reorder()
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    gr.set_options(direction=dirmap[args.direction])
    stream_r = torch.cuda.ExternalStream(gr.stream)
    r_lv = torch.empty(n, dtype=torch.int32, device="cuda")
    r_pa = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    same_r = True
    for i, r in enumerate(roots):
      gr.bfs_device(r, r_lv, r_pa)
      gr.last_stats()
      same_r = same_r and bool(torch.equal(r_lv, d_lv[i]) and torch.equal(r_pa, d_pa[i]))
    ev_r = [[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
            for _ in range(k)]
    r_ms = np.zeros(k)
    for step in range(max(args.warmup, 3) + args.steps):
      for i, r in enumerate(roots):
        ev_r[i][0].record(stream_r)
        gr.bfs_device(r, r_lv, r_pa)
        ev_r[i][1].record(stream_r)
      torch.cuda.synchronize()
      if step >= max(args.warmup, 3):
        r_ms += np.array([ev_r[i][0].elapsed_time(ev_r[i][1]) for i in range(k)])
    r_ms /= args.steps
    str_ = gr.last_stats()
    gr.close()
    del r_lv, r_pa
    r_gteps = m / (r_ms * 1e-3) / 1e9
    reordered = {"order": "descending in-degree (cg_graph_reorder, CG_ORDER_DEGREE)",
                 "hm_gteps": harmonic_mean(r_gteps), "ms_median": float(np.median(r_ms)),
                 "vs_original_order": harmonic_mean(r_gteps) / harmonic_mean(
                     m / (per_root_ms * 1e-3) / 1e9),
                 "bit_exact_vs_original_order": same_r, "build_s": round(build_s, 3),
                 "status": str_["status"]}

  # batched: the same roots as bit lanes (64 or 128 per pass), one CUDA graph
  # per step; every lane is checked against the per-root outputs
  batched = None
  if not args.no_batched:
    ref_lv, ref_pa = d_lv.clone(), d_pa.clone()
    lane_words = 1 if k <= 64 else 2
    g.set_options(lane_words=lane_words)
    g.msbfs_device(roots, d_lv, d_pa)
    g.last_stats()
    exe = g.capture(lambda: g.msbfs_device(roots, d_lv, d_pa))
    for _ in range(max(args.warmup, 3)):
      exe.launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
      exe.launch()
    e1.record(stream)
    torch.cuda.synchronize()
    batch_ms = e0.elapsed_time(e1) / args.steps
    stb = g.last_stats()
    same = bool(torch.equal(ref_lv, d_lv) and torch.equal(ref_pa, d_pa))
    exe.close()
    del ref_lv, ref_pa
    pin_lv, pin_pa = PinnedBuffer((k, n)), PinnedBuffer((k, n))
    g.msbfs(roots, pin_lv.array, pin_pa.array)
    t0 = time.perf_counter()
    for _ in range(args.steps):
      g.msbfs(roots, pin_lv.array, pin_pa.array)
    batch_e2e_s = (time.perf_counter() - t0) / args.steps
    pin_lv.free()
    pin_pa.free()
    batched_gteps = float(m.sum() / (batch_ms * 1e-3) / 1e9)
    hm_per_root = harmonic_mean(m / (per_root_ms * 1e-3) / 1e9)
    lanes = 64 * lane_words
    bk = 4 * a.nnz + 8 * (n + 1) + stb["rounds"] * 2 * n * lanes // 8 + 8 * n * k
    batched = {"gteps": batched_gteps, "ms": batch_ms,
               "vs_per_root_harmonic_mean": batched_gteps / hm_per_root,
               "e2e_gteps": float(m.sum() / batch_e2e_s / 1e9), "e2e_ms": batch_e2e_s * 1e3,
               "e2e_d2h_bytes": 2 * 4 * n * k,
               "lanes": lanes, "rounds": stb["rounds"],
               "pull_rounds": stb["pull_rounds"], "bit_exact_vs_per_root": same,
               "roofline": roofline(bk / (batch_ms * 1e-3) / 1e9, None,
                                    "msbfs_ledger + msbfs_scan + msbfs_outputs + msbfs_fixup",
                                    "B_k = 4*nnz + 8*(n+1) + rounds*2*n*lanes/8 + 8*n*k per "
                                    "batch"),
               "launch": "per 64/128 roots: the rounds (one cooperative kernel), then the "
                         "scan, output and fix-up passes, replayed as one CUDA graph"}
  clocks = sampler.stop()

  gteps_dev = m / (per_root_ms * 1e-3) / 1e9
  gteps_e2e = m / e2e_s / 1e9
  step_ms = wall / args.steps * 1e3
  m_step = float(m.sum())
  if dist is not None:
    from ceregraphs_gb300.replicas import gather
    gteps_dev = np.array(gather(list(gteps_dev)))
    gteps_e2e = np.array(gather(list(gteps_e2e)))
    t = torch.tensor([step_ms, m_step], device="cuda", dtype=torch.float64)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    step_ms, m_step = float(tmax[0].item()), float(t[1].item())
  value = harmonic_mean(gteps_dev)
  e2e_value = harmonic_mean(gteps_e2e)
  achieved = float(alg_bytes.sum() / (per_root_ms.sum() * 1e-3) / 1e9)
  traffic = NCU_TRAFFIC_BYTES.get((args.scale, args.edgefactor, args.seed, args.root_seed))
  line = {
      "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
      "warmup": max(args.warmup, 3), "ms_per_step": step_ms, "higher_is_better": True,
      "scaling": "weak", "vs_baseline": None, "dtype": "int32",
      "data": "synthetic (R-MAT, the reference generator's recipe, bit-identical)",
      "config": workload_config(args, n, a.nnz),
      "construction_s": round(gen_s, 3),
      "e2e": {"value": e2e_value, "unit": "GTEPS", "h2d_bytes_per_step": 8 * k,
              "d2h_bytes_per_step": 4 * n * k,
              "note": "cg_bfs: launch + all rounds + parents in page-locked host memory; "
                      "each root's median over the steps"},
      "gpu_launches": k * args.steps,
      "roofline": roofline(achieved, traffic, "bfs_persistent",
                           "4*nnz_visited + 8*(n+1) + 8*n per search"),
      "per_root": {"direction": args.direction, "ms_median": float(np.median(per_root_ms)),
                   "ms_min": float(per_root_ms.min()), "ms_max": float(per_root_ms.max()),
                   "gteps_min": float(gteps_dev.min()), "gteps_max": float(gteps_dev.max()),
                   "e2e_ms_median": float(np.median(e2e_s) * 1e3),
                   "rounds": st["rounds"], "pull_rounds_last": st["pull_rounds"]},
      "aggregate_gteps": m_step / (step_ms * 1e-3) / 1e9,
  }
  if batched:
    line["batched"] = batched
  if reordered:
    line["reordered"] = reordered
  if clocks:
    line["clocks"] = clocks
  if rank == 0 and not args.no_cpu_baseline:
    res = cpu_reference_sample(a, roots, args.cpu_seconds)
    g_cpu = [mm / dt / 1e9 for (_, dt, mm) in res]
    line["cpu_baseline"] = {
        "value": harmonic_mean(g_cpu), "unit": "GTEPS", "cores": 1, "kind": "reference",
        "sample": f"{len(res)} of the {k} roots, one at a time: scipy breadth_first_order on "
                  f"A^T (run_graph500.py:383-395), single-threaded, {os.cpu_count()} host "
                  "cores seen"}
  g.close()
  if rank == 0:
    print(json.dumps(line), flush=True)
  if dist is not None:
    dist.destroy_process_group()
  return 0


def run_uneven(args):
  """Three graphs of uneven depth, 256 roots each (seed 5) in batches of up to
  128 lanes, knobs chosen per graph by the autotuner.  Every lane of the first
  batch of each graph passes the device tree checks (lowest-index parents
  included); the CPU baseline's searches are checked level for level."""
  import torch
  from ceregraphs_gb300 import autotune, generators
  from ceregraphs_gb300.bfs_timing import harmonic_mean
  from ceregraphs_gb300.engine import Graph, PinnedBuffer
  from ceregraphs_gb300.graph500 import pick_sources
  torch.cuda.set_device(0)
  specs = [("rmat22-e32", lambda: generators.rmat_device(22, 32, 0)),
           ("er22-d8-directed", lambda: generators.er_directed_device(22, 8, 4)),
           ("grid4096", lambda: (lambda a: (Graph(a), a))(generators.grid2d(4096)))]
  out = {}
  tot_m = tot_s = tot_b = roof_s = 0.0
  e2e_m = e2e_s = 0.0
  launches = 0
  cpu_g = []
  cpu_note = []
  sampler = ClockSampler(0).start()
  for name, make in specs:
    t0 = time.perf_counter()
    g, a = make()
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    roots = pick_sources(a, 256, 5)
    k = len(roots)
    tune = autotune.tune(g, a, roots[:128], mode="batched",
                         space={"lane_words": [1, 2], "ms_alpha": [1.0, 4.0, 16.0],
                                "block_size": [512]}, reps=1, cache=autotune.Cache())
    lanes = 64 * g.options().lane_words
    d_lv = torch.empty((k, a.n), dtype=torch.int32, device="cuda")
    d_pa = torch.empty((k, a.n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(g.stream)
    g.msbfs_device(roots, d_lv, d_pa)
    g.last_stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
      g.msbfs_device(roots, d_lv, d_pa)
    e1.record(stream)
    torch.cuda.synchronize()
    st = g.last_stats()
    batch_ms = e0.elapsed_time(e1) / args.steps
    launches += args.steps * ((k + lanes - 1) // lanes) * 5
    m = g.count_edges(d_lv, k)
    # every lane of the first batch through the device tree checks
    first = min(k, lanes)
    val = g.validate(roots[:first], d_lv[:first], d_pa[:first])
    bad = sum(sum(v[c]["failures"] for c in v) for v in val)
    # B_k per batch: adjacency once, frontier read + written per round, outputs
    nb = (k + lanes - 1) // lanes
    bk = nb * (4 * a.nnz + 8 * (a.n + 1)) + st["rounds"] * 2 * a.n * lanes // 8 * nb + 8 * a.n * k
    # per-root sample: 8 roots, CUDA events on the handle's stream
    sample = roots[:8]
    per_ms = []
    for i, r in enumerate(sample):
      g.bfs_device(r, d_lv[i], d_pa[i])
      ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
      ev0.record(stream)
      g.bfs_device(r, d_lv[i], d_pa[i])
      ev1.record(stream)
      torch.cuda.synchronize()
      per_ms.append(ev0.elapsed_time(ev1))
    per_gteps = [float(m[i]) / (per_ms[i] * 1e-3) / 1e9 for i in range(len(sample))]
    # e2e: one batch of 64 roots through cg_msbfs into page-locked host buffers
    ke = min(64, k)
    g.set_options(lane_words=1)
    pin_lv, pin_pa = PinnedBuffer((ke, a.n)), PinnedBuffer((ke, a.n))
    g.msbfs(roots[:ke], pin_lv.array, pin_pa.array)
    t1 = time.perf_counter()
    g.msbfs(roots[:ke], pin_lv.array, pin_pa.array)
    e2e_t = time.perf_counter() - t1
    e2e_m += float(m[:ke].sum())
    e2e_s += e2e_t
    # CPU baseline: scipy on A^T, one core, two roots, levels checked
    if not args.no_cpu_baseline:
      res = cpu_reference_sample(a, roots[:2], args.cpu_seconds / 3)
      for (r, dt, mm) in res:
        cpu_g.append(mm / dt / 1e9)
      lv_ours = pin_lv.array[:len(res)]
      from scipy.sparse.csgraph import breadth_first_order
      same_lv = True
      for i, (r, _, _) in enumerate(res):
        # scipy's tree is a BFS tree: our levels equal its depths exactly when
        # the reached sets agree, the root is at 0 and every tree edge goes
        # one level down
        order, pred = breadth_first_order(_REF["At"], int(r), directed=True,
                                          return_predecessors=True)
        mine = lv_ours[i].astype(np.int64)
        reached = np.zeros(a.n, dtype=bool)
        reached[order] = True
        kids = order[1:]
        same_lv = same_lv and bool(np.array_equal(reached, mine >= 0) and mine[r] == 0 and
                                   np.array_equal(mine[kids], mine[pred[kids]] + 1))
      cpu_note.append(f"{name}: {len(res)} roots, levels equal to ours: {same_lv}")
      _REF.clear()
    pin_lv.free()
    pin_pa.free()
    out[name] = {"n": a.n, "nnz": a.nnz, "symmetric": a.symmetric, "roots": k,
                 "generation_s": round(gen_s, 2), "lanes": lanes,
                 "tuned": tune["options"], "batch_ms_all_roots": batch_ms,
                 "batched_gteps": float(m.sum()) / (batch_ms * 1e-3) / 1e9,
                 "per_root_sample_hm_gteps": harmonic_mean(per_gteps),
                 "batched_vs_per_root_sample": (float(m.sum()) / (batch_ms * 1e-3) / 1e9)
                 / harmonic_mean(per_gteps),
                 "rounds_max": st["rounds"], "device_checks_failures_first_batch": int(bad),
                 "lanes_checked": first, "B_k_GB": bk / 1e9,
                 "e2e_ms_64_roots": e2e_t * 1e3}
    tot_m += float(m.sum())
    tot_s += batch_ms * 1e-3
    if st["rounds"] <= 64:  # ledger mode: rounds sweep whole frontier planes, as B_k counts
      tot_b += bk
      roof_s += batch_ms * 1e-3
    g.close()
    del d_lv, d_pa
    torch.cuda.empty_cache()
  clocks = sampler.stop()
  line = {"metric": "batched GTEPS, 256 roots per graph in 64/128-lane batches (autotuned)",
          "value": tot_m / tot_s / 1e9, "unit": "GTEPS", "n_gpus": 1, "steps": args.steps,
          "warmup": 1, "ms_per_step": tot_s * 1e3, "higher_is_better": True, "scaling": "weak",
          "vs_baseline": None, "dtype": "int32", "data": "synthetic (R-MAT reference recipe, ER, grid)",
          "config": {"workload": "uneven-depth batching: rmat22-e32, er22-d8 directed, "
                                 "grid 4096x4096; roots seed 5",
                     "l2": "inputs larger than L2"},
          "e2e": {"value": e2e_m / e2e_s / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": 8 * 64 * 3,
                  "d2h_bytes_per_step": sum(8 * 64 * o["n"] for o in out.values()),
                  "note": "cg_msbfs, 64 roots per graph, outputs stored into page-locked host "
                          "memory by the batch's passes"},
          "gpu_launches": launches,
          "roofline": roofline(tot_b / max(roof_s, 1e-12) / 1e9, None,
                               "msbfs batch (rounds + passes)",
                               "B_k = batches*(4*nnz + 8*(n+1)) + rounds*2*n*lanes/8*batches "
                               "+ 8*n*k per graph, over the graphs searched in ledger mode "
                               "(<= 64 rounds); the grid's 7850-round batches run in the "
                               "direct kernel, which touches only frontier vertices a round"),
          "graphs": out}
  if clocks:
    line["clocks"] = clocks
  if cpu_g:
    line["cpu_baseline"] = {"value": harmonic_mean(cpu_g), "unit": "GTEPS", "cores": 1,
                            "kind": "reference",
                            "sample": "scipy breadth_first_order on A^T (run_graph500.py:383-395), "
                                      "single-threaded; " + "; ".join(cpu_note)}
  print(json.dumps(line), flush=True)
  return 0


def run_serving(args):
  """Serving over resident R-MAT graphs with Poisson arrivals: dynamic
  batching, continuous batching (lanes joining searches in flight) and the
  serial per-query loop, each run for the arrival window plus a bounded drain
  (time_limit), so overloaded modes report their sustained throughput."""
  import torch
  from ceregraphs_gb300 import generators, serving
  torch.cuda.set_device(0)
  graphs, roots, info = {}, {}, {}
  for sc in [int(x) for x in args.serving_scales.split(",")]:
    t0 = time.perf_counter()
    g, _ = generators.rmat_device(sc, 16, 0, export=False)
    off = g.export_offsets()
    torch.cuda.synchronize()
    cand = np.nonzero(np.diff(off) > 0)[0]
    name = f"rmat{sc}"
    graphs[name] = g
    roots[name] = cand
    info[name] = {"n": g.n, "nnz": g.nnz, "build_s": round(time.perf_counter() - t0, 2)}
    del off
  torch.cuda.empty_cache()
  budget = 96 << 30
  limit = 2.0 * args.serving_seconds + 1.0
  rows = []
  best = 0.0
  sampler = ClockSampler(0).start()
  t_all = time.perf_counter()
  for rate in [float(x) for x in args.serving_rates.split(",")]:
    count = int(max(100, rate * args.serving_seconds))
    arrivals = serving.poisson_arrivals(rate, count, roots, seed=6)
    bsrv = serving.BatchServer(graphs, lane_words=1, hbm_budget_bytes=budget, batch_min=4)
    dyn = bsrv.run(arrivals, realtime=True, time_limit=limit).summary()
    dyn["launches"] = dict(bsrv.launches)
    srv = serving.Server(graphs, lane_words=1, hbm_budget_bytes=budget, batch_min=8)
    pool = srv.run(arrivals, realtime=True, time_limit=limit).summary()
    pool["per_root_solo"] = srv.solo
    pool["batched_backlog"] = srv.batched
    srv.close()
    base = serving.serial_baseline(graphs, arrivals, realtime=True, time_limit=limit).summary()
    rows.append({"rate_qps": rate, "arrivals": count, "window_s": args.serving_seconds,
                 "time_limit_s": limit, "batched": dyn, "pool": pool, "serial": base})
    best = max(best, dyn["throughput_qps"], pool["throughput_qps"])
  wall = time.perf_counter() - t_all
  clocks = sampler.stop()
  line = {"metric": "queries/s and p50/p99 query ms, batched serving vs serial per-query BFS",
          "value": best, "unit": "queries/s", "n_gpus": 1, "steps": len(rows), "warmup": 0,
          "ms_per_step": wall / max(1, len(rows)) * 1e3,
          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
          "data": "synthetic (R-MAT reference recipe), Poisson arrivals seed 6",
          "config": {"workload": "serving over resident rmat " + args.serving_scales +
                                 ", edgefactor 16, uniform non-isolated roots",
                     "graphs": info, "hbm_budget_bytes": budget, "lanes_per_graph": 64,
                     "modes": {"batched": "dynamic batching: a graph's waiting queries start "
                                          "together (batched launch when >= 4, else "
                                          "per-root), outputs written after the rounds",
                               "pool": "continuous batching: queries join searches in "
                                       "flight as bit lanes of a resumable launch; a query "
                                       "finding its graph idle and alone runs per-root; an "
                                       "idle graph's backlog of >= 8 runs as one batched "
                                       "search",
                               "serial": "one per-root search at a time, FIFO"}},
          "e2e": {"value": best, "unit": "queries/s", "h2d_bytes_per_step": 8,
                  "d2h_bytes_per_step": 16,
                  "note": "host clock from each query's arrival to the host seeing it done; the "
                          "root goes in, the completion comes back, outputs stay in HBM for "
                          "the caller"},
          "rates": rows}
  if clocks:
    line["clocks"] = clocks
  print(json.dumps(line), flush=True)
  for g in graphs.values():
    g.close()
  return 0


def main():
  args = parse()
  if args.impl == "reference":
    return run_reference(args)
  if args.workload == "uneven":
    return run_uneven(args)
  if args.workload == "serving":
    return run_serving(args)
  return run_ours(args)


if __name__ == "__main__":
  sys.exit(main())
