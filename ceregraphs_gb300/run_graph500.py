"""Graph500 driver: the command-line counterpart of bfs/scripts/run_graph500.py.

    python -m ceregraphs_gb300.run_graph500 --infile_mtx graph.mtx [--num-searches 64]
    python -m ceregraphs_gb300.run_graph500 --rmat 21 16 0 --mode batched

Same flow and options as the reference's driver (run_graph500.py:64-101,
160-505), with the wafer-only options (PE grid, fabric, compiler) gone:

* Kernel 1 -- the graph file parsed by the native loader and built on the
  device (or an R-MAT graph of the reference generator drawn on the device),
  timed once and kept out of every search's time;
* roots -- ``--sources`` or the Graph500 rule with ``--seed``
  (run_graph500.py:106-127);
* Kernel 2 -- per root, launch + every round + levels and parents in host
  memory, on the host clock (the spec's rule, run_graph500.py:321-380); or,
  with ``--mode batched``, 64/128 roots per launch as bit lanes, timed with
  CUDA events, every root of a batch charged the batch time;
* correctness -- on by default as in the reference (``--nocorrectness`` skips
  it), here the Graph500 tree checks run on the device (cg_validate_device)
  instead of a host scipy search per root;
* per-search and summary CSVs, appended with the reference's header check.
"""
from __future__ import annotations

import argparse
import csv
import os
import sys
import time
from datetime import datetime, timezone

import numpy as np

CHECK_NAMES = ("root", "tree", "edges", "span", "tree_edge", "lowest")


def parse_args(argv=None):
  ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
  src = ap.add_mutually_exclusive_group(required=True)
  src.add_argument("--infile_mtx", help="graph file: Matrix Market or SNAP edge list (.gz ok)")
  src.add_argument("--rmat", nargs=3, type=int, metavar=("SCALE", "EDGEFACTOR", "SEED"),
                   help="R-MAT graph of datasets/gen_rmat.py, drawn on the device")
  ap.add_argument("--num-searches", type=int, default=64)
  ap.add_argument("--seed", type=int, default=0, help="seed of the root sample")
  ap.add_argument("--sources", default=None, help="comma-separated roots (overrides the sample)")
  ap.add_argument("--max-rounds", type=int, default=15,
                  help="rounds whose timing goes into the per-search rows (at most 64)")
  ap.add_argument("--nocorrectness", action="store_true", help="skip the device tree checks")
  ap.add_argument("--csv", default=None, help="append per-search rows here")
  ap.add_argument("--summary-csv", default=None, help="append the summary row here")
  ap.add_argument("--mode", choices=["per-root", "batched"], default="per-root")
  ap.add_argument("--lanes", type=int, choices=[64, 128], default=64,
                  help="roots per batched launch")
  ap.add_argument("--direction", choices=["auto", "topdown", "bottomup", "tau"], default="auto")
  ap.add_argument("--parent-rule", choices=["lowest", "fifo"], default="lowest",
                  help="lowest-index parents, or those of scipy's breadth_first_order "
                       "(the reference's host check; a pass after each search)")
  ap.add_argument("--warmup", type=int, default=1,
                  help="untimed passes over the roots before the recorded one")
  ap.add_argument("--quiet", action="store_true", help="no per-search lines")
  return ap.parse_args(argv)


def pick_roots(args, arrays):
  from .graph500 import pick_sources
  if args.sources is not None:
    roots = [int(s) for s in args.sources.split(",")]
    for r in roots:
      if not 0 <= r < arrays.n:
        raise SystemExit(f"--sources entry {r} out of range [0, {arrays.n})")
    return roots
  roots = pick_sources(arrays, args.num_searches, args.seed)
  if len(roots) < args.num_searches:
    print(f"[[ NOTE: only {len(roots)} vertices have degree >= 1 (excluding self-loops); "
          f"using all of them ]]")
  return roots


def kernel1(args):
  """Returns (Graph, GraphArrays, seconds, name)."""
  import torch
  from . import generators, loader
  torch.cuda.synchronize()
  t0 = time.perf_counter()
  if args.rmat:
    s, ef, seed = args.rmat
    g, _ = generators.rmat_device(s, ef, seed, export=False)
    name = f"rmat_s{s}_e{ef}_seed{seed}"
  else:
    g = loader.load_graph(args.infile_mtx)
    name = os.path.basename(args.infile_mtx)
  torch.cuda.synchronize()
  secs = time.perf_counter() - t0
  return g, g.export(), secs, name


def append_csv(path, rows):
  """Append rows, refusing a file whose header differs (run_graph500.py:470-482)."""
  if not rows:
    return
  os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
  keys = list(rows[0].keys())
  write_header = not os.path.exists(path)
  if not write_header:
    with open(path, newline="", encoding="utf-8") as f:
      existing = next(csv.reader(f), [])
    if existing != keys:
      raise SystemExit(f"{path}'s header does not match this run's columns; "
                       "pass another path or move the old file")
  with open(path, "a", newline="", encoding="utf-8") as f:
    w = csv.DictWriter(f, fieldnames=keys)
    if write_header:
      w.writeheader()
    w.writerows(rows)


def run(args):
  import torch
  from . import _lib
  from .bfs_timing import gteps, harmonic_mean
  from .engine import PinnedBuffer
  from .graph500 import EdgeCounter

  g, a, construction_s, name = kernel1(args)
  n, nnz = a.n, a.nnz
  print(f"Kernel 1: {name} n={n} nnz={nnz} symmetric={a.symmetric} "
        f"construction={construction_s:.3f} s (not part of any search's time)")
  roots = pick_roots(args, a)
  print(f"selected {len(roots)} search roots (seed={args.seed})")
  dirmap = {"auto": _lib.CG_DIR_AUTO, "topdown": _lib.CG_DIR_TOPDOWN,
            "bottomup": _lib.CG_DIR_BOTTOMUP, "tau": _lib.CG_DIR_TAU}
  g.set_options(direction=dirmap[args.direction],
                lane_words=1 if args.lanes == 64 else 2,
                parent_rule=_lib.CG_PARENT_FIFO if args.parent_rule == "fifo"
                else _lib.CG_PARENT_LOWEST)
  # FIFO parents are valid Graph500 trees but not the lowest-index ones
  judged = [c for c in CHECK_NAMES if not (c == "lowest" and args.parent_rule == "fifo")]
  counter = EdgeCounter(a)
  rows = []
  now = datetime.now(timezone.utc).isoformat
  base = {"infile_mtx": name, "n": n, "nnz": nnz, "matrix_symmetric": a.symmetric,
          "mode": args.mode, "parent_rule": args.parent_rule}

  def check(batch_roots, d_lv, d_pa):
    """(ok per root, check tallies per root), or Nones with --nocorrectness."""
    if args.nocorrectness:
      return [None] * len(batch_roots), [None] * len(batch_roots)
    res = g.validate(batch_roots, d_lv, d_pa)
    return [all(r[c]["failures"] == 0 for c in judged) for r in res], res

  if args.mode == "per-root":
    pin_lv, pin_pa = PinnedBuffer(n), PinnedBuffer(n)
    d_lv = torch.empty(n, dtype=torch.int32, device="cuda")
    d_pa = torch.empty_like(d_lv)
    for _ in range(args.warmup):
      for r in roots:
        g.bfs(r, pin_lv.array, pin_pa.array)
    for i, r in enumerate(roots):
      t0 = time.perf_counter()
      _, _, st = g.bfs(r, pin_lv.array, pin_pa.array)
      secs = time.perf_counter() - t0
      visited = pin_pa.array >= 0
      m = counter.m(visited)
      ok, detail = None, None
      if not args.nocorrectness:
        d_lv.copy_(torch.from_numpy(pin_lv.array))
        d_pa.copy_(torch.from_numpy(pin_pa.array))
        oks, dets = check([r], d_lv, d_pa)
        ok, detail = oks[0], dets[0]
      rows.append(search_row(now(), base, i, i, r, st, args.max_rounds, ok, int(visited.sum()),
                             m, counter.convention, secs, detail))
  else:
    lanes = args.lanes
    k_all = len(roots)
    stream = torch.cuda.ExternalStream(g.stream)
    for b0 in range(0, k_all, lanes):
      batch = roots[b0:b0 + lanes]
      k = len(batch)
      d_lv = torch.empty((k, n), dtype=torch.int32, device="cuda")
      d_pa = torch.empty_like(d_lv)
      torch.cuda.synchronize()
      for _ in range(args.warmup):
        g.msbfs_device(batch, d_lv, d_pa)
      e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
      e0.record(stream)
      g.msbfs_device(batch, d_lv, d_pa)
      e1.record(stream)
      st = g.last_stats()
      secs = e0.elapsed_time(e1) * 1e-3
      ms = g.count_edges(d_lv, k)
      visited = (d_lv >= 0).sum(dim=1).cpu().numpy()
      oks, dets = check(batch, d_lv, d_pa)
      for j, r in enumerate(batch):
        rows.append(search_row(now(), base, b0 + j, b0 // lanes, r, st, args.max_rounds, oks[j],
                               int(visited[j]), int(ms[j]), counter.convention, secs, dets[j]))
  g.close()

  fails = sum(1 for r in rows if r["correctness_ok"] is False)
  if not args.quiet:
    for r in rows:
      ok = r["correctness_ok"]
      print(f"search {r['search_idx'] + 1}/{len(rows)}: source={r['source']} "
            f"visited={r['visited_count']}/{n} rounds={r['rounds_completed']} "
            f"m={r['m_edges_traversed']} time={r['search_time_seconds'] * 1e6:.2f}us "
            f"gteps={r['gteps']:.3f}" + ("" if ok is None else (" OK" if ok else " FAILED")))
  gv = [r["gteps"] for r in rows if np.isfinite(r["gteps"]) and r["gteps"] > 0]
  summary = dict(timestamp=now(), **base, num_searches=len(rows), num_correctness_fail=fails,
                 construction_time_seconds=construction_s,
                 harmonic_mean_gteps=harmonic_mean(gv),
                 min_gteps=min(gv) if gv else float("nan"),
                 median_gteps=float(np.median(gv)) if gv else float("nan"),
                 max_gteps=max(gv) if gv else float("nan"))
  if args.mode == "batched":
    t = {}
    for r in rows:
      t[r["batch"]] = r["search_time_seconds"]
    summary["batched_gteps"] = gteps(sum(r["m_edges_traversed"] for r in rows), sum(t.values()))
  print(f"\n[[ {len(rows)} searches complete, {fails} correctness FAILURES ]]")
  print(f"[[ GTEPS across searches: harmonic_mean={summary['harmonic_mean_gteps']:.3f}, "
        f"min={summary['min_gteps']:.3f}, median={summary['median_gteps']:.3f}, "
        f"max={summary['max_gteps']:.3f} ]]"
        + ("" if a.symmetric else "  -- directed graph: not Graph500-spec-comparable")
        + (f"\n[[ batched GTEPS (sum m / sum batch time): {summary['batched_gteps']:.3f} ]]"
           if "batched_gteps" in summary else ""))
  if args.csv:
    append_csv(args.csv, rows)
  if args.summary_csv:
    append_csv(args.summary_csv, [summary])
  return 1 if fails else 0


def search_row(ts, base, i, batch, root, st, max_rounds, ok, visited, m, convention, secs,
               detail):
  """One per-search CSV row (the reference's columns, run_graph500.py:408-430,
  with cycle counts replaced by seconds and the per-round device times)."""
  from .bfs_timing import gteps
  h = min(len(st["round_ns"]), max_rounds)
  row = dict(timestamp=ts, **base, search_idx=i, batch=batch, source=int(root),
             rounds_completed=st["rounds"], profiled_rounds=h, max_rounds=max_rounds,
             pull_rounds=st["pull_rounds"], correctness_ok=ok, visited_count=visited,
             m_edges_traversed=m, m_convention=convention, search_time_seconds=secs,
             gteps=gteps(m, secs), device_ms=st["device_ms"])
  row["round_us"] = ";".join(f"{x / 1e3:.1f}" for x in st["round_ns"][:h])
  # T = top-down (push) round, B = bottom-up (pull) round
  row["directions"] = "".join("TB"[d] if d in (0, 1) else "?" for d in
                              st["direction_history"][:h])
  row["failed_checks"] = "" if detail is None else ";".join(
      f"{c}={detail[c]['failures']}" for c in CHECK_NAMES if detail[c]["failures"])
  return row


def main(argv=None):
  return run(parse_args(argv))


if __name__ == "__main__":
  sys.exit(main())
