"""Single-search driver: the command-line counterpart of bfs/scripts/run_bfs.py.

    python -m ceregraphs_gb300.run_bfs --infile_mtx graph.mtx --source 0
    python -m ceregraphs_gb300.run_bfs --rmat 16 16 0 --source 0 --directional

One search from one source with a per-round report, as the reference's
single-run driver (run_bfs.py:80-150, 160-760), without its wafer-only options
(PE grid, fabric, compiler, per-PE timing dumps) and its plots:

* Kernel 1 -- a graph file through the native loader, or an R-MAT graph of the
  reference generator drawn on the device, kept out of the search's time;
* direction -- top-down by default, as the reference runs without
  --directional; --directional turns on its one-way switch at
  tau = round(0.15 n) (run_bfs.py:112-117, 239-243); --direction picks the
  Beamer rule or pure bottom-up instead;
* the search -- through cg_bfs into page-locked host buffers, timed on the host
  (launch + every round + levels and parents in host memory, the Graph500
  Kernel-2 rule) and on the device;
* per-round report -- device time, direction and vertices found in each round,
  the reference's ts_buf / direction_history / nf_history, up to --max-rounds;
* correctness (skipped by --nocorrectness) -- the Graph500 tree checks on the
  device, and how many parents differ from those scipy's breadth_first_order
  would pick (the reference's "tie-break diffs" next to its scipy cross-check:
  valid alternatives, not errors), from a second search under the FIFO rule;
* GTEPS with and without the host transfers, and one CSV row appended with the
  reference's header check (run_bfs.py:734-753).
"""
from __future__ import annotations

import argparse
import sys
import time
from datetime import datetime, timezone

import numpy as np

DIRECTIONS = ("topdown", "tau", "auto", "bottomup")


def parse_args(argv=None):
  ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
  src = ap.add_mutually_exclusive_group(required=True)
  src.add_argument("--infile_mtx", help="graph file: Matrix Market or SNAP edge list (.gz ok)")
  src.add_argument("--rmat", nargs=3, type=int, metavar=("SCALE", "EDGEFACTOR", "SEED"),
                   help="R-MAT graph of datasets/gen_rmat.py, drawn on the device")
  ap.add_argument("--source", type=int, default=0, help="single BFS source vertex")
  ap.add_argument("--directional", action="store_true",
                  help="the reference's one-way top-down -> bottom-up switch at "
                       "tau = round(0.15 n)")
  ap.add_argument("--direction", choices=DIRECTIONS, default=None,
                  help="direction rule (default: topdown, or tau with --directional)")
  ap.add_argument("--max-rounds", type=int, default=10,
                  help="rounds reported one by one (at most 64)")
  ap.add_argument("--nocorrectness", action="store_true",
                  help="skip the device tree checks and the scipy tie-break count")
  ap.add_argument("--notimings", action="store_true", help="no per-round report")
  ap.add_argument("--warmup", type=int, default=1, help="untimed searches before the timed one")
  ap.add_argument("--csv", default=None, help="append this run's row here")
  args = ap.parse_args(argv)
  if args.direction is None:
    args.direction = "tau" if args.directional else "topdown"
  elif args.directional and args.direction != "tau":
    ap.error("--directional is the tau rule; drop it or pass --direction tau")
  return args


def host_buffers(n):
  """Page-locked levels and parents buffers of n int32."""
  from .engine import PinnedBuffer
  return PinnedBuffer(n), PinnedBuffer(n)


def device_copy(array):
  """A device tensor copy of a host array (for the device tree checks)."""
  import torch
  return torch.from_numpy(np.ascontiguousarray(array)).cuda()


def run(args):
  from . import _lib
  from .bfs_timing import gteps
  from .graph500 import EdgeCounter
  from .run_graph500 import CHECK_NAMES, append_csv, kernel1

  g, a, construction_s, name = kernel1(args)
  n = a.n
  if not 0 <= args.source < n:
    g.close()
    raise SystemExit(f"--source {args.source} out of range [0, {n})")
  print(f"Kernel 1: {name} n={n} nnz={a.nnz} symmetric={a.symmetric} "
        f"construction={construction_s:.3f} s (not part of the search's time)")
  dirmap = {"topdown": _lib.CG_DIR_TOPDOWN, "tau": _lib.CG_DIR_TAU,
            "auto": _lib.CG_DIR_AUTO, "bottomup": _lib.CG_DIR_BOTTOMUP}
  g.set_options(direction=dirmap[args.direction], parent_rule=_lib.CG_PARENT_LOWEST)
  lv_buf, pa_buf = host_buffers(n)
  for _ in range(args.warmup):
    g.bfs(args.source, lv_buf.array, pa_buf.array)
  t0 = time.perf_counter()
  _, _, st = g.bfs(args.source, lv_buf.array, pa_buf.array)
  secs = time.perf_counter() - t0
  levels = np.array(lv_buf.array)
  parents = np.array(pa_buf.array)
  visited = parents >= 0
  counter = EdgeCounter(a)
  m = counter.m(visited)
  device_s = st["device_ms"] * 1e-3
  rounds = st["rounds"]
  h = min(len(st["round_ns"]), args.max_rounds)
  if not args.notimings:
    for i in range(h):
      d = st["direction_history"][i]
      print(f"round {i}: {'top-down' if d == 0 else 'bottom-up'} "
            f"found {st['nf_history'][i]} time {st['round_ns'][i] / 1e3:.1f} us")
    if rounds > h:
      print(f"({rounds - h} more rounds not listed; --max-rounds {rounds} lists them)")

  ok, detail, differs = None, None, None
  if not args.nocorrectness:
    res = g.validate([args.source], device_copy(levels), device_copy(parents))[0]
    detail = {c: res[c]["failures"] for c in CHECK_NAMES}
    ok = all(v == 0 for v in detail.values())
    # the parents scipy's breadth_first_order would pick: the FIFO rule
    g.set_options(parent_rule=_lib.CG_PARENT_FIFO)
    try:
      _, fifo_parents, _ = g.bfs(args.source)
    finally:
      g.set_options(parent_rule=_lib.CG_PARENT_LOWEST)
    differs = int(np.sum((fifo_parents != parents) & (levels > 0)))
    print(f"[[ Graph500 tree checks: {'OK' if ok else 'FAILED ' + str(detail)} ]]")
    print(f"[[ parents that differ from scipy's pick (valid alternatives): {differs} ]]")
  g.close()

  g_e2e = gteps(m, secs)
  g_dev = gteps(m, device_s) if device_s > 0 else float("nan")
  print(f"[[ visited_count = {int(visited.sum())} / {n}, m_edges_traversed = {m} "
        f"({counter.convention}) ]]")
  print(f"[[ GTEPS = {m} edges / {secs * 1e6:.2f} us = {g_e2e:.3f} GTEPS ]]"
        + ("" if a.symmetric else "  -- directed graph: not Graph500-spec-comparable"))
  print(f"[[ GTEPS w/o host transfers = {m} edges / {device_s * 1e6:.2f} us = "
        f"{g_dev:.3f} GTEPS ]]")
  row = dict(
      timestamp=datetime.now(timezone.utc).isoformat(), infile_mtx=name, n=n, nnz=a.nnz,
      matrix_symmetric=a.symmetric, source=args.source, direction=args.direction,
      rounds_completed=rounds, pull_rounds=st["pull_rounds"], switches=st["switches"],
      visited_count=int(visited.sum()), m_edges_traversed=m,
      m_convention=counter.convention, search_time_seconds=secs, gteps=g_e2e,
      device_time_seconds=device_s, gteps_no_transfer=g_dev,
      round_us=";".join(f"{x / 1e3:.1f}" for x in st["round_ns"][:h]),
      directions="".join("TB"[d] if d in (0, 1) else "?" for d in st["direction_history"][:h]),
      nf_history=";".join(str(x) for x in st["nf_history"][:h]),
      correctness_ok=ok,
      failed_checks="" if detail is None else ";".join(
          f"{c}={v}" for c, v in detail.items() if v),
      scipy_parent_differs=differs)
  if args.csv:
    append_csv(args.csv, [row])
    print(f"appended the run's row to {args.csv}")
  return 1 if ok is False else 0


def main(argv=None):
  return run(parse_args(argv))


if __name__ == "__main__":
  sys.exit(main())
