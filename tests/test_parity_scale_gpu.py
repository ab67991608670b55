"""Parity at the benchmark sizes, through the C ABI: levels and lowest-index
parents of the CUDA searches equal the C oracle's bit for bit on the graphs the
benchmark runs, not only on small ones.

* R-MAT scale 21, edgefactor 16, seed 0 with the 64 Graph500 roots of seed 1
  (the per-root workload);
* R-MAT scale 23, edgefactor 16, seed 2 with the 64 roots of seed 3 (the
  batched-vs-per-root workload): every per-root search and every lane of the
  64-lane batch;
* the uneven-depth graphs at full size: R-MAT scale 22 edgefactor 32, the
  directed Erdos-Renyi graph with 2^22 vertices and mean out-degree 8 (seed 4)
  and the 4096 x 4096 grid, roots of seed 5: every lane of a 128-lane batch
  (the grid's is deeper than the round history, so it runs in the direct
  kernel), a batch forced into the direct kernel, and per-root searches.

The reference checks every search of a run against its host BFS at the run's
own scale (run_graph500.py:383-395); so do these tests.  The oracle's searches
run on all host cores (its ctypes calls release the GIL) in groups, compared
lane by lane so the host holds only a group's outputs at a time.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from ceregraphs_gb300 import generators, graph500
from ceregraphs_gb300.engine import Graph

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


def _oracle_groups(oracle_mod, a, roots):
  """Yields (i, (levels, parents, rounds)) for every root, THREADS at a time."""
  out_off, out_idx = a.out_lists()

  def one(r):
    return oracle_mod.bfs(out_off, out_idx, a.in_off, a.in_idx, int(r))

  with ThreadPoolExecutor(THREADS) as ex:
    for g0 in range(0, len(roots), THREADS):
      part = roots[g0:g0 + THREADS]
      for j, res in enumerate(ex.map(one, part)):
        yield g0 + j, res


def _check_batch(torch, oracle_mod, g, a, roots, lane_words, ms_history=0, label=""):
  """One batched search of `roots` on the device; every lane against the oracle."""
  k = len(roots)
  g.set_options(lane_words=lane_words, ms_history=ms_history)
  d_lv = torch.empty((k, a.n), dtype=torch.int32, device="cuda")
  d_pa = torch.empty((k, a.n), dtype=torch.int32, device="cuda")
  torch.cuda.synchronize()
  g.msbfs_device(roots, d_lv, d_pa)
  st = g.last_stats()
  assert st["status"] == 0, (label, st)
  max_rounds = 0
  for i, (rl, rp, rounds) in _oracle_groups(oracle_mod, a, roots):
    lv = d_lv[i].cpu().numpy()
    pa = d_pa[i].cpu().numpy()
    assert np.array_equal(lv, rl), (label, "levels", i, roots[i])
    assert np.array_equal(pa, rp), (label, "parents", i, roots[i])
    max_rounds = max(max_rounds, rounds)
  assert st["rounds"] == max_rounds, (label, st["rounds"], max_rounds)
  g.set_options(ms_history=0)
  del d_lv, d_pa
  torch.cuda.empty_cache()
  return st


def _check_per_root(torch, oracle_mod, g, a, roots, label=""):
  """Per-root searches (default direction policy) against the oracle."""
  d_lv = torch.empty(a.n, dtype=torch.int32, device="cuda")
  d_pa = torch.empty(a.n, dtype=torch.int32, device="cuda")
  torch.cuda.synchronize()
  for i, (rl, rp, rounds) in _oracle_groups(oracle_mod, a, roots):
    g.bfs_device(roots[i], d_lv, d_pa)
    st = g.last_stats()
    assert st["status"] == 0, (label, st)
    assert np.array_equal(d_lv.cpu().numpy(), rl), (label, "levels", roots[i])
    assert np.array_equal(d_pa.cpu().numpy(), rp), (label, "parents", roots[i])
    assert st["rounds"] == rounds, (label, roots[i], st["rounds"], rounds)


@pytest.mark.parametrize("scale,seed,root_seed", [(21, 0, 1), (23, 2, 3)])
def test_graph500_workload_every_search_vs_oracle(built_lib, oracle_mod, scale, seed, root_seed):
  torch = pytest.importorskip("torch")
  g, a = generators.rmat_device(scale, 16, seed)
  with g:
    roots = graph500.pick_sources(a, 64, root_seed)
    assert len(roots) == 64
    _check_per_root(torch, oracle_mod, g, a, roots, f"s{scale} per-root")
    _check_batch(torch, oracle_mod, g, a, roots, 1, label=f"s{scale} batch")
    # Graph500 m of a few lanes, device count against the C restatement
    d_lv = torch.empty((4, a.n), dtype=torch.int32, device="cuda")
    d_pa = torch.empty((4, a.n), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    g.msbfs_device(roots[:4], d_lv, d_pa)
    m = g.count_edges(d_lv, 4)
    for i in range(4):
      assert m[i] == oracle_mod.count_m(a.in_off, a.in_idx, d_lv[i].cpu().numpy(), True)


def _uneven_graph(name):
  if name == "rmat22-e32":
    return generators.rmat_device(22, 32, 0)
  if name == "er22-d8":
    return generators.er_directed_device(22, 8, 4)
  a = generators.grid2d(4096)
  return Graph(a), a


@pytest.mark.parametrize("name", ["rmat22-e32", "er22-d8", "grid4096"])
def test_uneven_depth_graphs_full_size_vs_oracle(built_lib, oracle_mod, name):
  torch = pytest.importorskip("torch")
  g, a = _uneven_graph(name)
  with g:
    roots = graph500.pick_sources(a, 256, 5)
    # one 128-lane batch, every lane (the grid's runs in the direct kernel:
    # it is deeper than the round history)
    _check_batch(torch, oracle_mod, g, a, roots[:128], 2, label=f"{name} 128 lanes")
    # the direct kernel on purpose (no round history), 64 lanes
    if name != "grid4096":
      _check_batch(torch, oracle_mod, g, a, roots[128:192], 1, ms_history=-1,
                   label=f"{name} direct kernel")
    _check_per_root(torch, oracle_mod, g, a, roots[192:194], f"{name} per-root")
