"""Regenerate the golden fixtures in this folder from the reference itself.

Run in a container that has the reference checked out (it is NOT needed at
test time; the fixtures are committed):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/CereGraphs

Every number stored here comes from the reference's own Python modules,
imported unmodified:

* datasets/gen_rmat.py:15-44            rmat()                -> graph hashes
* bfs/scripts/run_graph500.py:106-134   pick_sources(), harmonic_mean()
* bfs/implementation/bfs_timing.py:379  compute_m_and_gteps()
* bfs/implementation/device_io.py:157   extract_parent_result(), derive_visited_from_parent()
* bfs/plots/bfs_tree_plot.py:140        invalid_parents()
* bfs/implementation/graph_loader.py:27 load_graph()          -> (dst, src) rule
* scipy.sparse.csgraph.breadth_first_order on A^T, as run_graph500.py:383-395
  calls it, for levels (derived from its predecessors), reached sets and its
  own predecessors (the FIFO parent rule).

The lowest-index parents stored next to the levels are derived from those
levels with np.minimum.at over the edge list (bfs/README.md:208-224), i.e.
from the reference's own search, not from this repository's oracle.

Modules that import the Cerebras SDK or matplotlib at top level get empty
stand-in modules in sys.modules; none of the functions used touches them.
"""
import hashlib
import json
import os
import sys
import tempfile
import types

import numpy as np
from scipy import sparse
from scipy.sparse.csgraph import breadth_first_order

HERE = os.path.dirname(os.path.abspath(__file__))


def sha(a):
  return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def canon(A):
  A = sparse.csr_matrix(A)
  A.sort_indices()
  return A.indptr.astype(np.int64), A.indices.astype(np.int32)


def stub(name, **attrs):
  mod = types.ModuleType(name)
  for k, v in attrs.items():
    setattr(mod, k, v)
  sys.modules[name] = mod
  return mod


def import_reference(ref):
  sys.path.insert(0, os.path.join(ref, "datasets"))
  sys.path.insert(0, os.path.join(ref, "bfs", "implementation"))
  sys.path.insert(0, os.path.join(ref, "bfs", "plots"))
  sys.path.insert(0, os.path.join(ref, "bfs", "scripts"))
  # Cerebras SDK and matplotlib stand-ins (not installed here).
  for name in ("cerebras", "cerebras.sdk", "cerebras.sdk.runtime"):
    stub(name)
  stub("cerebras.sdk.runtime.sdkruntimepybind", MemcpyDataType=None, MemcpyOrder=None,
       SdkRuntime=None)
  stub("cerebras.sdk.debug")
  stub("cerebras.sdk.debug.debug_util", debug_util=None)
  mpl = stub("matplotlib", use=lambda *a, **k: None)
  mpl.pyplot = stub("matplotlib.pyplot")
  stub("matplotlib.colors")
  import gen_rmat  # noqa: E402
  import bfs_timing  # noqa: E402
  import device_io  # noqa: E402
  import graph_loader  # noqa: E402
  import bfs_tree_plot  # noqa: E402
  import run_graph500  # noqa: E402
  return gen_rmat, bfs_timing, device_io, graph_loader, bfs_tree_plot, run_graph500


def scipy_levels(A_csr, source):
  A_fwd = A_csr.transpose().tocsr()
  order, pred = breadth_first_order(A_fwd, source, directed=True, return_predecessors=True)
  n = A_csr.shape[0]
  lv = np.full(n, -1, dtype=np.int32)
  lv[source] = 0
  for v in order[1:]:
    lv[v] = lv[pred[v]] + 1
  pred = pred.astype(np.int64)
  pred[pred < 0] = -1
  pred[source] = source
  return lv, pred


def min_parent(A_csr, lv, source):
  coo = A_csr.tocoo()
  r, c = coo.row.astype(np.int64), coo.col.astype(np.int64)
  lv = lv.astype(np.int64)
  sel = (lv[r] >= 1) & (lv[c] == lv[r] - 1)
  big = np.iinfo(np.int64).max
  p = np.full(len(lv), big, dtype=np.int64)
  np.minimum.at(p, r[sel], c[sel])
  p[p == big] = -1
  p[source] = source
  return p.astype(np.int32)


def search_record(A, source, is_symmetric, bfs_timing, device_io, bfs_tree_plot, full):
  lv, pred = scipy_levels(A, source)
  mp = min_parent(A, lv, source)
  n = A.shape[0]
  # round-trip the parents through the reference's own readback convention
  raw = np.where(mp < 0, device_io.PARENT_NONE_GLOBAL, mp.astype(np.int64)).astype(np.uint32)
  parent = device_io.extract_parent_result(n, n, 1, raw.reshape(1, 1, n))
  parent[source] = source
  visited = device_io.derive_visited_from_parent(n, parent, source)
  assert np.array_equal(visited, lv >= 0)
  bad = bfs_tree_plot.invalid_parents(parent, visited, A, source)
  assert not bad, bad
  m, conv, _, _ = bfs_timing.compute_m_and_gteps(A.tocoo(), visited, is_symmetric, 875e6)
  rec = {"source": int(source), "rounds": int(lv.max()) + 1, "visited": int(visited.sum()),
         "m": int(m), "m_convention": conv, "levels_sha": sha(lv), "parents_sha": sha(mp),
         "scipy_parents_sha": sha(pred.astype(np.int32)),
         "scipy_parent_differs": int(np.sum((pred != mp) & (lv > 0)))}
  if full:
    rec["levels"] = lv
    rec["parents"] = mp
    rec["scipy_parents"] = pred.astype(np.int32)
  return rec


# Graph files for the loader, each read by the reference's load_graph
# (graph_loader.py:27-95): format detection, the (dst, src) rule, "Nodes:"
# declarations, Python's universal newlines, mmread's symmetric expansion.
LOADER_CASES = {
    "snap": ("tiny.txt",
             "# Directed graph\n# Nodes: 7 Edges: 6\n0\t1\n0\t2\n2\t3\n3\t0\n4\t5\n5 5\n"),
    "snap_crlf_extra_columns": ("crlf.txt",
                                "# Nodes: 10\r\n1 2 0.5 x\r\n\r\n  3\t4  \r\n2 1\r\n9 0\r\n"),
    "snap_cr_only": ("cr.txt", "0 1\r1 2\r# c\r2 0\r"),
    "snap_declared_too_small": ("small.txt", "# Nodes: 3\n0 5\n5 0\n"),
    "snap_duplicates_and_loops": ("dup.txt", "1 1\n1 2\n1 2\n2 1\n# Nodes:   4 Edges: 9\n"),
    "snap_gzip": ("g.txt.gz", "# Nodes: 6\n0 1\n1 2\n2 3\n3 4\n4 5\n5 0\n"),
    "mtx": ("tiny.mtx", "%%MatrixMarket matrix coordinate real general\n% tiny\n5 5 6\n"
                        "1 2 1.0\n2 1 1.0\n2 3 1.0\n3 2 1.0\n4 5 1.0\n5 4 1.0\n"),
    "mtx_pattern_symmetric": ("sym.mtx", "%%MatrixMarket matrix coordinate pattern symmetric\n"
                                         "% c1\n%c2\n6 6 5\n2 1\n3 1\n3 3\n6 4\n5 2\n"),
    "mtx_integer_skew": ("skew.mtx", "%%MatrixMarket matrix coordinate integer skew-symmetric\n"
                                     "4 4 3\n2 1 5\n3 2 -1\n4 1 7\n"),
    "mtx_duplicates_zero": ("dupz.mtx", "%%MatrixMarket matrix coordinate real general\n"
                                        "3 3 4\n1 2 0.0\n1 2 1.5\n3 1 2\n3 3 0\n"),
}


def loader_cases(graph_loader):
  import gzip
  cases = {}
  with tempfile.TemporaryDirectory() as td:
    for name, (fname, text) in LOADER_CASES.items():
      path = os.path.join(td, fname)
      if fname.endswith(".gz"):
        with gzip.open(path, "wb") as f:
          f.write(text.encode())
      else:
        with open(path, "w", encoding="utf-8", newline="") as f:
          f.write(text)
      M = sparse.csr_matrix(graph_loader.load_graph(path))
      M.sum_duplicates()
      M.sort_indices()
      cases[name] = {"file": fname, "text": text, "shape": list(M.shape),
                     "indptr": M.indptr.tolist(), "indices": M.indices.tolist()}
  return cases


def main(ref):
  gen_rmat, bfs_timing, device_io, graph_loader, bfs_tree_plot, rg = import_reference(ref)
  out = {"graphs": {}, "searches": {}, "pick_sources": {}, "harmonic_mean": [],
         "invalid_parents": {}, "loader": {}}

  # --- graphs: hashes of the reference generator's CSR ---
  graphs = [(8, 16, 0), (10, 16, 0), (12, 16, 0), (12, 4, 0), (14, 16, 3), (16, 16, 0)]
  mats = {}
  for (s, ef, seed) in graphs:
    A = gen_rmat.rmat(s, ef, seed)
    indptr, indices = canon(A)
    deg = np.diff(indptr)
    key = f"s{s}_e{ef}_seed{seed}"
    out["graphs"][key] = {"scale": s, "edgefactor": ef, "seed": seed, "n": int(A.shape[0]),
                          "nnz": int(A.nnz), "indptr_sha": sha(indptr),
                          "indices_sha": sha(indices), "max_degree": int(deg.max()),
                          "isolated": int(np.sum(deg == 0))}
    mats[key] = sparse.csr_matrix((np.ones(len(indices)), indices, indptr), shape=A.shape)

  # --- root sampling (the Graph500 rule) ---
  class Args:
    sources = None
  for key, k, seed in [("s12_e16_seed0", 16, 1), ("s16_e16_seed0", 64, 1),
                       ("s14_e16_seed3", 64, 3), ("s8_e16_seed0", 400, 5)]:
    A = mats[key]
    a = Args()
    a.num_searches, a.seed = k, seed
    roots = rg.pick_sources(a, A.tocsc(), A.shape[0])
    out["pick_sources"][f"{key}_k{k}_seed{seed}"] = [int(r) for r in roots]

  # --- searches ---
  arrays = {}
  for key in ("s10_e16_seed0", "s12_e16_seed0", "s12_e4_seed0"):
    A = mats[key]
    roots = [0] + out["pick_sources"].get(f"{key}_k16_seed1", [])[:7]
    if key != "s12_e16_seed0":
      a = Args()
      a.num_searches, a.seed = 8, 1
      roots = [0] + [int(r) for r in rg.pick_sources(a, A.tocsc(), A.shape[0])]
    # an isolated vertex as a root too: the reference still runs it
    deg = np.diff(A.indptr)
    iso = np.nonzero(deg == 0)[0]
    if len(iso):
      roots.append(int(iso[0]))
    recs = []
    for r in roots:
      rec = search_record(A, r, True, bfs_timing, device_io, bfs_tree_plot, full=True)
      arrays[f"{key}_r{r}_levels"] = rec.pop("levels")
      arrays[f"{key}_r{r}_parents"] = rec.pop("parents")
      arrays[f"{key}_r{r}_scipy_parents"] = rec.pop("scipy_parents")
      recs.append(rec)
    out["searches"][key] = recs
  for key, roots in (("s16_e16_seed0", [0] + out["pick_sources"]["s16_e16_seed0_k64_seed1"][:3]),):
    out["searches"][key] = [search_record(mats[key], r, True, bfs_timing, device_io,
                                          bfs_tree_plot, full=False) for r in roots]

  # --- a directed matrix with self-loops (the rand600.mtx kind of input) ---
  rng = np.random.default_rng(600)
  n = 600
  e = 2400
  src = rng.integers(0, n, e)
  dst = rng.integers(0, n, e)
  src = np.concatenate([src, np.arange(0, n, 37)])  # a few self-loops
  dst = np.concatenate([dst, np.arange(0, n, 37)])
  D = sparse.coo_matrix((np.ones(len(src)), (dst, src)), shape=(n, n)).tocsr()
  D.sum_duplicates()
  D.data[:] = 1.0
  D.sort_indices()
  arrays["dir600_indptr"], arrays["dir600_indices"] = canon(D)
  recs = []
  a = Args()
  a.num_searches, a.seed = 6, 7
  droots = [int(r) for r in rg.pick_sources(a, D.tocsc(), n)]
  out["pick_sources"]["dir600_k6_seed7"] = droots
  for r in droots:
    rec = search_record(D, r, False, bfs_timing, device_io, bfs_tree_plot, full=True)
    arrays[f"dir600_r{r}_levels"] = rec.pop("levels")
    arrays[f"dir600_r{r}_parents"] = rec.pop("parents")
    arrays[f"dir600_r{r}_scipy_parents"] = rec.pop("scipy_parents")
    recs.append(rec)
  out["searches"]["dir600"] = recs

  # --- harmonic mean ---
  for vals in ([1.0, 2.0, 4.0], [0.5, float("inf"), 3.0, -1.0, 2.0], [0.0], [12.5]):
    hm = rg.harmonic_mean(vals)
    out["harmonic_mean"].append({"values": [str(v) for v in vals], "hm": repr(float(hm))})

  # --- invalid_parents on a planted mistake (s10 root 0) ---
  A = mats["s10_e16_seed0"]
  lv = arrays["s10_e16_seed0_r0_levels"]
  p = arrays["s10_e16_seed0_r0_parents"].astype(np.int64).copy()
  visited = lv >= 0
  reached = np.nonzero(visited & (np.arange(len(lv)) != 0))[0]
  p[reached[3]] = reached[3]          # self as parent: no such edge (no loops)
  p[reached[10]] = -1                 # visited but no parent
  unreached = np.nonzero(~visited)[0]
  if len(unreached):
    p[reached[20]] = unreached[0]     # parent is not visited
  out["invalid_parents"]["s10_e16_seed0_r0"] = {
      "planted": p.tolist(),
      "bad": [int(x) for x in bfs_tree_plot.invalid_parents(p, visited, A, 0)]}

  out["loader"] = loader_cases(graph_loader)

  with open(os.path.join(HERE, "golden.json"), "w", encoding="utf-8") as f:
    json.dump(out, f, indent=1, sort_keys=True)
  np.savez_compressed(os.path.join(HERE, "golden_arrays.npz"), **arrays)
  print("wrote golden.json and golden_arrays.npz")


def main_loader_only(ref):
  """Refresh only the loader section of golden.json."""
  mods = import_reference(ref)
  path = os.path.join(HERE, "golden.json")
  with open(path, encoding="utf-8") as f:
    out = json.load(f)
  out["loader"] = loader_cases(mods[3])
  with open(path, "w", encoding="utf-8") as f:
    json.dump(out, f, indent=1, sort_keys=True)
  print("refreshed the loader section of golden.json")


if __name__ == "__main__":
  args = [a for a in sys.argv[1:] if not a.startswith("--")]
  if len(args) != 1:
    sys.exit("usage: make_golden.py REFERENCE_CHECKOUT [--loader-only]")
  ref_dir = args[0]
  if "--loader-only" in sys.argv:
    main_loader_only(ref_dir)
  else:
    main(ref_dir)
