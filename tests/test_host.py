"""Host-side logic of the package (no GPU): generators, root sampling, the
edge-count metric, readback conventions, CSR/CSC preparation, the ABI."""
import ctypes
import os
import re

import numpy as np
import pytest

from golden_data import arrays, csr_from, golden, sha
from ceregraphs_gb300 import bfs_timing, device_io, generators, graph500, preprocess

G = golden()
ARR = arrays()
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("key", ["s8_e16_seed0", "s10_e16_seed0", "s12_e4_seed0",
                                 "s14_e16_seed3"])
def test_product_rmat_is_bit_identical_to_reference(key):
  g = G["graphs"][key]
  a = generators.rmat(g["scale"], g["edgefactor"], g["seed"])
  assert a.symmetric and a.n == g["n"] and a.nnz == g["nnz"]
  assert sha(a.in_off.astype(np.int64)) == g["indptr_sha"]
  assert sha(a.in_idx.astype(np.int32)) == g["indices_sha"]


def test_product_rmat_chunked_draws_match_unchunked():
  u1, v1 = generators.rmat_edge_endpoints(9, 8, 4, chunk=1 << 30)
  u2, v2 = generators.rmat_edge_endpoints(9, 8, 4, chunk=777)
  assert np.array_equal(u1, u2) and np.array_equal(v1, v2)


def test_pick_sources_matches_reference():
  for key, roots in G["pick_sources"].items():
    if key.startswith("dir600"):
      A = csr_from(ARR["dir600_indptr"], ARR["dir600_indices"], 600)
      a = preprocess.preprocess(A)
      k, seed = 6, 7
    else:
      gk, rest = key.rsplit("_k", 1)
      k, seed = (int(x) for x in rest.split("_seed"))
      g = G["graphs"][gk]
      a = generators.rmat(g["scale"], g["edgefactor"], g["seed"])
    assert graph500.pick_sources(a, k, seed) == roots, key


def test_harmonic_mean_matches_reference():
  for case in G["harmonic_mean"]:
    vals = [float(v) for v in case["values"]]
    got, want = bfs_timing.harmonic_mean(vals), float(case["hm"])
    assert (np.isnan(got) and np.isnan(want)) or got == want


def test_edge_counter_matches_reference_m():
  g = G["graphs"]["s12_e16_seed0"]
  a = generators.rmat(g["scale"], g["edgefactor"], g["seed"])
  ec = graph500.EdgeCounter(a)
  for rec in G["searches"]["s12_e16_seed0"]:
    lv = ARR[f"s12_e16_seed0_r{rec['source']}_levels"]
    assert ec.m(lv >= 0) == rec["m"]
    assert bfs_timing.compute_m(a.scipy_csr(), lv >= 0, True) == rec["m"]
  D = csr_from(ARR["dir600_indptr"], ARR["dir600_indices"], 600)
  d = preprocess.preprocess(D)
  assert not d.symmetric
  ec = graph500.EdgeCounter(d)
  for rec in G["searches"]["dir600"]:
    lv = ARR[f"dir600_r{rec['source']}_levels"]
    assert ec.m(lv >= 0) == rec["m"]


def test_device_io_conventions():
  raw = np.array([5, 0xFFFFFFFF, 2, 0xFFFFFFFF], dtype=np.uint32)
  p = device_io.extract_parent_result(4, raw)
  assert p.tolist() == [5, -1, 2, -1]
  assert device_io.extract_parent_result(4, raw.view(np.int32)).tolist() == [5, -1, 2, -1]
  assert device_io.derive_visited_from_parent(4, p, 1).tolist() == [True, True, True, False]
  with pytest.raises(ValueError):
    device_io.check_root(4, 4)


def test_preprocess_directed_keeps_both_orientations():
  D = csr_from(ARR["dir600_indptr"], ARR["dir600_indices"], 600)
  a = preprocess.preprocess(D)
  C = D.tocsc()
  C.sort_indices()
  assert np.array_equal(a.out_off, C.indptr) and np.array_equal(a.out_idx, C.indices)
  for off, idx in ((a.in_off, a.in_idx), (a.out_off, a.out_idx)):
    for v in range(0, 600, 13):
      row = idx[off[v]:off[v + 1]]
      assert np.all(np.diff(row) > 0)


def test_er_and_grid_generators():
  e = generators.er_directed(10, 8, 4)
  assert not e.symmetric and e.n == 1024
  A = e.scipy_csr()
  assert A.diagonal().sum() == 0 and A.nnz == e.nnz <= 1024 * 8
  g = generators.grid2d(5)
  assert g.symmetric and g.n == 25 and g.nnz == 2 * 2 * 5 * 4
  deg = np.diff(g.in_off)
  assert deg[0] == 2 and deg[6] == 4


def _declared_functions():
  text = open(os.path.join(ROOT, "include", "ceregraphs.h"), encoding="utf-8").read()
  text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
  return sorted(set(re.findall(r"\b(cg_\w+)\s*\(", text)))


def test_abi_library_exports_every_declared_symbol(built_lib):
  from ceregraphs_gb300 import _lib
  declared = _declared_functions()
  assert declared, "no declarations parsed"
  for name in declared:
    assert name in _lib.SIGNATURES, f"{name} has no binding"
    assert hasattr(built_lib, name), f"{name} not exported"
  assert set(_lib.SIGNATURES) == set(declared)


def test_abi_calls_that_need_no_gpu(built_lib):
  from ceregraphs_gb300 import _lib
  assert built_lib.cg_version() >= 10000
  assert built_lib.cg_strerror(_lib.CG_ERR_TIMEOUT).decode().startswith("device-side wait")
  opt = _lib.default_options()
  assert opt.direction == _lib.CG_DIR_AUTO and opt.lane_words == 1
  assert opt.parent_rule == _lib.CG_PARENT_LOWEST
  # argument checks return before any CUDA call
  h = ctypes.c_void_p()
  assert built_lib.cg_graph_create(0, 0, None, None, None, None, 0, ctypes.byref(h)) == \
      _lib.CG_ERR_INVALID_ARG
  off = np.array([0, 1, 1], dtype=np.int64)
  bad = np.array([7], dtype=np.int32)  # index out of range
  assert built_lib.cg_graph_create(2, 1, off.ctypes.data_as(ctypes.c_void_p),
                                   bad.ctypes.data_as(ctypes.c_void_p), None, None,
                                   _lib.CG_GRAPH_SYMMETRIC, ctypes.byref(h)) == \
      _lib.CG_ERR_INVALID_ARG
  assert built_lib.cg_bfs(None, 0, None, None, None) == _lib.CG_ERR_INVALID_ARG
  assert built_lib.cg_graph_destroy(None) == _lib.CG_ERR_INVALID_ARG


def test_grid_csr_is_sorted_and_symmetric():
  a = generators.grid2d(7)
  A = a.scipy_csr()
  assert (A != A.T).nnz == 0
  for v in range(a.n):
    row = a.in_idx[a.in_off[v]:a.in_off[v + 1]]
    assert np.all(np.diff(row) > 0)


def test_driver_csv_header_guard(tmp_path):
  from ceregraphs_gb300 import run_graph500
  p = tmp_path / "s.csv"
  run_graph500.append_csv(str(p), [{"a": 1, "b": 2}])
  run_graph500.append_csv(str(p), [{"a": 3, "b": 4}])
  assert p.read_text().splitlines() == ["a,b", "1,2", "3,4"]
  with pytest.raises(SystemExit):
    run_graph500.append_csv(str(p), [{"a": 1, "c": 2}])


def test_driver_arguments():
  from ceregraphs_gb300 import run_graph500
  a = run_graph500.parse_args(["--rmat", "12", "16", "0", "--mode", "batched", "--lanes", "128"])
  assert a.rmat == [12, 16, 0] and a.mode == "batched" and a.lanes == 128
  assert a.num_searches == 64 and not a.nocorrectness
  assert a.parent_rule == "lowest"
  assert run_graph500.parse_args(["--rmat", "8", "16", "0", "--parent-rule",
                                  "fifo"]).parent_rule == "fifo"
  with pytest.raises(SystemExit):
    run_graph500.parse_args(["--num-searches", "3"])   # a graph source is required
  with pytest.raises(SystemExit):
    run_graph500.parse_args(["--rmat", "8", "16", "0", "--parent-rule", "last"])


def test_abi_struct_layouts_match_the_header(tmp_path):
  """Every ctypes mirror of a struct in include/ceregraphs.h has the C
  layout: a C program compiled against the header prints each field's offset
  and each struct's size."""
  import shutil
  import subprocess
  from ceregraphs_gb300 import _lib
  cc = shutil.which("gcc") or shutil.which("cc")
  if cc is None:
    pytest.skip("no C compiler")
  structs = {"cg_options": _lib.CgOptions, "cg_stats": _lib.CgStats,
             "cg_edge_list": _lib.CgEdgeList, "cg_validation": _lib.CgValidation}
  lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "ceregraphs.h"',
           "int main(void) {"]
  for cname, cls in structs.items():
    lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
    for f, _ in cls._fields_:
      lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
  lines += ["  return 0;", "}"]
  src = tmp_path / "layout.c"
  src.write_text("\n".join(lines) + "\n")
  exe = tmp_path / "layout"
  inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
  subprocess.check_call([cc, "-std=c99", "-I", inc, str(src), "-o", str(exe)])
  got = {}
  for line in subprocess.check_output([str(exe)]).decode().splitlines():
    name, field, val = line.split()
    got[(name, field)] = int(val)
  for cname, cls in structs.items():
    assert got[(cname, "size")] == ctypes.sizeof(cls), cname
    for f, _ in cls._fields_:
      assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)
