"""Graph files: the native parser and the device build against the
reference's own load_graph (fixtures in golden.json's "loader" section, made
by tests/golden/make_golden.py from bfs/implementation/graph_loader.py)."""
import ctypes
import gzip

import numpy as np
import pytest

from ceregraphs_gb300 import _lib, loader
from golden_data import golden


def _cases():
  return golden()["loader"]


def _write(tmp_path, case):
  path = tmp_path / case["file"]
  data = case["text"].encode()
  if case["file"].endswith(".gz"):
    with gzip.open(path, "wb") as f:
      f.write(data)
  else:
    path.write_bytes(data)
  return path


@pytest.mark.parametrize("name", sorted(golden()["loader"]))
def test_parse_matches_reference_loader(built_lib, tmp_path, name):
  case = _cases()[name]
  path = _write(tmp_path, case)
  a = loader.load_arrays(path)
  assert [a.n, a.n] == case["shape"]
  np.testing.assert_array_equal(a.in_off, case["indptr"])
  np.testing.assert_array_equal(a.in_idx, case["indices"])
  # symmetric exactly when A == A^T
  ind = np.asarray(case["indices"])
  rows = np.repeat(np.arange(a.n), np.diff(case["indptr"]))
  entries = set(zip(rows.tolist(), ind.tolist()))
  assert a.symmetric == (entries == {(c, r) for r, c in entries})


def test_parse_threads_agree(built_lib):
  rng = np.random.default_rng(11)
  m = 400_000
  u = rng.integers(0, 1 << 20, m)
  v = rng.integers(0, 1 << 20, m)
  lines = [f"{a}\t{b}" for a, b in zip(u.tolist(), v.tolist())]
  text = ("# Nodes: 2000000\n" + "\n".join(lines) + "\n").encode()
  one = loader.parse_edges(text, threads=1)
  many = loader.parse_edges(text, threads=8)
  assert one.n == many.n == 2_000_000
  np.testing.assert_array_equal(one.src, u)
  np.testing.assert_array_equal(one.dst, v)
  np.testing.assert_array_equal(many.src, u)
  np.testing.assert_array_equal(many.dst, v)
  mtx = ("%%MatrixMarket matrix coordinate pattern general\n% x\n"
         f"{1 << 20} {1 << 20} {m}\n" +
         "\n".join(f"{b + 1} {a + 1}" for a, b in zip(u.tolist(), v.tolist())) + "\n").encode()
  el = loader.parse_edges(mtx, threads=8)
  assert el.format == "mtx" and el.n == 1 << 20
  np.testing.assert_array_equal(el.src, u)
  np.testing.assert_array_equal(el.dst, v)


@pytest.mark.parametrize("text,status,needle", [
    (b"0 1\n2 x\n", _lib.CG_ERR_PARSE, "line 2"),
    (b"0 1\n3\n", _lib.CG_ERR_PARSE, "two vertex ids"),
    (b"0 -1\n", _lib.CG_ERR_PARSE, "negative"),
    (b"0 99999999999\n", _lib.CG_ERR_PARSE, "int32"),
    (b"%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1\n", _lib.CG_ERR_PARSE,
     "declares 2"),
    (b"%%MatrixMarket matrix coordinate real general\n3 4 1\n1 1 1\n", _lib.CG_ERR_PARSE,
     "square"),
    (b"%%MatrixMarket matrix coordinate real general\n3 3 1\n4 1 1\n", _lib.CG_ERR_PARSE,
     "out of range"),
    (b"%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", _lib.CG_ERR_NOT_SUPPORTED,
     "array"),
    (b"%%MatrixMarket matrix coordinate real sideways\n2 2 0\n", _lib.CG_ERR_PARSE, "symmetry"),
])
def test_parse_errors(built_lib, text, status, needle):
  with pytest.raises(_lib.CgError) as e:
    loader.parse_edges(text)
  assert e.value.status == status and needle in str(e.value)


def test_empty_and_comment_only(built_lib):
  el = loader.parse_edges(b"")
  assert el.n == 0 and len(el.src) == 0
  el = loader.parse_edges(b"# Nodes: 5\n\n   \n")
  assert el.n == 5 and len(el.src) == 0


def test_load_missing_file_is_an_io_error(built_lib, tmp_path):
  lib = _lib.load()
  h = ctypes.c_void_p()
  rc = lib.cg_graph_load(str(tmp_path / "nope.mtx").encode(), 0, ctypes.byref(h))
  assert rc == _lib.CG_ERR_IO and not h.value


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(golden()["loader"]))
def test_device_build_from_file(built_lib, tmp_path, name):
  case = _cases()[name]
  path = _write(tmp_path, case)
  with loader.load_graph(path) as g:
    a = g.export()
    assert [g.n, g.n] == case["shape"]
    np.testing.assert_array_equal(a.in_off, case["indptr"])
    np.testing.assert_array_equal(a.in_idx, case["indices"])
    host = loader.load_arrays(path)
    assert g.symmetric == host.symmetric
    if not g.symmetric:
      np.testing.assert_array_equal(a.out_off, host.out_off)
      np.testing.assert_array_equal(a.out_idx, host.out_idx)


@pytest.mark.gpu
def test_load_then_search_matches_oracle(built_lib, oracle_mod, tmp_path):
  """A directed edge list and a symmetric Matrix Market file through
  cg_graph_load, then searched; levels and parents equal the oracle's."""
  rng = np.random.default_rng(12)
  n, m = 5000, 40000
  u = rng.integers(0, n, m)
  v = rng.integers(0, n, m)
  p1 = tmp_path / "d.txt"
  p1.write_text(f"# Nodes: {n}\n" + "\n".join(f"{a} {b}" for a, b in zip(u, v)) + "\n")
  keep = u != v
  p2 = tmp_path / "s.mtx"
  p2.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n"
                f"{n} {n} {int(keep.sum())}\n" +
                "\n".join(f"{a + 1} {b + 1}" for a, b in zip(u[keep], v[keep])) + "\n")
  for path, sym in ((p1, False), (p2, True)):
    lib = _lib.load()
    h = ctypes.c_void_p()
    _lib.check(lib.cg_graph_load(str(path).encode(), 0, ctypes.byref(h)), "cg_graph_load")
    from ceregraphs_gb300.engine import Graph
    with Graph.from_handle(h) as g:
      assert g.symmetric == sym
      a = loader.load_arrays(path)
      out_off, out_idx = a.out_lists()
      for root in (0, 17, 4999):
        lv, pa, _ = g.bfs(root)
        wl, wp, _ = oracle_mod.bfs(out_off, out_idx, a.in_off, a.in_idx, root)
        np.testing.assert_array_equal(lv, wl)
        np.testing.assert_array_equal(pa, wp)
