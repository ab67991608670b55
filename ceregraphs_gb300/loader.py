"""Graph files: the replacement of bfs/implementation/graph_loader.py.

``load_graph(path)`` is Kernel 1 from a file: the text is parsed by the
library's multithreaded host parser (cg_parse_edges / cg_graph_from_text) and
the CSR, the CSC and the symmetry test are built on the device.  Formats and
the direction rule follow graph_loader.py:27-95:

* Matrix Market (first line starts with ``%%MatrixMarket``): coordinate
  storage, entry (i, j) is A[i-1, j-1] (the edge j-1 -> i-1), symmetric /
  skew-symmetric / hermitian storage mirrored as scipy.io.mmread does; values
  are ignored, as the reference only consumes indptr/indices.
* anything else is a SNAP edge list: "u v" per line is the edge u -> v
  (A[v, u], graph_loader.py:78-93), '#' comment lines, "Nodes: N" declares
  the vertex count, n = max(N, max id + 1) (graph_loader.py:60-73).

Compressed files (.gz, and .bz2 which mmread also accepts) are decompressed
here before the text reaches the library.
"""
from __future__ import annotations

import bz2
import ctypes
import gzip
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import CgEdgeList, check


@dataclass
class EdgeList:
  n: int
  src: np.ndarray          # uint32, edge src[e] -> dst[e], duplicates kept
  dst: np.ndarray
  format: str              # "mtx" or "edgelist"
  mtx_symmetry: str        # "general", "symmetric", "skew-symmetric", "hermitian"


_SYMMETRY = {0: "general", 1: "symmetric", 2: "skew-symmetric", 3: "hermitian"}


def read_text(path) -> bytes:
  """The file's bytes, decompressed when gzip or bzip2 (by content)."""
  with open(path, "rb") as f:
    head = f.read(3)
  if head[:2] == b"\x1f\x8b":
    with gzip.open(path, "rb") as f:
      return f.read()
  if head == b"BZh":
    with bz2.open(path, "rb") as f:
      return f.read()
  with open(path, "rb") as f:
    return f.read()


def _text(source) -> bytes:
  if isinstance(source, (bytes, bytearray, memoryview)):
    return bytes(source)
  return read_text(source)


def parse_edges(source, threads=0) -> EdgeList:
  """Parse a graph file (path) or its text (bytes) into a host edge list.
  Host-only: needs no GPU."""
  data = _text(source)
  lib = _lib.load()
  el = CgEdgeList()
  check(lib.cg_parse_edges(data, len(data), int(threads), ctypes.byref(el)), "cg_parse_edges")
  try:
    m = el.m
    src = np.ctypeslib.as_array(el.src, shape=(m,)).copy() if m else np.empty(0, np.uint32)
    dst = np.ctypeslib.as_array(el.dst, shape=(m,)).copy() if m else np.empty(0, np.uint32)
    fmt = "mtx" if el.format == _lib.CG_FORMAT_MTX else "edgelist"
    return EdgeList(int(el.n), src, dst, fmt, _SYMMETRY[el.mtx_symmetry])
  finally:
    lib.cg_edge_list_free(ctypes.byref(el))


def load_arrays(source, threads=0):
  """Host GraphArrays of a graph file: the reference's load_graph + tocsr +
  sorted_indices (+ tocsc when A != A^T), for callers that want host CSR."""
  from .preprocess import from_edges
  el = parse_edges(source, threads)
  return from_edges(el.n, el.src.astype(np.int64), el.dst.astype(np.int64))


def load_graph(source, flags=0):
  """Kernel 1 from a graph file (path) or text (bytes): a resident Graph,
  stored once when A == A^T."""
  from .engine import Graph
  data = _text(source)
  h = ctypes.c_void_p()
  check(_lib.load().cg_graph_from_text(data, len(data), int(flags), ctypes.byref(h)),
        "cg_graph_from_text")
  return Graph.from_handle(h)
