"""ctypes binding of include/ceregraphs.h.

The shared library is the product path: if it is missing, every call raises
(there is no CPU fallback).  Build it with ``ceregraphs_gb300.build.build()``
or ``__graft_entry__.build()``.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

CG_OK = 0
CG_ERR_INVALID_ARG = 1
CG_ERR_OUT_OF_MEMORY = 2
CG_ERR_CUDA = 3
CG_ERR_LEVEL_CAP = 4
CG_ERR_TIMEOUT = 5
CG_ERR_NOT_SUPPORTED = 6
CG_ERR_ADMISSION = 7
CG_ERR_PARSE = 8
CG_ERR_IO = 9

CG_EDGES_SYMMETRIZE = 1
CG_EDGES_DROP_LOOPS = 2
CG_EDGES_DETECT_SYMMETRIC = 4

CG_FORMAT_MTX = 1
CG_FORMAT_EDGELIST = 2

CG_DIR_AUTO = 0
CG_DIR_TOPDOWN = 1
CG_DIR_BOTTOMUP = 2
CG_DIR_TAU = 3
CG_PARENT_LOWEST = 0  # lowest-index in-neighbour one level up (bfs/README.md:208-224)
CG_PARENT_FIFO = 1    # scipy breadth_first_order's predecessor (run_graph500.py:383-395)

CG_GRAPH_DEVICE_PTRS = 1
CG_GRAPH_SYMMETRIC = 2

CG_ORDER_DEGREE = 1  # cg_graph_reorder: descending in-degree (util/analyze.cpp:226-372)

CG_HISTORY = 64


class CgOptions(ctypes.Structure):
  _fields_ = [("direction", ctypes.c_int32), ("alpha", ctypes.c_float),
              ("beta", ctypes.c_float), ("tau_switch_count", ctypes.c_int64),
              ("block_size", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
              ("level_cap", ctypes.c_int32), ("wait_timeout_ms", ctypes.c_int32),
              ("lane_words", ctypes.c_int32), ("ms_alpha", ctypes.c_float),
              ("test_unmatched_wait", ctypes.c_int32), ("ms_history", ctypes.c_int32),
              ("parent_rule", ctypes.c_int32)]

  def as_dict(self):
    return {k: getattr(self, k) for k, _ in self._fields_}


class CgStats(ctypes.Structure):
  _fields_ = [("status", ctypes.c_int32), ("rounds", ctypes.c_int32),
              ("visited", ctypes.c_int64), ("pull_rounds", ctypes.c_int32),
              ("switches", ctypes.c_int32), ("device_ms", ctypes.c_float),
              ("history_len", ctypes.c_int32),
              ("nf_history", ctypes.c_int64 * CG_HISTORY),
              ("direction_history", ctypes.c_int32 * CG_HISTORY),
              ("round_ns", ctypes.c_int64 * CG_HISTORY), ("setup_ns", ctypes.c_int64),
              ("finish_ns", ctypes.c_int64)]

  def as_dict(self):
    h = self.history_len
    return {"status": self.status, "rounds": self.rounds, "visited": self.visited,
            "pull_rounds": self.pull_rounds, "switches": self.switches,
            "device_ms": self.device_ms, "nf_history": list(self.nf_history[:h]),
            "direction_history": list(self.direction_history[:h]),
            "round_ns": list(self.round_ns[:h]), "setup_ns": self.setup_ns,
            "finish_ns": self.finish_ns}


class CgEdgeList(ctypes.Structure):
  _fields_ = [("n", ctypes.c_int64), ("m", ctypes.c_int64),
              ("src", ctypes.POINTER(ctypes.c_uint32)), ("dst", ctypes.POINTER(ctypes.c_uint32)),
              ("format", ctypes.c_int32), ("mtx_symmetry", ctypes.c_int32)]


CG_CHECK_NAMES = ("root", "tree", "edges", "span", "tree_edge", "lowest")


class CgValidation(ctypes.Structure):
  _fields_ = [("failures", ctypes.c_int64 * 6), ("first", ctypes.c_int64 * 6)]

  def as_dict(self):
    return {name: {"failures": int(self.failures[i]), "first": int(self.first[i])}
            for i, name in enumerate(CG_CHECK_NAMES)}

  def ok(self, lowest=True):
    return all(self.failures[i] == 0 for i in range(6) if lowest or i != 5)


class CgError(RuntimeError):
  def __init__(self, status, what=""):
    self.status = status
    msg = f"{what}: {strerror(status)} ({status})"
    detail = last_error_string()
    if status in (CG_ERR_CUDA, CG_ERR_PARSE, CG_ERR_IO, CG_ERR_NOT_SUPPORTED) and detail:
      msg += f" -- {detail}"
    super().__init__(msg)


# Every symbol declared in include/ceregraphs.h, with its ctypes signature.
_P = ctypes.c_void_p
_I64P = ctypes.POINTER(ctypes.c_int64)
SIGNATURES = {
    "cg_version": ([], ctypes.c_int),
    "cg_strerror": ([ctypes.c_int], ctypes.c_char_p),
    "cg_last_error_string": ([], ctypes.c_char_p),
    "cg_default_options": ([ctypes.POINTER(CgOptions)], None),
    "cg_graph_create": ([ctypes.c_int64, ctypes.c_int64, _P, _P, _P, _P, ctypes.c_int32,
                         ctypes.POINTER(_P)], ctypes.c_int),
    "cg_graph_destroy": ([_P], ctypes.c_int),
    "cg_graph_set_options": ([_P, ctypes.POINTER(CgOptions)], ctypes.c_int),
    "cg_graph_get_options": ([_P, ctypes.POINTER(CgOptions)], ctypes.c_int),
    "cg_graph_info": ([_P, _I64P, _I64P, ctypes.POINTER(ctypes.c_int32), _I64P], ctypes.c_int),
    "cg_graph_stream": ([_P], _P),
    "cg_bfs": ([_P, ctypes.c_int64, _P, _P, ctypes.POINTER(CgStats)], ctypes.c_int),
    "cg_bfs_device": ([_P, ctypes.c_int64, _P, _P], ctypes.c_int),
    "cg_graph_last_stats": ([_P, ctypes.POINTER(CgStats)], ctypes.c_int),
    "cg_msbfs": ([_P, _P, ctypes.c_int32, _P, _P, ctypes.POINTER(CgStats)], ctypes.c_int),
    "cg_msbfs_device": ([_P, _P, ctypes.c_int32, _P, _P], ctypes.c_int),
    "cg_count_edges": ([_P, _P, ctypes.c_int32, _I64P], ctypes.c_int),
    "cg_host_alloc": ([ctypes.POINTER(_P), ctypes.c_int64], ctypes.c_int),
    "cg_host_free": ([_P], ctypes.c_int),
    "cg_rmat_edges": ([ctypes.c_int32, ctypes.c_int64, _P, _P, _P, _P, _P], ctypes.c_int),
    "cg_uniform_bits": ([_P, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int32, _P, _P],
                        ctypes.c_int),
    "cg_graph_from_edges": ([ctypes.c_int64, ctypes.c_int64, _P, _P, ctypes.c_int32,
                             ctypes.POINTER(_P)], ctypes.c_int),
    "cg_graph_export": ([_P, _P, _P, _P, _P], ctypes.c_int),
    "cg_graph_reorder": ([_P, ctypes.c_int32, ctypes.POINTER(_P)], ctypes.c_int),
    "cg_parse_edges": ([ctypes.c_char_p, ctypes.c_int64, ctypes.c_int32,
                        ctypes.POINTER(CgEdgeList)], ctypes.c_int),
    "cg_edge_list_free": ([ctypes.POINTER(CgEdgeList)], ctypes.c_int),
    "cg_graph_from_text": ([ctypes.c_char_p, ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(_P)],
                           ctypes.c_int),
    "cg_graph_load": ([ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(_P)], ctypes.c_int),
    "cg_validate_device": ([_P, _P, ctypes.c_int32, _P, _P, ctypes.POINTER(CgValidation)],
                           ctypes.c_int),
    "cg_bfs_noalloc": ([ctypes.c_int64, ctypes.c_int64, _P, _P, _P, _P, ctypes.c_int64, _P, _P,
                        ctypes.POINTER(CgStats), _P], ctypes.c_int),
    "cg_pool_create": ([_P, ctypes.c_int32, ctypes.POINTER(_P)], ctypes.c_int),
    "cg_pool_destroy": ([_P], ctypes.c_int),
    "cg_pool_admit": ([_P, ctypes.c_int64, _P, _P, ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
    "cg_pool_step": ([_P, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64),
                      ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
    "cg_pool_release": ([_P, ctypes.c_int32], ctypes.c_int),
    "cg_pool_info": ([_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)],
                     ctypes.c_int),
    "cg_capture_begin": ([_P], ctypes.c_int),
    "cg_capture_end": ([_P, ctypes.POINTER(_P)], ctypes.c_int),
    "cg_exec_launch": ([_P], ctypes.c_int),
    "cg_exec_destroy": ([_P], ctypes.c_int),
}

_lib = None


def library_path():
  return _build.LIB


def load():
  """Load the engine library.  Raises if it has not been built."""
  global _lib
  if _lib is not None:
    return _lib
  path = _build.LIB
  if not os.path.exists(path):
    raise RuntimeError(f"CereGraphs-GB300 CUDA library not built ({path}); run "
                       "`python -c 'import __graft_entry__ as g; g.build()'`")
  lib = ctypes.CDLL(path)
  for name, (argtypes, restype) in SIGNATURES.items():
    fn = getattr(lib, name)
    fn.argtypes = argtypes
    fn.restype = restype
  _lib = lib
  return lib


def strerror(status):
  if _lib is None:
    return f"status {status}"
  return _lib.cg_strerror(status).decode()


def last_error_string():
  if _lib is None:
    return ""
  return _lib.cg_last_error_string().decode()


def check(status, what):
  if status != CG_OK:
    raise CgError(status, what)
  return status


def default_options():
  opt = CgOptions()
  load().cg_default_options(ctypes.byref(opt))
  return opt
