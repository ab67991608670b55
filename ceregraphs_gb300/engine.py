"""Python face of the C ABI: a resident graph handle and its searches.

Stands where the reference's SdkRuntime session stands in
bfs/scripts/run_graph500.py:246-375: ``Graph(...)`` is Kernel 1 (the one-time
upload), ``Graph.bfs(root)`` is one Kernel-2 search with its output read back
to host memory, ``Graph.msbfs(roots)`` runs many roots as bit lanes.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import CgOptions, CgStats, check
from .preprocess import GraphArrays, preprocess


def _ptr(a):
  """Data pointer of a numpy array or a torch tensor (host or device)."""
  if a is None:
    return None
  if hasattr(a, "data_ptr"):
    return ctypes.c_void_p(a.data_ptr())
  return a.ctypes.data_as(ctypes.c_void_p)


class PinnedBuffer:
  """Page-locked host array from cg_host_alloc (fast device->host readback)."""

  def __init__(self, shape, dtype=np.int32):
    lib = _lib.load()
    self.dtype = np.dtype(dtype)
    self.shape = tuple(np.atleast_1d(shape).tolist())
    nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
    p = ctypes.c_void_p()
    check(lib.cg_host_alloc(ctypes.byref(p), max(nbytes, 1)), "cg_host_alloc")
    self._p = p
    buf = (ctypes.c_byte * max(nbytes, 1)).from_address(p.value)
    self.array = np.frombuffer(buf, dtype=self.dtype, count=int(np.prod(self.shape)))
    self.array = self.array.reshape(self.shape)

  def free(self):
    if self._p is not None and self._p.value:
      self.array = None
      _lib.load().cg_host_free(self._p)
      self._p = None

  def __del__(self):
    try:
      self.free()
    except Exception:  # interpreter shutdown
      pass


class Exec:
  """An instantiated CUDA graph of captured searches (cg_exec)."""

  def __init__(self, handle):
    self._x = handle

  def launch(self):
    check(_lib.load().cg_exec_launch(self._x), "cg_exec_launch")

  def close(self):
    if self._x is not None and self._x.value:
      _lib.load().cg_exec_destroy(self._x)
    self._x = None

  def __del__(self):
    try:
      self.close()
    except Exception:
      pass


class Graph:
  """A graph resident in HBM (in-lists, plus out-lists when directed)."""

  def __init__(self, arrays: GraphArrays | None = None, *, A=None, device_arrays=None):
    lib = _lib.load()
    self._h = ctypes.c_void_p()
    if A is not None:
      arrays = preprocess(A)
    if device_arrays is not None:
      # (n, nnz, in_off, in_idx, out_off, out_idx, symmetric) with torch CUDA tensors
      n, nnz, io, ii, oo, oi, sym = device_arrays
      flags = _lib.CG_GRAPH_DEVICE_PTRS | (_lib.CG_GRAPH_SYMMETRIC if sym else 0)
      check(lib.cg_graph_create(int(n), int(nnz), _ptr(io), _ptr(ii), _ptr(oo), _ptr(oi), flags,
                                ctypes.byref(self._h)), "cg_graph_create")
      self.n, self.nnz, self.symmetric = int(n), int(nnz), bool(sym)
      return
    if arrays is None:
      raise ValueError("need GraphArrays, A, or device_arrays")
    a = arrays
    io = np.ascontiguousarray(a.in_off, dtype=np.int64)
    ii = np.ascontiguousarray(a.in_idx, dtype=np.int32)
    flags = _lib.CG_GRAPH_SYMMETRIC if a.symmetric else 0
    oo = oi = None
    if not a.symmetric:
      oo = np.ascontiguousarray(a.out_off, dtype=np.int64)
      oi = np.ascontiguousarray(a.out_idx, dtype=np.int32)
    check(lib.cg_graph_create(a.n, a.nnz, _ptr(io), _ptr(ii), _ptr(oo), _ptr(oi), flags,
                              ctypes.byref(self._h)), "cg_graph_create")
    self.n, self.nnz, self.symmetric = a.n, a.nnz, a.symmetric

  @classmethod
  def from_handle(cls, handle):
    """Adopt a cg_graph* made by another C-ABI call (e.g. cg_graph_from_edges)."""
    g = cls.__new__(cls)
    g._h = handle
    info = g.info()
    g.n, g.nnz, g.symmetric = info["n"], info["nnz"], info["symmetric"]
    return g

  def export(self) -> GraphArrays:
    """Copy the resident CSR (and CSC when directed) back to host arrays."""
    io = np.empty(self.n + 1, dtype=np.int64)
    ii = np.empty(self.nnz, dtype=np.int32)
    oo = oi = None
    if not self.symmetric:
      oo = np.empty(self.n + 1, dtype=np.int64)
      oi = np.empty(self.nnz, dtype=np.int32)
    check(_lib.load().cg_graph_export(self._h, _ptr(io), _ptr(ii), _ptr(oo), _ptr(oi)),
          "cg_graph_export")
    return GraphArrays(self.n, self.nnz, io, ii, oo, oi, self.symmetric)

  def reorder(self, order=_lib.CG_ORDER_DEGREE):
    """A degree-ordered resident copy for per-root searches (cg_graph_reorder):
    same roots, same outputs in original ids, vertices laid out hubs first."""
    h = ctypes.c_void_p()
    check(_lib.load().cg_graph_reorder(self._h, int(order), ctypes.byref(h)), "cg_graph_reorder")
    return Graph.from_handle(h)

  def export_offsets(self):
    """The resident CSR offsets (n + 1 int64) on the host."""
    io = np.empty(self.n + 1, dtype=np.int64)
    check(_lib.load().cg_graph_export(self._h, _ptr(io), None, None, None), "cg_graph_export")
    return io

  # -- lifecycle -----------------------------------------------------------
  def close(self):
    if self._h is not None and self._h.value:
      _lib.load().cg_graph_destroy(self._h)
    self._h = None

  def __enter__(self):
    return self

  def __exit__(self, *exc):
    self.close()

  def __del__(self):
    try:
      self.close()
    except Exception:
      pass

  @property
  def handle(self):
    return self._h

  @property
  def stream(self):
    """The handle's cudaStream_t as an int."""
    return _lib.load().cg_graph_stream(self._h) or 0

  def info(self):
    n, nnz, b = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    s = ctypes.c_int32()
    check(_lib.load().cg_graph_info(self._h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(s),
                                    ctypes.byref(b)), "cg_graph_info")
    return {"n": n.value, "nnz": nnz.value, "symmetric": bool(s.value), "device_bytes": b.value}

  # -- options ---------------------------------------------------------------
  def options(self) -> CgOptions:
    opt = CgOptions()
    check(_lib.load().cg_graph_get_options(self._h, ctypes.byref(opt)), "cg_graph_get_options")
    return opt

  def set_options(self, opt: CgOptions | None = None, **kw):
    opt = opt if opt is not None else self.options()
    for k, v in kw.items():
      if not hasattr(opt, k):
        raise AttributeError(k)
      setattr(opt, k, v)
    check(_lib.load().cg_graph_set_options(self._h, ctypes.byref(opt)), "cg_graph_set_options")
    return opt

  # -- searches --------------------------------------------------------------
  def bfs(self, root, levels=None, parents=None, want_levels=True, want_parents=True):
    """One search with host outputs (numpy int32 arrays of n).  Returns
    (levels, parents, stats)."""
    if levels is None and want_levels:
      levels = np.empty(self.n, dtype=np.int32)
    if parents is None and want_parents:
      parents = np.empty(self.n, dtype=np.int32)
    st = CgStats()
    check(_lib.load().cg_bfs(self._h, int(root), _ptr(levels), _ptr(parents), ctypes.byref(st)),
          "cg_bfs")
    return levels, parents, st.as_dict()

  def bfs_device(self, root, d_levels, d_parents):
    """Enqueue one search writing device buffers (torch tensors or raw
    pointers) on the handle's stream; does not wait."""
    lp = d_levels if isinstance(d_levels, int) else d_levels.data_ptr()
    pp = d_parents if isinstance(d_parents, int) else d_parents.data_ptr()
    check(_lib.load().cg_bfs_device(self._h, int(root), ctypes.c_void_p(lp), ctypes.c_void_p(pp)),
          "cg_bfs_device")

  def last_stats(self):
    st = CgStats()
    check(_lib.load().cg_graph_last_stats(self._h, ctypes.byref(st)), "cg_graph_last_stats")
    return st.as_dict()

  def msbfs(self, roots, levels=None, parents=None):
    """Batched search of k roots with host outputs (k x n int32 each)."""
    roots = np.ascontiguousarray(roots, dtype=np.int64)
    k = len(roots)
    if levels is None:
      levels = np.empty((k, self.n), dtype=np.int32)
    if parents is None:
      parents = np.empty((k, self.n), dtype=np.int32)
    st = CgStats()
    check(_lib.load().cg_msbfs(self._h, _ptr(roots), k, _ptr(levels), _ptr(parents),
                               ctypes.byref(st)), "cg_msbfs")
    return levels, parents, st.as_dict()

  def msbfs_device(self, roots, d_levels, d_parents):
    roots = np.ascontiguousarray(roots, dtype=np.int64)
    lp = d_levels if isinstance(d_levels, int) else d_levels.data_ptr()
    pp = d_parents if isinstance(d_parents, int) else d_parents.data_ptr()
    check(_lib.load().cg_msbfs_device(self._h, _ptr(roots), len(roots), ctypes.c_void_p(lp),
                                      ctypes.c_void_p(pp)), "cg_msbfs_device")

  def capture(self, body):
    """Record the searches that ``body()`` enqueues on this handle (the
    ``*_device`` calls) into one CUDA graph; returns an Exec to replay it."""
    lib = _lib.load()
    check(lib.cg_capture_begin(self._h), "cg_capture_begin")
    try:
      body()
    except BaseException:
      # end the capture so the stream is usable again; drop what it recorded
      x = ctypes.c_void_p()
      if lib.cg_capture_end(self._h, ctypes.byref(x)) == 0 and x.value:
        lib.cg_exec_destroy(x)
      raise
    x = ctypes.c_void_p()
    check(lib.cg_capture_end(self._h, ctypes.byref(x)), "cg_capture_end")
    return Exec(x)

  def validate(self, roots, d_levels, d_parents):
    """Graph500 tree checks on the device for searches whose outputs are
    device tensors (k x n, or n for one search).  Returns one dict per search:
    check name -> {"failures", "first"}; see cg_validate_device."""
    roots = np.ascontiguousarray(np.atleast_1d(roots), dtype=np.int64)
    k = len(roots)
    out = (_lib.CgValidation * k)()
    lp = d_levels if isinstance(d_levels, int) else d_levels.data_ptr()
    pp = d_parents if isinstance(d_parents, int) else d_parents.data_ptr()
    check(_lib.load().cg_validate_device(self._h, _ptr(roots), k, ctypes.c_void_p(lp),
                                         ctypes.c_void_p(pp), out), "cg_validate_device")
    return [out[i].as_dict() for i in range(k)]

  def count_edges(self, d_levels, k=1):
    """Graph500 m for k searches whose levels are on the device (k x n)."""
    lp = d_levels if isinstance(d_levels, int) else d_levels.data_ptr()
    out = np.zeros(k, dtype=np.int64)
    check(_lib.load().cg_count_edges(self._h, ctypes.c_void_p(lp), k,
                                     out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))),
          "cg_count_edges")
    return out
