"""CereGraphs-GB300: level-synchronous BFS on one GB300 (sm_103a).

The search itself runs in hand-written CUDA behind the C ABI of
include/ceregraphs.h; this package is the host side that mirrors the
reference's Python drivers (device_io, preprocess_bool, bfs_timing,
run_graph500).
"""
from ._lib import CgError, CgOptions, load, library_path  # noqa: F401
from .engine import Graph, PinnedBuffer  # noqa: F401
from .preprocess import GraphArrays, from_edges  # noqa: F401

__version__ = "1.0.0"
