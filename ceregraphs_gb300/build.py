"""Builds the engine's C-ABI shared library for sm_103a with nvcc.

Each .cu file under csrc/ compiles to an object in parallel, then nvcc links
them into ceregraphs_gb300/libceregraphs_gb300.so (in-tree, git-ignored).
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libceregraphs_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def _nvcc():
  for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
    if cand and os.path.exists(cand):
      return cand
  return "nvcc"


def _sources():
  return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
  return (_sources() + glob.glob(os.path.join(CSRC, "*.cuh")) +
          glob.glob(os.path.join(INCLUDE, "*.h")) + [os.path.abspath(__file__)])


def up_to_date():
  if not os.path.exists(LIB):
    return False
  t = os.path.getmtime(LIB)
  return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False):
  """Compile (if stale) and return the library path."""
  if not force and up_to_date():
    return LIB
  os.makedirs(BUILD, exist_ok=True)
  nvcc = _nvcc()
  procs = []
  objs = []
  for src in _sources():
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    objs.append(obj)
    cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", src, "-o", obj]
    if verbose:
      print(" ".join(cmd), file=sys.stderr)
    procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
  failed = []
  for src, p in procs:
    out, _ = p.communicate()
    if p.returncode != 0:
      failed.append((src, out.decode(errors="replace")))
  if failed:
    msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
    raise RuntimeError(f"nvcc failed:\n{msg}")
  tmp = LIB + f".{os.getpid()}.tmp"
  cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
  r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
  if r.returncode != 0:
    raise RuntimeError("nvcc link failed:\n" + r.stdout.decode(errors="replace"))
  os.replace(tmp, LIB)
  return LIB


if __name__ == "__main__":
  print(build(force="--force" in sys.argv, verbose=True))
