import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
  sys.path.insert(0, ROOT)


def pytest_configure(config):
  config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
  """The engine library, compiled in-tree if stale (nvcc runs without a GPU)."""
  from ceregraphs_gb300 import build
  build.build()
  from ceregraphs_gb300 import _lib
  return _lib.load()


@pytest.fixture(scope="session")
def oracle_mod():
  from oracle import oracle
  oracle.build()
  return oracle
