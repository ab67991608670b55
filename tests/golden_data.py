"""Loads the committed golden fixtures (made by tests/golden/make_golden.py
from the reference's own modules)."""
import hashlib
import json
import os

import numpy as np
from scipy import sparse

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden():
  with open(os.path.join(HERE, "golden.json"), encoding="utf-8") as f:
    return json.load(f)


def arrays():
  return np.load(os.path.join(HERE, "golden_arrays.npz"))


def sha(a):
  return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def csr_from(indptr, indices, n):
  return sparse.csr_matrix((np.ones(len(indices)), np.asarray(indices, dtype=np.int32),
                            np.asarray(indptr, dtype=np.int64)), shape=(n, n))
