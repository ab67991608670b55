"""Pins the oracle to the reference: every check compares oracle/oracle.py or
oracle/bfs_oracle.c with fixtures produced by the reference's own modules
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest
from scipy import sparse

from golden_data import arrays, csr_from, golden, sha

G = golden()
ARR = arrays()


@pytest.mark.parametrize("key", ["s8_e16_seed0", "s10_e16_seed0", "s12_e16_seed0",
                                 "s12_e4_seed0", "s14_e16_seed3"])
def test_oracle_rmat_matches_reference_generator(oracle_mod, key):
  g = G["graphs"][key]
  A = oracle_mod.rmat(g["scale"], g["edgefactor"], g["seed"])
  assert A.shape == (g["n"], g["n"])
  assert A.nnz == g["nnz"]
  assert sha(A.indptr.astype(np.int64)) == g["indptr_sha"]
  assert sha(A.indices.astype(np.int32)) == g["indices_sha"]
  deg = np.diff(A.indptr)
  assert deg.max() == g["max_degree"]
  assert int(np.sum(deg == 0)) == g["isolated"]


def _graph(oracle_mod, key):
  g = G["graphs"][key]
  return oracle_mod.rmat(g["scale"], g["edgefactor"], g["seed"])


@pytest.mark.parametrize("key", ["s10_e16_seed0", "s12_e16_seed0", "s12_e4_seed0"])
def test_oracle_bfs_matches_reference_search(oracle_mod, key):
  A = _graph(oracle_mod, key)
  for rec in G["searches"][key]:
    r = rec["source"]
    lv, pa, rounds = oracle_mod.bfs_csr(A, r)
    assert np.array_equal(lv, ARR[f"{key}_r{r}_levels"])
    assert np.array_equal(pa, ARR[f"{key}_r{r}_parents"])
    assert sha(lv) == rec["levels_sha"] and sha(pa) == rec["parents_sha"]
    assert rounds == rec["rounds"]
    assert int((lv >= 0).sum()) == rec["visited"]
    assert oracle_mod.compute_m(A, lv >= 0, True) == rec["m"]
    assert oracle_mod.count_m(A.indptr, A.indices, lv, True) == rec["m"]
    # the independent numpy derivation agrees with the C restatement
    sl, _, _ = oracle_mod.scipy_bfs(A, r)
    assert np.array_equal(sl, lv)
    assert np.array_equal(oracle_mod.min_parents(A, sl, r), pa)
    assert oracle_mod.graph500_validate(A, r, lv, pa) == []


def test_oracle_bfs_s16_hashes(oracle_mod):
  A = _graph(oracle_mod, "s16_e16_seed0")
  for rec in G["searches"]["s16_e16_seed0"]:
    lv, pa, rounds = oracle_mod.bfs_csr(A, rec["source"])
    assert sha(lv) == rec["levels_sha"]
    assert sha(pa) == rec["parents_sha"]
    assert rounds == rec["rounds"]
    assert oracle_mod.count_m(A.indptr, A.indices, lv, True) == rec["m"]


def test_oracle_directed_with_self_loops(oracle_mod):
  n = 600
  D = csr_from(ARR["dir600_indptr"], ARR["dir600_indices"], n)
  for rec in G["searches"]["dir600"]:
    r = rec["source"]
    lv, pa, rounds = oracle_mod.bfs_csr(D, r)
    assert np.array_equal(lv, ARR[f"dir600_r{r}_levels"])
    assert np.array_equal(pa, ARR[f"dir600_r{r}_parents"])
    assert rounds == rec["rounds"]
    assert oracle_mod.compute_m(D, lv >= 0, False) == rec["m"]
    assert oracle_mod.count_m(D.indptr, D.indices, lv, False) == rec["m"]
    assert oracle_mod.graph500_validate(D, r, lv, pa) == []


def test_oracle_pick_sources(oracle_mod):
  for key, roots in G["pick_sources"].items():
    if key.startswith("dir600"):
      A = csr_from(ARR["dir600_indptr"], ARR["dir600_indices"], 600)
      k, seed = 6, 7
    else:
      gk, rest = key.rsplit("_k", 1)
      k, seed = (int(x) for x in rest.split("_seed"))
      A = _graph(oracle_mod, gk)
    assert oracle_mod.pick_sources(A.tocsc(), A.shape[0], k, seed) == roots


def test_oracle_harmonic_mean(oracle_mod):
  for case in G["harmonic_mean"]:
    vals = [float(v) for v in case["values"]]
    got = oracle_mod.harmonic_mean(vals)
    want = float(case["hm"])
    assert (np.isnan(got) and np.isnan(want)) or got == want


def test_oracle_invalid_parents_and_validator_catch_planted_mistakes(oracle_mod):
  A = _graph(oracle_mod, "s10_e16_seed0")
  case = G["invalid_parents"]["s10_e16_seed0_r0"]
  p = np.array(case["planted"], dtype=np.int64)
  lv = ARR["s10_e16_seed0_r0_levels"]
  assert oracle_mod.invalid_parents(p, lv >= 0, A, 0) == case["bad"]
  assert oracle_mod.graph500_validate(A, 0, lv, p) != []


def test_oracle_readback_conventions(oracle_mod):
  raw = np.array([5, 0xFFFFFFFF, 2, 0xFFFFFFFF], dtype=np.uint32)
  p = oracle_mod.extract_parent_result(raw, 4)
  assert p.tolist() == [5, -1, 2, -1]
  v = oracle_mod.derive_visited(p, 1)
  assert v.tolist() == [True, True, True, False]


def test_validator_rejects_wrong_levels(oracle_mod):
  A = _graph(oracle_mod, "s10_e16_seed0")
  lv = ARR["s10_e16_seed0_r0_levels"].copy()
  pa = ARR["s10_e16_seed0_r0_parents"].copy()
  v = int(np.nonzero(lv == 2)[0][0])
  lv[v] = 3
  assert oracle_mod.graph500_validate(A, 0, lv, pa) != []
  # a cycle: two reached vertices pointing at each other
  lv = ARR["s10_e16_seed0_r0_levels"]
  pa = ARR["s10_e16_seed0_r0_parents"].copy()
  a, b = np.nonzero(lv == 2)[0][:2]
  pa[a], pa[b] = b, a
  assert oracle_mod.graph500_validate(A, 0, lv, pa) != []
  # the isolated-root search is a one-vertex tree
  iso = np.nonzero(np.diff(A.indptr) == 0)[0][0]
  l2, p2, rounds = oracle_mod.bfs_csr(A, iso)
  assert rounds == 1 and (l2 >= 0).sum() == 1 and p2[iso] == iso
  assert oracle_mod.graph500_validate(sparse.csr_matrix(A), iso, l2, p2) == []


def test_oracle_fifo_parents_match_scipy(oracle_mod):
  """The oracle's restatement of scipy's predecessor (FIFO) rule gives the
  reference's own breadth_first_order parents, on R-MAT and on the directed
  matrix with self-loops."""
  for key in ("s10_e16_seed0", "s12_e16_seed0", "s12_e4_seed0"):
    A = _graph(oracle_mod, key)
    for rec in G["searches"][key]:
      r = rec["source"]
      lv = ARR[f"{key}_r{r}_levels"]
      fp = oracle_mod.fifo_parents(A.indptr, A.indices, lv, r)
      assert np.array_equal(fp, ARR[f"{key}_r{r}_scipy_parents"]), (key, r)
      assert sha(fp) == rec["scipy_parents_sha"]
  A = _graph(oracle_mod, "s16_e16_seed0")
  for rec in G["searches"]["s16_e16_seed0"]:
    lv, _, _ = oracle_mod.bfs_csr(A, rec["source"])
    assert sha(oracle_mod.fifo_parents(A.indptr, A.indices, lv, rec["source"])) == \
        rec["scipy_parents_sha"]
  D = csr_from(ARR["dir600_indptr"], ARR["dir600_indices"], 600)
  for rec in G["searches"]["dir600"]:
    r = rec["source"]
    fp = oracle_mod.fifo_parents(D.indptr, D.indices, ARR[f"dir600_r{r}_levels"], r)
    assert np.array_equal(fp, ARR[f"dir600_r{r}_scipy_parents"])
    assert oracle_mod.graph500_validate(D, r, ARR[f"dir600_r{r}_levels"], fp) == []


@pytest.mark.parametrize("seed", range(12))
def test_oracle_against_scipy_on_random_graphs(oracle_mod, seed):
  """Seeded random graphs (directed and symmetric, with self-loops, isolated
  vertices and several components): the C restatement's levels, the
  lowest-index parents and the FIFO restatement all equal what scipy's
  breadth_first_order (the reference's host search) gives."""
  rng = np.random.default_rng(1000 + seed)
  n = int(rng.integers(20, 400))
  e = int(rng.integers(n // 2, 4 * n))
  src = rng.integers(0, n, e)
  dst = rng.integers(0, n, e)
  if seed % 2:
    src, dst = np.concatenate([src, dst]), np.concatenate([dst, src])
  A = sparse.coo_matrix((np.ones(len(src)), (dst, src)), shape=(n, n)).tocsr()
  A.sum_duplicates()
  A.data[:] = 1.0
  A.sort_indices()
  for r in rng.choice(n, size=4, replace=False):
    r = int(r)
    lv, pa, rounds = oracle_mod.bfs_csr(A, r)
    sl, sp, _ = oracle_mod.scipy_bfs(A, r)
    assert np.array_equal(lv, sl)
    assert np.array_equal(pa, oracle_mod.min_parents(A, sl, r))
    assert np.array_equal(oracle_mod.fifo_parents(A.indptr, A.indices, sl, r),
                          sp.astype(np.int32))
    assert oracle_mod.graph500_validate(A, r, lv, pa) == []
