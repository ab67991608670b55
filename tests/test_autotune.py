"""Autotuner: fingerprints and the cache (CPU); on the GPU, tuning changes no
result and the cached choice is reused."""
import numpy as np
import pytest

from ceregraphs_gb300 import autotune, generators, graph500


def test_fingerprint_and_cache(tmp_path):
  a = generators.rmat(10, 16, 0)
  b = generators.rmat(10, 16, 1)
  assert autotune.fingerprint(a) == autotune.fingerprint(generators.rmat(10, 16, 0))
  assert autotune.fingerprint(a) != autotune.fingerprint(b)
  c = autotune.Cache(str(tmp_path / "t.json"))
  c.put("k", {"options": {"alpha": 8.0}})
  assert autotune.Cache(str(tmp_path / "t.json")).get("k") == {"options": {"alpha": 8.0}}


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["per_root", "batched"])
def test_tuning_keeps_results_and_caches(built_lib, oracle_mod, tmp_path, mode):
  from ceregraphs_gb300.engine import Graph
  a = generators.rmat(14, 16, 2)
  roots = graph500.pick_sources(a, 64 if mode == "batched" else 4, 3)
  cache = autotune.Cache(str(tmp_path / "tune.json"))
  space = ({"alpha": [4.0, 15.0], "beta": [18.0], "block_size": [256, 512]}
           if mode == "per_root" else
           {"lane_words": [1, 2], "ms_alpha": [2.0, 8.0], "block_size": [512]})
  with Graph(a) as g:
    res = autotune.tune(g, a, roots, mode=mode, space=space, reps=1, cache=cache)
    assert not res["cached"] and np.isfinite(res["ms_per_root"])
    assert len(res["candidates"]) == 4
    opt = g.options().as_dict()
    for k, v in res["options"].items():
      assert opt[k] == pytest.approx(v)
    for r in roots[:4]:
      lv, pa, _ = g.bfs(r)
      rl, rp, _ = oracle_mod.bfs(a.in_off, a.in_idx, a.in_off, a.in_idx, r)
      assert np.array_equal(lv, rl) and np.array_equal(pa, rp)
    if mode == "batched":
      lv, pa, _ = g.msbfs(roots)
      for i, r in enumerate(roots[:8]):
        rl, rp, _ = oracle_mod.bfs(a.in_off, a.in_idx, a.in_off, a.in_idx, r)
        assert np.array_equal(lv[i], rl) and np.array_equal(pa[i], rp)
    again = autotune.tune(g, a, roots, mode=mode, space=space, reps=1, cache=cache)
    assert again["cached"] and again["options"] == res["options"]
