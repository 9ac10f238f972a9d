"""Autotuner front end: sampling, workload signatures and the on-disk cache (CPU), and the native search
(GPU)."""
import json

import numpy as np
import pytest

from gatk_gb300 import autotune as A
from gatk_gb300 import workload as W


def _same(a, b):
    for k in ("region_read_off", "region_hap_off", "read_off", "bases", "quals", "ins", "dels", "gcp", "hap_off",
              "hap_bases", "out_off"):
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)


def test_concat_of_subsets_is_the_workload():
    wl = W.generate(1, regions=25)
    parts = [wl.subset(0, 7), wl.subset(7, 8), wl.subset(8, 25)]
    _same(A.concat(parts), wl)


def test_sample_spreads_over_regions_and_keeps_small_workloads():
    wl = W.generate(1, regions=200)
    small = A.sample(wl, cells=1e18)
    assert small is wl
    s = A.sample(wl, cells=wl.cells_per_region().sum() / 10)
    assert 5 <= s.n_regions <= 40
    # every sampled region is one of the workload's regions, in order
    assert s.n_pairs > 0 and int(s.cells_per_region().sum()) < int(wl.cells_per_region().sum())


def test_signature_is_stable_and_shape_sensitive():
    a = A.workload_signature(W.generate(1, regions=300))
    b = A.workload_signature(W.generate(1, regions=300))
    c = A.workload_signature(W.generate(2, regions=20))
    assert a == b and a != c


class _FakeEngine:
    double_precision = False

    def __init__(self):
        self.set = None

    def set_tuning(self, *t):
        self.set = t


def test_cache_hit_sets_the_stored_tuning(tmp_path, monkeypatch):
    wl = W.generate(1, regions=50)
    path = str(tmp_path / "tuning.json")
    monkeypatch.setattr(A, "_device_id", lambda d: "fake-gpu")
    key = f"fake-gpu|{A._library_id()}|{A.workload_signature(wl)}|fp32"
    with open(path, "w") as f:
        json.dump({key: {"max_rows_per_lane": 6, "max_rows_per_lane_multi": 4, "chunk_cols": 4096}}, f)
    e = _FakeEngine()
    t = A.autotune(e, wl, path=path)
    assert t["cached"] and e.set == (6, 4, 4096)


@pytest.mark.gpu
def test_native_search_picks_a_candidate_and_keeps_results(engine, tmp_path):
    wl = W.generate(1, regions=300)
    cands = [(8, 8, 16384), (4, 4, 4096), (6, 8, 16384)]
    base = engine.compute(wl)
    try:
        t = engine.autotune(wl, candidates=cands, path=str(tmp_path / "t.json"))
        assert not t["cached"]
        assert (t["max_rows_per_lane"], t["max_rows_per_lane_multi"], t["chunk_cols"]) in cands
        assert engine.get_tuning() == (t["max_rows_per_lane"], t["max_rows_per_lane_multi"], t["chunk_cols"])
        assert all(m > 0 for m in t["ms"].values()) and len(t["ms"]) == 3
        tuned = engine.compute(wl)
        assert np.abs(tuned - base).max() <= 1e-3
        t2 = engine.autotune(wl, candidates=cands, path=str(tmp_path / "t.json"))
        assert t2["cached"]
    finally:
        engine.set_tuning(0, 0, 0)
