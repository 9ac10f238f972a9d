"""The streaming queue (ghmm_queue_*) and the pipelined synchronous path, against the one-batch path.

A region's tasks (read pairing, haplotype chunks) depend only on the region, so a region gives bit-identical
results whichever batch carries it: the tests compare exactly, and a sample against the FP64 oracle.
"""
import ctypes

import numpy as np
import pytest

from gatk_gb300 import native, workload as W
from gatk_gb300.pairhmm import Engine
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _one_batch(engine, wl, mode=native.MODE_FP32_RERUN):
    with engine.batch(wl) as b:
        b.forward(mode)
        return b.results()


def test_pipelined_compute_regions_matches_one_batch(engine):
    wl = W.generate(1, regions=1500)  # about 1.6e11 cells: above the pipelining threshold of 1.5e11
    assert int(wl.cells_per_region().sum()) >= 1.5e11
    ref = _one_batch(engine, wl)
    got = engine.compute(wl, via_regions=True)
    np.testing.assert_array_equal(got, ref)
    got_flat = engine.compute(wl, via_regions=False)
    np.testing.assert_array_equal(got_flat, ref)
    # and a sample against the oracle
    sub = wl.subset(0, 3)
    o = O.compute_workload(sub)
    assert np.abs(got[: sub.n_pairs] - o).max() <= 1e-3


def test_queue_region_at_a_time_matches_one_batch(engine):
    wl = W.generate(1, regions=300)
    ref = _one_batch(engine, wl)
    with engine.queue(batch_cells=int(3e9)) as q:
        out = q.push(wl)
        q.flush()
        info = q.info()
    np.testing.assert_array_equal(out, ref)
    assert info["n_regions"] == wl.n_regions
    assert info["n_pairs"] == wl.n_pairs
    assert info["n_cells"] == int(wl.cells_per_region().sum())
    assert info["n_batches"] >= 4
    assert info["n_launches"] >= info["n_batches"]


def test_queue_long_pairs_with_reruns(engine):
    wl = W.generate(2, regions=12)
    ref = _one_batch(engine, wl)
    with engine.queue(batch_cells=int(3e9)) as q:
        out = q.push(wl)
        q.flush()
        info = q.info()
    np.testing.assert_array_equal(out, ref)
    assert info["n_rerun"] + info["n_fp64_direct"] > 0


def test_queue_destroy_delivers_without_flush(engine):
    wl = W.generate(0)
    ref = _one_batch(engine, wl)
    q = engine.queue()
    out = q.push(wl)
    q.close()  # destroy flushes the open batch
    np.testing.assert_array_equal(out, ref)


def test_queue_fp64_context():
    e = Engine(use_double_precision=True)
    try:
        wl = W.generate(1, regions=40)
        ref = _one_batch(e, wl, native.MODE_FP64)
        with e.queue(batch_cells=int(1e9)) as q:
            out = q.push(wl)
            q.flush()
            info = q.info()
        np.testing.assert_array_equal(out, ref)
        assert info["n_fp64_direct"] == wl.n_pairs
    finally:
        e.close()


def test_queue_rejects_bad_push_and_keeps_working(engine):
    wl = W.generate(0)
    ref = _one_batch(engine, wl)
    bad = W.from_pairs([([b"ACGTACGT"], [(b"ACGT", np.array([30, 30, 255, 30], np.uint8),
                                           np.full(4, 45, np.uint8), np.full(4, 45, np.uint8),
                                           np.full(4, 10, np.uint8))])])
    with engine.queue() as q:
        with pytest.raises(native.GhmmError) as ei:
            q.push(bad)
        assert ei.value.code == native.GHMM_ERR_ARG
        out = q.push(wl)
        q.flush()
        info = q.info()
    np.testing.assert_array_equal(out, ref)
    assert info["n_regions"] == wl.n_regions


def test_queue_blocks_tuning_changes(engine):
    q = engine.queue()
    try:
        with pytest.raises(native.GhmmError) as ei:
            engine.set_tuning(6, 4, 8192)
        assert ei.value.code == native.GHMM_ERR_STATE
    finally:
        q.close()
    engine.set_tuning(0, 0, 0)


def test_queue_empty_regions_and_empty_flush(engine):
    wl = W.from_pairs([([b"ACGT"], []), ([], []), ([b"ACGTTT", b"AC"], [(b"ACG", np.full(3, 30, np.uint8),
                                                                         np.full(3, 45, np.uint8),
                                                                         np.full(3, 45, np.uint8),
                                                                         np.full(3, 10, np.uint8))])])
    with engine.queue() as q:
        q.flush()  # nothing pushed
        out = q.push(wl)
        q.flush()
    ref = _one_batch(engine, wl)
    np.testing.assert_array_equal(out, ref)
