"""The no-allocation entry point, ghmm_forward_pairs_noalloc, against the existing entry points.

Callers that cannot allocate GPU memory (code inside another framework's memory pool or a fixed device
budget) keep their reads and haplotypes in device memory they already own and call
ghmm_forward_pairs_noalloc, whose scratch is a static device array.  Here the test itself allocates the
device inputs and the output (with torch), calls the entry point twice in a row through the C-ABI, and
checks each result against the existing entry points on the same pairs: the FP64 batch path within the
FP64 tolerance of the other tests (1e-9) and the default FP32 + FP64-rerun path within 1e-3.
"""
import ctypes

import numpy as np
import pytest

from gatk_gb300 import native, workload as W
from gatk_gb300.pairhmm import Engine

pytestmark = pytest.mark.gpu

TOL64 = 1e-9
TOL32 = 1e-3


def _workload():
    wl0 = W.generate(0)  # 150 bp reads: two 128-row strips per read
    rng = np.random.default_rng(23)
    regions = [([wl0.hap(h) for h in range(wl0.n_haps)], [wl0.read(r) for r in range(wl0.n_reads)])]
    for R, H in ((60, 90), (400, 700), (700, 2048), (128, 128), (129, 40)):
        base = rng.choice(list(b"ACGT"), size=H).astype(np.uint8)
        hap2 = base.copy()
        hap2[H // 2] = ord("A") if hap2[H // 2] != ord("A") else ord("C")
        reads = []
        for _ in range(3):
            start = int(rng.integers(0, max(1, H - R + 1)))
            rd = np.concatenate([base[start:start + R], rng.choice(list(b"ACGT"), size=max(0, R - H)).astype(np.uint8)])
            rd = rd[:R].copy()
            reads.append((rd, rng.integers(15, 41, size=R), np.full(R, 45), np.full(R, 45), np.full(R, 10)))
        regions.append(([base.tobytes(), hap2.tobytes()], reads))
    return W.from_pairs(regions)


def _absdiff(a, b):
    same_inf = np.isinf(a) & np.isinf(b) & (a == b)
    with np.errstate(invalid="ignore"):
        d = np.where(same_inf, 0.0, np.abs(a - b))
    assert not np.isnan(d).any()
    return d


def test_noalloc_entry_point_matches_existing_entry_points():
    torch = pytest.importorskip("torch")
    wl = _workload()
    eng = Engine()
    try:
        with eng.batch(wl) as b:
            b.forward(native.MODE_FP64)
            ref64 = b.results()
            b.forward(native.MODE_FP32_RERUN)
            ref32 = b.results()
    finally:
        eng.close()
    pr, ph = wl.pair_index()
    dev = torch.device("cuda:0")
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).astype(dt)).to(dev)
    planes = [t(x, np.uint8) for x in (wl.bases, wl.quals, wl.ins, wl.dels, wl.gcp)]
    read_off = t(wl.read_off, np.int64)
    hap_bases = t(wl.hap_bases, np.uint8)
    hap_off = t(wl.hap_off, np.int64)
    pair_read = t(pr, np.int32)
    pair_hap = t(ph, np.int32)
    out = torch.empty(len(pr), dtype=torch.float64, device=dev)
    dp = native.DevPairs(*[x.data_ptr() for x in planes], read_off.data_ptr(), hap_bases.data_ptr(),
                         hap_off.data_ptr(), pair_read.data_ptr(), pair_hap.data_ptr(), len(pr),
                         int(wl.hap_lengths().max()), 0)
    L = native.lib()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        out.fill_(float("nan"))
        rc = L.ghmm_forward_pairs_noalloc(0, ctypes.byref(dp), out.data_ptr(), stream)
        assert rc == native.GHMM_OK, native.last_error(None)
        torch.cuda.synchronize(dev)
        got = out.cpu().numpy()
        assert _absdiff(got, ref64).max() <= TOL64, call
        assert _absdiff(got, ref32).max() <= TOL32, call

    # sizes beyond the static scratch bound are rejected with a clear error
    dp.max_hap_len = native.NOALLOC_MAX_HAP_LEN + 1
    rc = L.ghmm_forward_pairs_noalloc(0, ctypes.byref(dp), out.data_ptr(), stream)
    assert rc == native.GHMM_ERR_ARG
    assert "2048" in native.last_error(None)
