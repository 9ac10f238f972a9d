"""The no-allocation entry point, ghmm_forward_pairs_noalloc, against the oracle and the existing entry points.

Callers that cannot allocate GPU memory (code inside another framework's memory pool or a fixed device
budget, or that must not take the synchronisation an allocation brings) keep their reads and haplotypes in
device memory they already own and call ghmm_forward_pairs_noalloc, whose scratch is a static device array.
Here the test itself allocates the device inputs and the output (with torch), calls the entry point through
the C-ABI, and checks the results directly against the FP64 oracle and against the existing entry points on
the same pairs: the FP64 batch path within the FP64 tolerance of the other tests (1e-9) and the default
FP32 + FP64-rerun path within 1e-3.  Two calls in a row must agree.  The first call of a process is made in a
fresh child process on a non-blocking stream, so the one-time table set-up is checked to land before a kernel
on such a stream reads it.  The device-side guards are exercised too: a haplotype longer than the static
scratch bound although max_hap_len promised otherwise, and penalty bytes out of range, give NaN for their
pairs only.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT
from gatk_gb300 import native, workload as W
from gatk_gb300.pairhmm import Engine
from oracle import oracle as O

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


class _Device:
    """The workload's planes and a pair list in device memory owned by the caller (torch)."""

    def __init__(self, torch, wl, pr, ph, max_hap_len):
        dev = torch.device("cuda:0")
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).astype(dt)).to(dev)
        self.keep = [t(x, np.uint8) for x in (wl.bases, wl.quals, wl.ins, wl.dels, wl.gcp)]
        self.keep += [t(wl.read_off, np.int64), t(wl.hap_bases, np.uint8), t(wl.hap_off, np.int64),
                      t(pr, np.int32), t(ph, np.int32)]
        self.out = torch.empty(len(pr), dtype=torch.float64, device=dev)
        self.pairs = native.DevPairs(*[x.data_ptr() for x in self.keep], len(pr), max_hap_len, 0)

    def call(self, stream):
        self.out.fill_(float("nan"))
        return native.lib().ghmm_forward_pairs_noalloc(0, ctypes.byref(self.pairs), self.out.data_ptr(), stream)


def test_noalloc_entry_point_matches_oracle_and_existing_entry_points():
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
    oracle = O.compute_workload(wl)
    pr, ph = wl.pair_index()
    d = _Device(torch, wl, pr, ph, int(wl.hap_lengths().max()))
    stream = torch.cuda.current_stream(torch.device("cuda:0")).cuda_stream
    for call in range(2):
        rc = d.call(stream)
        assert rc == native.GHMM_OK, native.last_error(None)
        torch.cuda.synchronize()
        got = d.out.cpu().numpy()
        assert _absdiff(got, oracle).max() <= TOL64, call
        assert _absdiff(got, ref64).max() <= TOL64, call
        assert _absdiff(got, ref32).max() <= TOL32, call

    # sizes beyond the static scratch bound are rejected with a clear error
    d.pairs.max_hap_len = native.NOALLOC_MAX_HAP_LEN + 1
    rc = d.call(stream)
    assert rc == native.GHMM_ERR_ARG
    assert "2048" in native.last_error(None)


def test_noalloc_device_guards_flag_their_pairs_only():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    long_hap = rng.choice(list(b"ACGT"), size=native.NOALLOC_MAX_HAP_LEN + 1).astype(np.uint8)
    short_hap = long_hap[:300].copy()
    reads = []
    for k in range(4):
        rd = short_hap[20 * k:20 * k + 150].copy()
        reads.append((rd, rng.integers(15, 41, size=150), np.full(150, 45), np.full(150, 45), np.full(150, 10)))
    wl = W.from_pairs([([short_hap.tobytes(), long_hap.tobytes()], reads)])
    wl.ins[wl.read_off[2] + 7] = 200  # read 2: an insertion penalty above 127 (a negative Java byte)
    pr, ph = wl.pair_index()
    # the caller promises max_hap_len = 2048, but haplotype 1 holds 2049 bases on the device
    d = _Device(torch, wl, pr, ph, native.NOALLOC_MAX_HAP_LEN)
    stream = torch.cuda.current_stream(torch.device("cuda:0")).cuda_stream
    assert d.call(stream) == native.GHMM_OK, native.last_error(None)
    torch.cuda.synchronize()
    got = d.out.cpu().numpy()
    flagged = (ph == 1) | (pr == 2)
    assert np.isnan(got[flagged]).all()
    sel = np.nonzero(~flagged)[0]
    want = O.compute_pairs(wl, pr[sel], ph[sel])
    assert _absdiff(got[sel], want).max() <= TOL64


_FIRST_CALL = r"""
import ctypes, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from gatk_gb300 import native, workload as W
from oracle import oracle as O
wl = W.generate(0)
pr, ph = wl.pair_index()
dev = torch.device("cuda:0")
t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).astype(dt)).to(dev)
keep = [t(x, np.uint8) for x in (wl.bases, wl.quals, wl.ins, wl.dels, wl.gcp)]
keep += [t(wl.read_off, np.int64), t(wl.hap_bases, np.uint8), t(wl.hap_off, np.int64), t(pr, np.int32), t(ph, np.int32)]
out = torch.full((len(pr),), float("nan"), dtype=torch.float64, device=dev)
dp = native.DevPairs(*[x.data_ptr() for x in keep], len(pr), int(wl.hap_lengths().max()), 0)
torch.cuda.synchronize()
s = torch.cuda.Stream(device=dev)  # a pool stream: created non-blocking, not ordered after the legacy stream
for call in range(2):
    rc = native.lib().ghmm_forward_pairs_noalloc(0, ctypes.byref(dp), out.data_ptr(), s.cuda_stream)
    assert rc == 0, native.last_error(None)
    s.synchronize()
    got = out.cpu().numpy()
    err = float(np.max(np.abs(got - O.compute_workload(wl))))
    assert err <= 1e-9, (call, err)
    print("first-call", call, err)
"""


def test_noalloc_first_call_on_a_non_blocking_stream_in_a_fresh_process():
    pytest.importorskip("torch")
    r = subprocess.run([sys.executable, "-c", _FIRST_CALL, ROOT], capture_output=True, text=True, timeout=600,
                       env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "first-call 1" in r.stdout
