"""Several devices from one caller, and multi-rank host logic, on CPU.

The library's split (ghmm_multi_plan, the split ghmm_multi_compute_regions applies) cuts a call's reads, numbered in
region order, into one contiguous range per device of about equal cells; each range owns a contiguous slice of the
read-major output.  Checked here without a GPU: the slices tile the reads and the output exactly once and balance the
cells; host-only stand-in devices (GHMM_MULTI_STUB_DEVICES) write every output exactly once through the real
multi-device call; a read range as a self-contained workload gives the oracle's results for exactly its slice; and two
gloo ranks take their strong-scaling slices, compute them and reassemble the whole result with no data-path
collective beyond the final check, reducing timings (max) and cells (sum) the way bench.py does under torchrun.
"""
import ctypes
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT
from gatk_gb300 import native, sharding, workload as W
from oracle import oracle as O


def _random_workload(seed, n_regions=40):
    rng = np.random.default_rng(seed)
    regions = []
    for g in range(n_regions):
        nh = int(rng.integers(0, 5)) if g % 7 else 0  # some regions without haplotypes
        nr = int(rng.integers(0, 30)) if g % 5 else 0  # and some without reads
        haps = [bytes(rng.choice(list(b"ACGT"), size=int(rng.integers(20, 90))).astype(np.uint8)) for _ in range(nh)]
        reads = []
        for _ in range(nr):
            n = int(rng.integers(5, 60))
            reads.append((bytes(rng.choice(list(b"ACGT"), size=n).astype(np.uint8)), rng.integers(10, 41, size=n), np.full(n, 45),
                          np.full(n, 45), np.full(n, 10)))
        regions.append((haps, reads))
    return W.from_pairs(regions)


def _read_cells(wl):
    hl = np.concatenate([[0], np.cumsum(wl.hap_lengths())])
    per_region = hl[wl.region_hap_off[1:]] - hl[wl.region_hap_off[:-1]]
    region_of = np.repeat(np.arange(wl.n_regions), np.diff(wl.region_read_off))
    return wl.read_lengths() * per_region[region_of]


@pytest.mark.parametrize("devices", [1, 2, 3, 8, 50])
def test_plan_tiles_reads_and_output_and_balances_cells(devices):
    wl = _random_workload(devices)
    sl = sharding.read_slices(wl, devices)
    assert sl[0]["read_begin"] == 0 and sl[0]["out_begin"] == 0
    assert sl[-1]["read_end"] == wl.n_reads and sl[-1]["out_end"] == wl.n_pairs
    for a, b in zip(sl, sl[1:]):
        assert a["read_end"] == b["read_begin"] and a["out_end"] == b["out_begin"]
    cost = _read_cells(wl)
    assert sum(s["cells"] for s in sl) == int(cost.sum())
    for s in sl:
        assert s["cells"] == int(cost[s["read_begin"]:s["read_end"]].sum())
        assert s["read_begin"] <= s["read_end"]
    # every slice within one read's cells of the equal share
    share = cost.sum() / devices
    assert all(abs(s["cells"] - share) <= cost.max() for s in sl)


def test_read_slices_as_workloads_give_their_output_slices():
    wl = _random_workload(11)
    full = O.compute_workload(wl)
    got = np.full(wl.n_pairs, np.nan)
    for s in sharding.read_slices(wl, 3):
        sub = wl.read_slice(s["read_begin"], s["read_end"])
        assert sub.n_pairs == s["out_end"] - s["out_begin"]
        got[s["out_begin"]:s["out_end"]] = O.compute_workload(sub)
    assert np.array_equal(got, full)


_STUB = r"""
import ctypes, os, sys
sys.path.insert(0, sys.argv[1])
os.environ["GHMM_MULTI_STUB_DEVICES"] = "1"
import numpy as np
from gatk_gb300 import native, sharding
from gatk_gb300.pairhmm import MultiEngine
sys.path.insert(0, os.path.join(sys.argv[1], "tests"))
from test_distributed import _random_workload
wl = _random_workload(5, 60)
for n in (1, 2, 5):
    with MultiEngine([0] * n) as m:
        out = np.zeros(wl.n_pairs)
        m.compute(wl, out)
    want = np.zeros(wl.n_pairs)
    for d, s in enumerate(sharding.read_slices(wl, n)):
        want[s["out_begin"]:s["out_end"]] -= d + 1
    assert np.array_equal(out, want), n
    assert set(np.unique(out)) <= set(-np.arange(1, n + 1, dtype=float)), n
print("stub ok")
"""


def test_stub_devices_write_every_output_once():
    # the real ghmm_multi_compute_regions, with host-only stand-ins for the devices (no GPU needed)
    r = subprocess.run([sys.executable, "-c", _STUB, ROOT], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "stub ok" in r.stdout


def test_multi_device_argument_errors():
    L = native.lib()
    h = ctypes.c_void_p()
    devs = (ctypes.c_int32 * 2)(0, 0)
    a = native.Args(0, 0, 0, 0)
    assert L.ghmm_multi_create(devs, 0, ctypes.byref(a), ctypes.byref(h)) == native.GHMM_ERR_ARG
    assert L.ghmm_multi_create(None, 2, ctypes.byref(a), ctypes.byref(h)) == native.GHMM_ERR_ARG
    sl = (native.MultiSlice * 2)()
    assert L.ghmm_multi_plan(None, 3, 2, sl) == native.GHMM_ERR_ARG  # regions missing
    assert L.ghmm_multi_plan(None, 0, 0, sl) == native.GHMM_ERR_ARG  # no device
    assert L.ghmm_multi_plan(None, 0, 2, sl) == native.GHMM_OK       # nothing to split
    assert [(s.read_begin, s.read_end, s.out_begin, s.out_end) for s in sl] == [(0, 0, 0, 0)] * 2
    assert L.ghmm_multi_compute_regions(None, None, 0, None) == native.GHMM_ERR_STATE
    assert L.ghmm_multi_destroy(None) == native.GHMM_OK
    if not L.ghmm_load():  # without a usable GPU the real devices cannot be opened
        assert L.ghmm_multi_create(devs, 2, ctypes.byref(a), ctypes.byref(h)) == native.GHMM_ERR_UNSUPPORTED


def test_block_range_is_disjoint():
    assert sharding.block_range(10000, 0) == (0, 10000)
    assert sharding.block_range(10000, 3) == (30000, 40000)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from gatk_gb300 import sharding as S

        wl = _random_workload(21, 50)
        s = S.read_slices(wl, world)[rank]  # strong scaling: this rank's share of the one workload
        mine = O.compute_workload(wl.read_slice(s["read_begin"], s["read_end"]))
        local_ms = 10.0 + rank  # rank 1 is the slower one
        total = S.reduce_sum(float(s["cells"]))
        slowest = S.reduce_max(local_ms)
        q.put((rank, s["out_begin"], s["out_end"], mine.tolist(), total, slowest))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_compute_and_reduce():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    wl = _random_workload(21, 50)
    full = O.compute_workload(wl)
    got = np.full(wl.n_pairs, np.nan)
    covered = np.zeros(wl.n_pairs, dtype=int)
    for _, a, b, vals, _, _ in out:
        got[a:b] = vals
        covered[a:b] += 1
    assert (covered == 1).all()
    assert np.array_equal(got, full)
    cells = int(_read_cells(wl).sum())
    for *_, total, slowest in out:
        assert total == float(cells)
        assert slowest == 11.0


@pytest.mark.gpu
def test_two_contexts_on_one_gpu_match_one_context():
    from gatk_gb300.pairhmm import Engine, MultiEngine

    wl = W.generate(1, regions=40)
    eng = Engine()
    try:
        one = eng.compute(wl, via_regions=True)
    finally:
        eng.close()
    for devs in ([0], [0, 0], [0, 0, 0]):
        with MultiEngine(devs) as m:
            got = m.compute(wl)
        # a read's result does not depend on which reads share its warp task or its batch
        assert np.array_equal(got, one), devs
    assert np.abs(one - O.compute_workload(wl)).max() <= 1e-3
