"""CPU tests of the host side: the C-ABI library loads and exports every declared symbol, the synthetic
generator is deterministic and has the stated shapes, the product's tables equal the oracle's, and the
STR analyzer matches DragstrReadSTRAnalyzerTest's brute-force definition and empirical case."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from gatk_gb300 import native, workload as W
from oracle import oracle as O


def _declared_functions(synth: bool):
    """ghmm_* functions declared by the product headers (synth False) or by the generator's header (True)."""
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h") or (h == "ghmm_synth.h") != synth:
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"\b(ghmm_\w+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    L = native.lib()
    declared = _declared_functions(False)
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(L, name), name
    assert declared == set(native.exported_symbols())


def test_generator_lives_outside_the_product_library():
    # the synthetic generator is test and benchmark input: its own library exports it, the product does not
    S = native.synth_lib()
    declared = _declared_functions(True)
    assert declared == set(native.synth_symbols())
    for name in declared:
        assert hasattr(S, name), name
        assert not hasattr(native.lib(), name), name


def test_header_constants_match_the_bindings():
    src = open(os.path.join(ROOT, "include", "ghmm.h")).read()
    defs = dict(re.findall(r"#define (GHMM_\w+) \(?([-0-9.e]+)f?\)?", src))
    for name in ("GHMM_OK", "GHMM_ERR_ARG", "GHMM_ERR_STATE", "GHMM_ERR_CUDA", "GHMM_ERR_UNSUPPORTED",
                 "GHMM_ERR_RESULT", "GHMM_ERR_NOMEM", "GHMM_ERR_TIMEOUT"):
        assert int(defs[name]) == getattr(native, name), name
    assert int(defs["GHMM_MODE_FP32_RERUN"]) == native.MODE_FP32_RERUN
    assert int(defs["GHMM_MODE_FP64"]) == native.MODE_FP64
    assert int(defs["GHMM_MODE_PLAIN_FP64"]) == native.MODE_PLAIN_FP64
    assert int(defs["GHMM_MODE_PD"]) == native.MODE_PD
    assert int(defs["GHMM_MODE_PD_FP32"]) == native.MODE_PD_FP32
    assert float(defs["GHMM_FP64_RESCALED_FLOOR"]) == native.FP64_RESCALED_FLOOR
    sw = open(os.path.join(ROOT, "include", "ghmm_sw.h")).read()
    swd = dict(re.findall(r"#define (GHMM_\w+) \(?([-0-9]+)", sw))
    assert int(swd["GHMM_SW_SOFTCLIP"]) == native.SW_SOFTCLIP
    assert int(swd["GHMM_SW_INDEL"]) == native.SW_INDEL
    assert int(swd["GHMM_SW_LEADING_INDEL"]) == native.SW_LEADING_INDEL
    assert int(swd["GHMM_SW_IGNORE"]) == native.SW_IGNORE
    assert int(swd["GHMM_SW_SUBSTRING_SHORTCUT"]) == native.SW_SUBSTRING_SHORTCUT
    for op in "MIDS":
        assert int(swd[f"GHMM_CIGAR_{op}"]) == getattr(native, f"CIGAR_{op}")
    assert "#define GHMM_SW_MAX_LEN (1 << 20)" in sw and native.SW_MAX_LEN == 1 << 20
    assert int(swd["GHMM_SW_OPT_INT32_ONLY"]) == native.SW_OPT_INT32_ONLY


def test_struct_layouts_match_the_header(tmp_path):
    # compile the headers with the host C compiler and compare every struct's size with the ctypes mirror
    import shutil
    import subprocess

    cc = shutil.which("cc") or shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"ghmm_args": native.Args, "ghmm_read": native.Read, "ghmm_hap": native.Hap,
               "ghmm_region": native.Region, "ghmm_flat": native.Flat, "ghmm_stats": native.Stats,
               "ghmm_tuning": native.Tuning, "ghmm_queue_info": native.QueueInfo,
               "ghmm_dev_pairs": native.DevPairs, "ghmm_calib_batch": native.CalibBatch,
               "ghmm_postprocess": native.Postprocess, "ghmm_pd_hap": native.PdHap, "ghmm_pd_region": native.PdRegion,
               "ghmm_raw_read": native.RawRead, "ghmm_raw_region": native.RawRegion, "ghmm_read_prep": native.ReadPrep,
               "ghmm_pd_raw_region": native.PdRawRegion,
               "ghmm_dragstr": native.Dragstr,
               "ghmm_sw_params": native.SwParams, "ghmm_sw_pair": native.SwPair, "ghmm_sw_result": native.SwResult,
               "ghmm_sw_stats": native.SwStats}
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "ghmm.h"\n#include "ghmm_calib.h"\n#include "ghmm_sw.h"\n'
                   'int main(void) {\n' +
                   "".join(f'printf("{n} %zu\\n", sizeof({n}));\n' for n in structs) + "return 0;\n}\n")
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    sizes = dict(zip(out[0::2], map(int, out[1::2])))
    for n, cls in structs.items():
        assert sizes[n] == ctypes.sizeof(cls), n


def test_no_gpu_here_reports_unsupported():
    L = native.lib()
    if L.ghmm_load():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    a = native.Args(0, 0, 0, 0)
    assert L.ghmm_initialize(ctypes.byref(a), ctypes.byref(h)) == native.GHMM_ERR_UNSUPPORTED
    assert native.last_error(None)


def test_product_tables_equal_oracle():
    err = np.zeros(256)
    prob = np.zeros(256)
    m2m = np.zeros(128 * 128)
    p = lambda a: a.ctypes.data_as(native._f64p)
    assert native.lib().ghmm_debug_tables(None, p(err), p(prob), p(m2m)) == 0
    for q in range(255):
        assert err[q] == O.lib().oracle_qual_to_error_prob(q)
        assert prob[q] == O.lib().oracle_qual_to_prob(q)
    m2m = m2m.reshape(128, 128)
    for i in range(128):
        for j in range(128):
            assert m2m[i, j] == O.lib().oracle_match_to_match_prob(i, j), (i, j)


def test_synth_deterministic_and_shaped():
    a = W.generate(0)
    b = W.generate(0)
    for f in ("bases", "quals", "ins", "dels", "gcp", "hap_bases", "read_off", "hap_off"):
        assert np.array_equal(getattr(a, f), getattr(b, f))
    assert a.n_regions == 1 and a.n_haps == 8 and a.n_reads == 64
    assert set(a.read_lengths()) == {150}
    assert a.hap_lengths()[0] == 300
    assert a.quals.min() >= 10 and a.quals.max() <= 40
    assert set(np.unique(a.ins)) == {45} and set(np.unique(a.gcp)) == {10}
    assert set(np.unique(a.hap_bases)) <= set(b"ACGT")


def test_synth_region_ranges_compose():
    whole = W.generate(1, regions=40)
    part = W.generate(1, regions=15, region_begin=25)
    sub = whole.subset(25, 40)
    for f in ("bases", "quals", "hap_bases", "read_off", "hap_off", "region_read_off", "out_off"):
        assert np.array_equal(getattr(sub, f), getattr(part, f)), f


def test_synth_workload1_distributions():
    wl = W.generate(1, regions=300)
    nh = np.diff(wl.region_hap_off)
    nr = np.diff(wl.region_read_off)
    assert nh.min() >= 2 and nh.max() <= 32
    assert nr.min() >= 1 and nr.max() <= 1000
    assert 40 < np.median(nr) < 90  # lognormal(4,1): median e^4 = 54.6
    rl = wl.read_lengths()
    assert rl.min() >= 100 and rl.max() <= 250


def test_synth_workload2_and_3_shapes():
    w2 = W.generate(2, regions=5)
    assert w2.read_lengths().min() >= 800 and w2.read_lengths().max() <= 2000
    assert w2.quals.min() >= 5 and w2.quals.max() <= 25
    assert w2.ins.min() >= 20 and w2.ins.max() <= 45
    w3 = W.generate(3)
    assert w3.n_regions == 512 and w3.n_reads == 4096 and w3.n_pairs == 4096
    assert set(w3.hap_lengths()) == {300} and set(w3.read_lengths()) == {150}


# ---- DRAGstr STR analyzer ----
def _brute_repeats(seq: bytes, pos: int, period: int) -> int:
    """DragstrReadSTRAnalyzerTest.calculateExpectedRepeatLength (DragstrReadSTRAnalyzerTest.java:131-168)."""
    n = len(seq)
    if period > n:
        return 0
    start = max(0, pos - period + 1)
    best = 0
    while start <= pos + 1 and start + period <= n:
        unit = seq[start:start + period]
        fwd = 1
        off = start + period
        while off <= n - period and seq[off:off + period] == unit:
            fwd += 1
            off += period
        bwd = 0
        off = start - period
        while off >= 0 and seq[off:off + period] == unit:
            bwd += 1
            off -= period
        cand = fwd + bwd
        if pos < period - 1 and start == 0:
            cand = max(1, cand - 1)
        best = max(best, cand)
        start += 1
    return best


def _analyze(seq: bytes, max_period: int):
    n = len(seq)
    a = np.frombuffer(seq, dtype=np.uint8).copy()
    bp = np.zeros(n, dtype=np.int32)
    br = np.zeros(n, dtype=np.int32)
    allr = np.zeros(max_period * n, dtype=np.int32)
    p32 = lambda x: x.ctypes.data_as(native._i32p)
    assert native.lib().ghmm_str_analyze(a.ctypes.data_as(native._u8p), n, max_period, p32(bp), p32(br), p32(allr)) == 0
    return bp, br, allr.reshape(max_period, n)


def test_str_empirical_case():
    # DragstrReadSTRAnalyzerTest.java:61-66 (hex digits, repeats capped at 20)
    seq = b"ATTTTTTCAATGTTTACACATTTCCTTCCTCCCTCCCTCCTTCCTTTCCTCCCTTCCTCCCTTCCTCCCTTCCTTCCTGTTTGCTTTATTATTGTATTG"
    periods = ("1 1 1 1 1 1 1 1 1 1 1 1 1 1 1 2 2 2 2 1 1 1 1 1 1 1 4 4 4 1 1 1 1 1 1 1 1 4 4 4 1 1 1 1 1 1 1 8 8 1 1 1 1 "
               "8 8 8 8 1 1 1 1 8 8 8 8 1 1 1 1 8 8 8 8 8 1 1 1 4 1 1 1 1 1 1 1 1 1 1 1 1 1 1 1 5 5 1 1 1")
    repeats = ("6 6 6 6 6 6 6 2 2 2 1 3 3 3 3 2 2 2 2 3 3 3 3 2 2 2 3 3 3 3 3 3 3 3 3 3 3 3 3 3 2 2 2 3 3 3 3 3 3 3 3 3 3 "
               "3 3 3 3 3 3 3 3 3 3 3 3 3 3 3 3 3 3 3 3 3 2 2 2 2 3 3 3 3 1 3 3 3 3 2 2 2 2 2 2 2 2 2 2 2")
    ep = [int(x, 16) for x in periods.split()]
    er = [int(x, 16) for x in repeats.split()]
    bp, br, _ = _analyze(seq, 8)
    # the reference checks positions 0..len(expected)-1 (98 of the 99 bases)
    assert list(bp[:len(ep)]) == ep
    assert [min(20, x) for x in br[:len(er)]] == er


FIXED = [b"TGATTTGCTCTGTCTGCTGCTGCTGCCTTCAGTAGGGTTGCACGCCTGGGCACGCCTGGAAT", b"AGTATACTGAT",
         b"GTCTATATATATTTTAATTAATTAATTAATTAAATATATTTTCTGCTGCCTTTTGGAT", b"AAAAA", b"A", b"ACGTAGATCTGTAGCACTATCGAGC"]


def _random_sequences(n=60, seed=131):
    # DragstrReadSTRAnalyzerTest.java:171-197 recipe (random bases with induced tandem repeats)
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        length = int(rng.integers(5, 200))
        b = bytearray(rng.choice(list(b"ACGT"), size=length).astype(np.uint8).tobytes())
        for pos in range(length):
            if rng.random() < 1.0 / length:
                ul = int(rng.integers(1, 11))
                reps = int(rng.integers(2, 12))
                unit = rng.choice(list(b"ACGT"), size=ul).astype(np.uint8).tobytes()
                off = pos
                for _r in range(reps):
                    if off >= length - ul:
                        break
                    m = min(ul, length - off)
                    b[off:off + m] = unit[:m]
                    off += ul
        out.append(bytes(b))
    return out


@pytest.mark.parametrize("seq", FIXED + _random_sequences())
def test_str_matches_bruteforce(seq):
    # DragstrReadSTRAnalyzerTest.testRepeatPeriodAndCount / testRepeatBestPeriodAndCount
    max_period = max(5, len(seq) // 4)
    bp, br, allr = _analyze(seq, max_period)
    for pos in range(len(seq)):
        exp = [_brute_repeats(seq, pos, p) for p in range(1, max_period + 1)]
        assert list(allr[:, pos]) == exp, (pos, list(allr[:, pos]), exp)
        best_p, best_r = 1, exp[0]
        for p in range(2, max_period + 1):
            if exp[p - 1] > best_r:
                best_p, best_r = p, exp[p - 1]
        assert (bp[pos], br[pos]) == (best_p, best_r)


def _pipeline_cuts(cells):
    """The library's chunk rule restated: below 5e11 cells, cuts where the running sum first reaches 1/8 and 1/2 of
    the total; from 5e11, chunks of 1/16 of the cells growing 2.5 times up to 1/3; no cut leaves fewer than 8 regions
    behind it."""
    G, total, cut = len(cells), int(sum(cells)), [0]
    if total < 500_000_000_000:
        marks, c, m = (total // 8, total // 2), 0, 0
        for g in range(G):
            if m >= 2:
                break
            c += int(cells[g])
            if c >= marks[m] and G - g - 1 >= 8:
                cut.append(g + 1)
                m += 1
        return cut + [G]
    target, g0 = max(total // 16, 1), 0
    while g0 < G:
        g1, c = g0, 0
        while g1 < G and (c < target or g1 == g0):
            c += int(cells[g1])
            g1 += 1
        if G - g1 < 8:
            g1 = G
        cut.append(g1)
        target = min(target * 5 // 2, max(total // 3, 1))
        g0 = g1
    return cut


def _library_cuts(cells):
    cells = np.ascontiguousarray(cells, dtype=np.int64)
    out = np.zeros(len(cells) + 2, dtype=np.int64)
    n = ctypes.c_int64(0)
    p = ctypes.POINTER(ctypes.c_int64)
    rc = native.lib().ghmm_debug_pipeline_cuts(cells.ctypes.data_as(p), len(cells), out.ctypes.data_as(p), len(out),
                                               ctypes.byref(n))
    assert rc == 0
    return out[: n.value].tolist()


def test_pipeline_cuts_of_a_pipelined_call():
    # three chunks at 1/8 and 1/2 of the cells below 5e11; growing chunks above; no cut with fewer than 8 regions after
    assert _library_cuts([10**8] * 1000) == [0, 125, 500, 1000]
    assert _library_cuts([10**8] * 12) == [0, 2, 12]  # the 1/2 cut would leave 6 regions
    assert _library_cuts([10**8] * 10000) == [0, 625, 2188, 5522, 8856, 10000]
    assert _library_cuts([10**8] * 5) == [0, 5]
    wl_cells = W.generate(1, regions=1000).cells_per_region()
    cuts = _library_cuts(wl_cells)
    assert len(cuts) == 4 and wl_cells[: cuts[1]].sum() >= wl_cells.sum() // 8
    rng = np.random.default_rng(5)
    for _ in range(200):
        G = int(rng.integers(1, 3000))
        scale = 10 ** int(rng.integers(6, 11))
        cells = rng.integers(0, 4, size=G) * rng.integers(1, 1000, size=G) * scale
        got = _library_cuts(cells)
        assert got == _pipeline_cuts(cells)
        assert got[0] == 0 and got[-1] == G and all(a < b for a, b in zip(got, got[1:]))
        assert all(G - c >= 8 for c in got[1:-1])


def test_pipeline_cuts_arguments():
    p = ctypes.POINTER(ctypes.c_int64)
    cells = np.array([5, -1, 7], dtype=np.int64)
    out = np.zeros(8, dtype=np.int64)
    n = ctypes.c_int64(0)
    L = native.lib()
    assert L.ghmm_debug_pipeline_cuts(cells.ctypes.data_as(p), 3, out.ctypes.data_as(p), 8, ctypes.byref(n)) != 0
    cells = np.full(1000, 10**8, dtype=np.int64)
    assert L.ghmm_debug_pipeline_cuts(cells.ctypes.data_as(p), 1000, out.ctypes.data_as(p), 2, ctypes.byref(n)) == 0
    assert n.value == 4 and out[:2].tolist() == [0, 125] and out[2] == 0  # the count of all, the first cap written
