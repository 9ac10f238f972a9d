"""The PD-HMM oracle (oracle/pdhmm_oracle.c) against an independent pure-Python restatement of
LoglessPDPairHMM.subComputeReadLikelihoodGivenHaplotypeLog10 (LoglessPDPairHMM.java:35-150) on small cases, and
against the plain LoglessPairHMM oracle where no PD flag is set.  The reference's PD-HMM golden file is a git-lfs
pointer in this checkout, so these restatements are the pin."""
import math

import numpy as np
import pytest

from gatk_gb300 import workload as W
from oracle import oracle as O

SNP, DS, DE = 1, 2, 4
BIT = {ord("A"): 8, ord("C"): 16, ord("G"): 32, ord("T"): 64}


def _py_pdhmm(hap, pd, read, q, ins, dl, gcp):
    """Full-matrix transliteration (small cases only)."""
    R, H = len(read), len(hap)
    M = [[0.0] * (H + 1) for _ in range(R + 1)]
    I = [[0.0] * (H + 1) for _ in range(R + 1)]
    D = [[0.0] * (H + 1) for _ in range(R + 1)]
    bM = [[0.0] * (H + 1) for _ in range(R + 1)]
    bI = [[0.0] * (H + 1) for _ in range(R + 1)]
    bD = [[0.0] * (H + 1) for _ in range(R + 1)]
    init = 2.0 ** 1020 / H
    for j in range(H + 1):
        D[0][j] = init
    state = 0  # 0 NORMAL, 1 INSIDE_DEL, 2 AFTER_DEL
    for i in range(1, R + 1):
        t = np.zeros(6)
        O.lib().oracle_qual_to_trans_probs(t.ctypes.data_as(O._f64p), int(ins[i - 1]), int(dl[i - 1]), int(gcp[i - 1]))
        MM, IM, MI, II, MD, DD = t
        x = read[i - 1]
        for j in range(1, H + 1):
            y, f = hap[j - 1], pd[j - 1]
            pdm = bool(f & SNP) and bool(f & BIT.get(x, 0))
            m = x == y or x == ord("N") or y == ord("N") or pdm
            prior = O.lib().oracle_qual_to_prob(int(q[i - 1])) if m else O.lib().oracle_qual_to_error_prob(int(q[i - 1])) / 3.0
            if state in (0, 1):
                if state == 0:
                    bM[i][j], bD[i][j], bI[i][j] = M[i][j - 1], D[i][j - 1], I[i][j - 1]
                else:
                    bM[i][j], bD[i][j], bI[i][j] = bM[i][j - 1], bD[i][j - 1], bI[i][j - 1]
                M[i][j] = prior * (M[i - 1][j - 1] * MM + I[i - 1][j - 1] * IM + D[i - 1][j - 1] * IM)
                D[i][j] = M[i][j - 1] * MD + D[i][j - 1] * DD
            else:
                bM[i][j] = max(bM[i][j - 1], M[i][j - 1])
                bD[i][j] = max(bD[i][j - 1], D[i][j - 1])
                bI[i][j] = max(bI[i][j - 1], I[i][j - 1])
                M[i][j] = prior * (max(bM[i - 1][j - 1], M[i - 1][j - 1]) * MM + max(bI[i - 1][j - 1], I[i - 1][j - 1]) * IM
                                   + max(bD[i - 1][j - 1], D[i - 1][j - 1]) * IM)
                D[i][j] = max(bM[i][j - 1], M[i][j - 1]) * MD + max(bD[i][j - 1], D[i][j - 1]) * DD
            if f & DE:
                I[i][j] = max(bM[i - 1][j], M[i - 1][j]) * MI + max(bI[i - 1][j], I[i - 1][j]) * II
            else:
                I[i][j] = M[i - 1][j] * MI + I[i - 1][j] * II
            if state == 2:
                state = 0
            if f & DS:
                state = 1
            if f & DE:
                state = 2
    s = 0.0
    for j in range(1, H + 1):
        s += M[R][j] + I[R][j]
    return math.log10(s) - math.log10(2.0 ** 1020)


def _case(rng, H=40, R=25, n_snp=2, n_del=1, dl=(1, 6), end_flag=False):
    hap = rng.choice(list(b"ACGT"), size=H).astype(np.uint8)
    pd = np.zeros(H, dtype=np.uint8)
    for _ in range(n_snp):
        j = int(rng.integers(0, H))
        alt = [c for c in b"ACGT" if c != hap[j]][int(rng.integers(0, 3))]
        pd[j] |= SNP | BIT[alt]
    for _ in range(n_del):
        n = int(rng.integers(dl[0], dl[1] + 1))
        j = int(rng.integers(1, H - n))
        pd[j] |= DS
        pd[j + n - 1] |= DE
    if end_flag:
        pd[H - 1] |= DS if rng.integers(0, 2) else DE
    off = int(rng.integers(0, H - R + 1))
    read = hap[off:off + R].copy()
    for k in range(R):  # a few substitutions, some to the SNP alternative
        if rng.random() < 0.1:
            read[k] = rng.choice(list(b"ACGT"))
    q = rng.integers(10, 41, size=R).astype(np.uint8)
    ins = rng.integers(20, 46, size=R).astype(np.uint8)
    dls = rng.integers(20, 46, size=R).astype(np.uint8)
    g = np.full(R, 10, dtype=np.uint8)
    return hap, pd, read, q, ins, dls, g


@pytest.mark.parametrize("seed", range(12))
def test_c_oracle_matches_python_restatement(seed):
    rng = np.random.default_rng(seed)
    case = _case(rng, n_del=1 + seed % 3, end_flag=(seed % 4 == 3))
    assert O.pd_logless(*case) == _py_pdhmm(*[np.asarray(c) for c in case]) or \
        abs(O.pd_logless(*case) - _py_pdhmm(*[np.asarray(c) for c in case])) <= 1e-12


def test_without_flags_equals_plain_logless():
    wl = W.generate(0)
    plain = O.compute_workload(wl)
    pd = O.pd_compute_workload(wl, np.zeros(len(wl.hap_bases), dtype=np.uint8))
    assert np.array_equal(plain, pd)


def test_flags_change_the_likelihood_and_snp_alt_matches():
    # a read carrying the SNP alternative: the PD haplotype gives a higher likelihood than the plain one
    hap = b"ACGTACGTACGTACGTACGTAAAACCCCGGGGTTTT"
    read = bytearray(hap[5:30])
    j = 12
    read[j - 5] = ord("G") if hap[j] != ord("G") else ord("T")
    pd = np.zeros(len(hap), dtype=np.uint8)
    pd[j] = SNP | BIT[read[j - 5]]
    n = len(read)
    args = ([30] * n, [45] * n, [45] * n, [10] * n)
    with_pd = O.pd_logless(hap, pd, bytes(read), *args)
    without = O.pd_logless(hap, np.zeros(len(hap), np.uint8), bytes(read), *args)
    assert with_pd > without + 1.0


def test_unexpected_base_with_snp_flag_raises():
    hap = b"ACGTACGTACGT"
    pd = np.zeros(len(hap), dtype=np.uint8)
    pd[3] = SNP | BIT[ord("A")]
    with pytest.raises(ValueError):
        O.pd_logless(hap, pd, b"ACGRAC", [30] * 6, [45] * 6, [45] * 6, [10] * 6)


def test_synthetic_flags_are_deterministic_and_well_formed():
    wl = W.generate(1, regions=30)
    a = W.pd_flags(wl)
    b = W.pd_flags(wl)
    assert np.array_equal(a, b)
    assert (a & SNP).sum() > 0 and (a & DS).sum() > 0
    # every SNP flag names an alternative base different from the haplotype base
    snp = (a & SNP) != 0
    for k in np.nonzero(snp)[0][:200]:
        assert not (a[k] & BIT[int(wl.hap_bases[k])]) or bin(int(a[k]) >> 3).count("1") > 1


# ---------------------------------------------------------------------------------------------------------------
# The packed FP32 kernel's scheme (pd_packed.cu) on the CPU, from the library's own op bytes (ghmm_debug_pd_ops):
# branch states materialised only where an op byte asks for them, the AFTER_DEL replacement of the previous column
# by max(bX, X), the DEL_END max, and the prior of SNP columns picked from rows of the read's prior table the way the
# kernel picks it.  Unscaled FP64 in the oracle's operation order, so it must reproduce the oracle bit for bit.

def _pd_ops(hap, pd):
    from gatk_gb300 import native

    H = len(hap)
    ops, codes = np.zeros(H, dtype=np.uint8), np.zeros(H, dtype=np.uint8)
    h, f = np.ascontiguousarray(hap, dtype=np.uint8), np.ascontiguousarray(pd, dtype=np.uint8)
    rc = native.lib().ghmm_debug_pd_ops(h.ctypes.data_as(native._u8p), f.ctypes.data_as(native._u8p), H,
                                        ops.ctypes.data_as(native._u8p), codes.ctypes.data_as(native._u8p))
    assert rc in (0, 1)
    return rc == 1, ops, codes


def _lazy_branch_pdhmm(hap, read, q, ins, dl, gcp, ops, codes):
    R, H = len(read), len(hap)
    init = 2.0 ** 1020 / H
    M, I, D = [0.0] * (H + 1), [0.0] * (H + 1), [init] * (H + 1)
    B = [[0.0] * (H + 1) for _ in range(3)]  # the branch registers (stale where no op wrote them)
    for i in range(R):
        t = np.zeros(6)
        O.lib().oracle_qual_to_trans_probs(t.ctypes.data_as(O._f64p), int(ins[i]), int(dl[i]), int(gcp[i]))
        MM, IM, MI, II, MD, DD = t
        pm = O.lib().oracle_qual_to_prob(int(q[i]))
        pe = pm if read[i] == ord("N") else O.lib().oracle_qual_to_error_prob(int(q[i])) / 3.0
        tbl = [pm if read[i] in (c, ord("N")) else pe for c in b"ACGT"] + [pm]  # prior table row: codes A,C,G,T,N
        cM, cI, cD = [0.0] * (H + 1), [0.0] * (H + 1), [0.0] * (H + 1)
        cB = [[0.0] * (H + 1) for _ in range(3)]
        for j in range(1, H + 1):
            o, code = int(ops[j - 1]), int(codes[j - 1])
            prior = tbl[code]
            if o & 16:
                alt = (o >> 5) & 3
                if o & 128:
                    tu, tn, tw = tbl[alt], tbl[4], tbl[0 if alt else 1]
                    prior = tw if tu == tn else tn
                else:
                    third = min(b for b in range(4) if b not in (code, alt))
                    t1, t2, t3 = tbl[code], tbl[alt], tbl[third]
                    prior = t1 if (t1 == t2 or t1 != t3) else t2
            xprev = [cM[j - 1], cI[j - 1], cD[j - 1]]
            for v in range(3):
                if o & 2:
                    xprev[v] = max(cB[v][j - 1], xprev[v])
                cB[v][j] = xprev[v] if o & 1 else cB[v][j - 1]  # stored only where a later column reads it
            above = [M[j - 1], I[j - 1], D[j - 1]]
            if o & 2:
                above = [max(B[v][j - 1], above[v]) for v in range(3)]
            cM[j] = prior * (above[0] * MM + above[1] * IM + above[2] * IM)
            cD[j] = xprev[0] * MD + xprev[2] * DD
            if o & 4:
                cI[j] = max(B[0][j], M[j]) * MI + max(B[1][j], I[j]) * II
            else:
                cI[j] = M[j] * MI + I[j] * II
        M, I, D, B = cM, cI, cD, cB
    s = 0.0
    for j in range(1, H + 1):
        s += M[j] + I[j]
    return math.log10(s) - math.log10(2.0 ** 1020)


def test_packed_kernel_ops_reproduce_the_oracle():
    rng = np.random.default_rng(29)
    n_packed = n_general = 0
    for k in range(160):
        H, R = int(rng.integers(20, 60)), int(rng.integers(4, 18))
        hap, pd, read, q, ins, dls, g = _case(rng, H=H, R=R, n_snp=int(rng.integers(0, 5)),
                                               n_del=int(rng.integers(0, 5)), dl=(1, 6), end_flag=(k % 9 == 8))
        hap, read = hap.copy(), read.copy()
        if k % 3 == 0:
            pd[int(rng.integers(1, H - 1))] |= DS | DE  # single-base deletion
        if k % 4 == 1:  # SNP columns with two and three alternatives, and one on an N column
            for j in rng.choice(np.arange(H), size=3, replace=False):
                pd[j] |= SNP
                for c in rng.choice(list(b"ACGT"), size=int(rng.integers(2, 4)), replace=False):
                    pd[j] |= BIT[int(c)]
            j = int(rng.integers(0, H))
            hap[j] = ord("N")
            pd[j] |= SNP | BIT[ord("C")]
        if k % 5 == 2:
            read[int(rng.integers(0, R))] = ord("N")
        packed, ops, codes = _pd_ops(hap, pd)
        if not packed:  # a state left open at the row's end: the general kernel's pairs
            n_general += 1
            continue
        n_packed += 1
        ref = O.pd_logless(hap, pd, read, q, ins, dls, g)
        assert _lazy_branch_pdhmm(hap, read, q, ins, dls, g, ops, codes) == ref, k
    assert n_packed > 120 and n_general > 0


def test_packed_kernel_ops_hand_cases():
    # a deletion from column 2 to 4 (0-based): copy at its start column, DEL_END and next-AFTER at its end, AFTER after
    hap = np.frombuffer(b"ACGTACGTAC", dtype=np.uint8)
    pd = np.zeros(10, dtype=np.uint8)
    pd[2] |= DS
    pd[4] |= DE
    pd[7] |= SNP | BIT[ord("G")]  # column base T, alternative G
    pd[8] |= SNP | BIT[ord("A")] | BIT[ord("C")] | BIT[ord("G")] | BIT[ord("T")]
    pd[9] |= SNP | BIT[ord("A")] | BIT[ord("G")]  # column base C: C, A and G match, T does not
    packed, ops, codes = _pd_ops(hap, pd)
    assert packed
    assert list(ops[:6]) == [0, 0, 1, 0, 4 | 8, 2]
    assert ops[7] == 16 | (2 << 5) and codes[7] == 3
    assert ops[8] == 0 and codes[8] == 4  # every base matches: the column reads as N
    assert ops[9] == 16 | 128 | (3 << 5) and codes[9] == 1
    pd[9] = DE  # a deletion ending on the last column: the next row starts in AFTER_DEL, which acts as NORMAL there
    packed, ops, _ = _pd_ops(hap, pd)
    assert packed and not ops[0] & 2
    pd[9] = DS  # a deletion left open: the next row starts INSIDE_DEL, for the general kernel
    assert not _pd_ops(hap, pd)[0]


# ---------------------------------------------------------------------------------------------------------------
# the GPU PD-HMM kernel (pd.cu) against the oracle

def _pd_workload(regions=6, seed=5):
    wl = W.generate(1, regions=regions)
    return wl, W.pd_flags(wl, seed)


@pytest.fixture(scope="module")
def engine64():
    """A double-precision engine: ghmm_pd_compute_* run every pair in FP64 (GHMM_MODE_PD)."""
    from gatk_gb300.pairhmm import Engine

    e = Engine(use_double_precision=True)
    yield e
    e.close()


@pytest.mark.gpu
def test_gpu_pdhmm_matches_oracle(engine, engine64):
    wl, pd = _pd_workload(8)
    ref = O.pd_compute_workload(wl, pd)
    assert np.abs(engine64.pd_compute(wl, pd) - ref).max() <= 1e-9  # FP64 PD kernel
    assert np.abs(engine.pd_compute(wl, pd) - ref).max() <= 1e-3    # FP32 PD kernel + FP64 reruns (the FP32 bar)


@pytest.mark.gpu
def test_gpu_pdhmm_without_flags_equals_plain(engine, engine64):
    wl = W.generate(1, regions=4)
    flags = np.zeros(len(wl.hap_bases), dtype=np.uint8)
    ref = O.compute_workload(wl)
    assert np.abs(engine64.pd_compute(wl, flags) - ref).max() <= 1e-9
    assert np.abs(engine.pd_compute(wl, flags) - ref).max() <= 1e-3


@pytest.mark.gpu
def test_gpu_pdhmm_fp32_reruns_underflows_in_fp64(engine):
    # long reads against long haplotypes with many mismatches: log10 L far below the FP32 range at 2^120, so the FP32
    # pass queues them and the FP64 kernel recomputes them; every result within the FP64 bar of the oracle for
    # those pairs and the FP32 bar for the rest
    from gatk_gb300 import native

    rng = np.random.default_rng(33)
    regions, pds = [], []
    for k in range(6):
        H = int(rng.integers(500, 900))
        R = int(rng.integers(200, 400)) if k % 2 == 0 else int(rng.integers(40, 80))
        hap, pd, read, q, ins, dls, g = _case(rng, H=H, R=R, n_snp=4, n_del=2, end_flag=False)
        read = bytearray(read)
        if k % 2 == 0:  # one base in four replaced: far beyond the FP32 range
            for i in range(0, len(read), 4):
                read[i] = ord("ACGT"[(("ACGT".index(chr(read[i])) if chr(read[i]) in "ACGT" else 0) + 1) % 4])
        regions.append(([bytes(hap)], [(bytes(read), q, ins, dls, g)]))
        pds.append(pd)
    wl = W.from_pairs(regions)
    pd = np.concatenate(pds)
    ref = O.pd_compute_workload(wl, pd)
    with engine.pd_batch(wl, pd) as b:
        b.forward(native.MODE_PD_FP32)
        got = b.results()
        st = b.stats()
    low = ref < -120.0
    assert low.any() and st["n_rerun"] >= int(low.sum())
    assert np.abs(got[low] - ref[low]).max() <= 1e-9
    assert np.abs(got - ref).max() <= 1e-3


@pytest.mark.gpu
def test_gpu_pdhmm_hand_cases_and_long_reads(engine):
    # deletions at the first and last columns (the state carries into the next row), single-base deletions,
    # SNP alternatives, and reads longer than one 128-row strip
    rng = np.random.default_rng(21)
    regions, pds = [], []
    for k in range(12):
        H = int(rng.integers(150, 400))
        R = int(rng.integers(60, 300))
        hap, pd, read, q, ins, dls, g = _case(rng, H=H, R=min(R, H - 5), n_snp=3, n_del=1 + k % 3,
                                               end_flag=(k % 3 == 0))
        if k % 4 == 1:
            pd[0] |= DS
        regions.append(([bytes(hap)], [(bytes(read), q, ins, dls, g)]))
        pds.append(pd)
    wl = W.from_pairs(regions)
    pd = np.concatenate(pds)
    ref = O.pd_compute_workload(wl, pd)
    from gatk_gb300 import native

    with engine.pd_batch(wl, pd) as b:
        b.forward(native.MODE_PD)
        assert np.abs(b.results() - ref).max() <= 1e-9
        b.forward(native.MODE_PD_FP32)
        assert np.abs(b.results() - ref).max() <= 1e-3


@pytest.mark.gpu
def test_gpu_pdhmm_packed_kernel_reads_of_several_strips(engine):
    # reads of 260-690 bases (two to four strips of the packed kernel) against 700-1,200-base haplotypes with every
    # kind of PD column: each strip's last row reaches the next strip through scratch, the PD max included
    from gatk_gb300 import native

    rng = np.random.default_rng(47)
    regions, pds = [], []
    for g in range(12):
        haps, hpd = [], []
        first = rng.choice(list(b"ACGT"), size=int(rng.integers(700, 1200))).astype(np.uint8)
        for h in range(int(rng.integers(1, 3))):
            hap = first.copy()  # the region's haplotypes: variants of one sequence
            if h:
                snv = rng.choice(np.arange(len(hap)), size=5, replace=False)
                hap[snv] = [[c for c in b"ACGT" if c != hap[k]][0] for k in snv]
                cut = int(rng.integers(100, len(hap) - 100))
                hap = np.concatenate([hap[:cut], hap[cut + 3:]])
            H = len(hap)
            pd = np.zeros(H, dtype=np.uint8)
            for _ in range(4):
                k = int(rng.integers(0, H))
                pd[k] |= SNP | BIT[[c for c in b"ACGT" if c != hap[k]][int(rng.integers(0, 3))]]
            for _ in range(3):
                n = int(rng.integers(1, 10))
                j = int(rng.integers(1, H - n - 1))
                pd[j] |= DS
                pd[j + n - 1] |= DE
            pd[int(rng.integers(2, H - 2))] |= DS | DE
            haps.append(bytes(hap))
            hpd.append(pd)
        base = np.frombuffer(haps[0], dtype=np.uint8)
        reads = []
        for _ in range(int(rng.integers(2, 6))):
            R = int(rng.integers(260, 690))
            start = int(rng.integers(0, len(base) - R))
            rd = base[start:start + R].copy()
            flip = rng.random(R) < 0.01
            rd[flip] = rng.choice(list(b"ACGT"), size=int(flip.sum())).astype(np.uint8)
            reads.append((bytes(rd), rng.integers(25, 41, size=R), rng.integers(30, 46, size=R),
                          rng.integers(30, 46, size=R), np.full(R, 10)))
        regions.append((haps, reads))
        pds.extend(hpd)
    wl, pd = W.from_pairs(regions), np.concatenate(pds)
    ref = O.pd_compute_workload(wl, pd)
    with engine.pd_batch(wl, pd) as b:
        b.forward(native.MODE_PD_FP32)
        got = b.results()
        st = b.stats()
    assert np.isfinite(ref).all() and st["n_tasks_fp32"] > 0
    assert st["n_rerun"] < wl.n_pairs // 4  # most pairs stay in the FP32 packed path
    assert np.abs(got - ref).max() <= 1e-3


@pytest.mark.gpu
def test_gpu_pdhmm_error_in_a_later_chunk(engine):
    # a read base outside ACGTacgtN meets an undetermined SNP in the last of 30 regions: the one-shot call marshals
    # that region's chunk while earlier chunks run, returns GHMM_ERR_ARG, and the engine computes correctly afterwards
    from gatk_gb300 import native

    wl, pd = _pd_workload(30, seed=6)
    g = wl.n_regions - 1
    r, h = int(wl.region_read_off[g]), int(wl.region_hap_off[g])
    a, j = int(wl.read_off[r]), int(wl.hap_off[h])
    bases = wl.bases.copy()
    bases[a] = ord("R")
    flags = pd.copy()
    flags[j] |= SNP | BIT[ord("A")]
    bad = W.Workload(region_read_off=wl.region_read_off, region_hap_off=wl.region_hap_off, read_off=wl.read_off,
                     bases=bases, quals=wl.quals, ins=wl.ins, dels=wl.dels, gcp=wl.gcp, hap_off=wl.hap_off,
                     hap_bases=wl.hap_bases, out_off=wl.out_off)
    if wl.hap_bases[j] == ord("R"):
        pytest.skip("the haplotype base equals the planted read base")
    with pytest.raises(native.GhmmError) as e:
        engine.pd_compute(bad, flags)
    assert e.value.code == native.GHMM_ERR_ARG
    ref = O.pd_compute_workload(wl, pd)
    assert np.abs(engine.pd_compute(wl, pd) - ref).max() <= 1e-3


@pytest.mark.gpu
def test_gpu_pdhmm_batch_and_errors(engine):
    from gatk_gb300 import native

    wl, pd = _pd_workload(3)
    with engine.pd_batch(wl, pd) as b:
        for mode in (native.MODE_PD, native.MODE_PD_FP32):
            b.forward(mode)
            a = b.results()
            b.forward(mode)
            assert np.array_equal(a, b.results())
        with pytest.raises(native.GhmmError):
            b.forward(native.MODE_FP32_RERUN)
    # a read base outside ACGTacgtN meeting an undetermined SNP: the reference throws
    hap = b"ACGTACGTACGTACGT"
    f = np.zeros(len(hap), dtype=np.uint8)
    f[5] = SNP | BIT[ord("A")]
    bad = W.from_pairs([([hap], [(b"ACGRAC", [30] * 6, [45] * 6, [45] * 6, [10] * 6)])])
    with pytest.raises(native.GhmmError) as e:
        engine.pd_compute(bad, f)
    assert e.value.code == native.GHMM_ERR_ARG


def _oracle_prepared(wl, mapq, dragstr):
    from oracle import readprep as RP

    planes = [np.empty_like(wl.bases) for _ in range(4)]
    for r in range(wl.n_reads):
        a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
        _, q, i, d, g = RP.prepare_read(wl.bases[a:b], wl.quals[a:b], wl.ins[a:b], wl.dels[a:b], int(mapq[r]),
                                        rate_factor=3.0, dragstr=dragstr)
        for k, v in enumerate((q, i, d, g)):
            planes[k][a:b] = np.frombuffer(v, dtype=np.uint8)
    return W.Workload(region_read_off=wl.region_read_off, region_hap_off=wl.region_hap_off, read_off=wl.read_off,
                      bases=wl.bases, quals=planes[0], ins=planes[1], dels=planes[2], gcp=planes[3],
                      hap_off=wl.hap_off, hap_bases=wl.hap_bases, out_off=wl.out_off)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["pcr", "dragstr"])
def test_gpu_pdhmm_from_raw_reads(engine, engine64, kind):
    # ghmm_pd_compute_regions_raw / ghmm_pd_batch_create_raw: the reads prepared on the device (the DRAGEN-GATK
    # chain with DRAGstr), then the PD-HMM; against the PD oracle on the restatement's own preparation
    import json
    import os

    wl, pd = _pd_workload(12, seed=8)  # enough regions for the one-shot calls to run in two pipelined chunks
    rng = np.random.default_rng(19)
    wl.quals[:] = rng.integers(2, 45, size=len(wl.quals)).astype(np.uint8)
    wl.ins[:] = rng.integers(10, 50, size=len(wl.ins)).astype(np.uint8)
    wl.dels[:] = rng.integers(10, 50, size=len(wl.dels)).astype(np.uint8)
    mapq = rng.integers(10, 70, size=wl.n_reads)
    dragstr = None
    if kind == "dragstr":
        with open(os.path.join(os.path.dirname(__file__), "golden", "dragstr_cases.json")) as f:
            t = json.load(f)["example_params"]
        dragstr = (np.array(t["gop"]), np.array(t["gcp"]))
    prepared = _oracle_prepared(wl, mapq, dragstr)
    ref = O.pd_compute_workload(prepared, pd)
    assert np.abs(engine64.pd_compute_raw(wl, pd, mapq, dragstr=dragstr) - ref).max() <= 1e-9
    assert np.abs(engine.pd_compute_raw(wl, pd, mapq, dragstr=dragstr) - ref).max() <= 1e-3
    with engine.pd_raw_batch(wl, pd, mapq, dragstr=dragstr) as b:
        _, q, i, d, g = b.read_planes()
    assert np.array_equal(q, prepared.quals) and np.array_equal(i, prepared.ins)
    assert np.array_equal(d, prepared.dels) and np.array_equal(g, prepared.gcp)


def _packed_case_workload(seed=41):
    """Regions of several reads (lengths 20-254, so read-pair tasks of 2 to 8 rows per lane pair reads of different
    lengths) against haplotypes whose flags reach every per-column op of the packed FP32 kernel (pd_packed.cu):
    single-base deletions (DEL_START and DEL_END on one column), a deletion from column 1, a DEL_END on the
    second-to-last column (AFTER_DEL at the last), an AFTER_DEL column that ends another deletion (AFTER_DEL twice in
    a row), SNP columns inside a deletion, an SNP on an N column, SNP columns with two and with three alternatives
    (three or four matching bases), reads with N, a deletion ending on the last column (the next row starts in
    AFTER_DEL); plus one region with a deletion left open at the last column, which the host sends to the general
    kernel."""
    rng = np.random.default_rng(seed)
    regions, pds = [], []
    lengths = [20, 33, 40, 62, 63, 64, 90, 126, 150, 190, 222, 254]
    for g in range(26):
        nh = int(rng.integers(1, 4))
        haps, hpd = [], []
        for h in range(nh):
            H = int(rng.integers(80, 420))
            hap = rng.choice(list(b"ACGT"), size=H).astype(np.uint8)
            pd = np.zeros(H, dtype=np.uint8)
            kind = (g + h) % 6
            if kind == 0:
                for j in rng.choice(np.arange(2, H - 2), size=4, replace=False):
                    pd[j] |= DS | DE
            elif kind == 1:
                n = int(rng.integers(1, 8))
                pd[1] |= DS
                pd[n] |= DE
            elif kind == 2:
                n = int(rng.integers(1, 8))
                pd[H - 1 - n] |= DS
                pd[H - 2] |= DE
            elif kind == 3:
                j = int(rng.integers(5, H - 12))
                pd[j] |= DS
                pd[j + 2] |= DE
                pd[j + 3] |= DE
                pd[j + 5] |= DS | DE
            elif kind == 4:
                j = int(rng.integers(5, H - 12))
                pd[j] |= DS
                pd[j + 6] |= DE
                for k in (j + 2, j + 6, j + 7):
                    alt = [c for c in b"ACGT" if c != hap[k]][int(rng.integers(0, 3))]
                    pd[k] |= SNP | BIT[alt]
                k = int(rng.integers(j + 10, H))
                hap[k] = ord("N")
                pd[k] |= SNP | BIT[ord("A")]
            else:
                for _ in range(4):
                    k = int(rng.integers(0, H))
                    alt = [c for c in b"ACGT" if c != hap[k]][int(rng.integers(0, 3))]
                    pd[k] |= SNP | BIT[alt]
                for _ in range(3):
                    n = int(rng.integers(1, 10))
                    j = int(rng.integers(1, H - n - 1))
                    pd[j] |= DS
                    pd[j + n - 1] |= DE
            if g == 24 and h == 0:
                pd[H - 1] |= DS  # a deletion left open at the row's end carries into the next row: general kernel
            if g == 23 and h == 0:
                pd[H - 1] |= DE  # the next row starts in AFTER_DEL (the packed kernel takes it)
            if g >= 20:  # SNP columns listing two and three alternatives
                for k in rng.choice(np.arange(H), size=6, replace=False):
                    others = [c for c in b"ACGT" if c != hap[k]]
                    chosen = others if k % 2 else [others[int(rng.integers(0, 3))], others[int(rng.integers(0, 3))]]
                    pd[k] |= SNP
                    for c in chosen:
                        pd[k] |= BIT[c]
            haps.append(bytes(hap))
            hpd.append(pd)
        base = np.frombuffer(haps[0], dtype=np.uint8)
        reads = []
        for _ in range(int(rng.integers(2, 9))):
            R = int(rng.choice(lengths))
            start = int(rng.integers(0, max(1, len(base) - R + 1)))
            rd = np.concatenate([base[start:start + R], rng.choice(list(b"ACGT"), size=max(0, R - len(base)))])
            rd = rd[:R].astype(np.uint8).copy()
            rd[rd == ord("N")] = ord("A")
            flip = rng.random(R) < 0.03
            rd[flip] = rng.choice(list(b"ACGT"), size=int(flip.sum()))
            if rng.random() < 0.3:
                rd[int(rng.integers(0, R))] = ord("N")
            reads.append((bytes(rd), rng.integers(10, 41, size=R), rng.integers(20, 46, size=R),
                          rng.integers(20, 46, size=R), np.full(R, 10)))
        regions.append((haps, reads))
        pds.extend(hpd)
    return W.from_pairs(regions), np.concatenate(pds)


@pytest.mark.gpu
def test_gpu_pdhmm_packed_kernel_every_op(engine, engine64):
    from gatk_gb300 import native

    wl, pd = _packed_case_workload()
    ref = O.pd_compute_workload(wl, pd)
    assert np.isfinite(ref).all()
    assert np.abs(engine64.pd_compute(wl, pd) - ref).max() <= 1e-9
    with engine.pd_batch(wl, pd) as b:
        b.forward(native.MODE_PD_FP32)
        got = b.results()
        st = b.stats()
        b.forward(native.MODE_PD_FP32)
        assert np.array_equal(got, b.results())
    assert st["n_tasks_fp32"] > 0  # read-pair tasks ran in the packed kernel
    assert np.abs(got - ref).max() <= 1e-3
    # the same pairs with one read per region: tasks of a single read, the other half empty
    single = [([wl.hap(h) for h in range(int(wl.region_hap_off[g]), int(wl.region_hap_off[g + 1]))], [wl.read(r)])
              for g in range(wl.n_regions) for r in range(int(wl.region_read_off[g]), int(wl.region_read_off[g + 1]))]
    wl1 = W.from_pairs(single)
    region_pd = [pd[int(wl.hap_off[wl.region_hap_off[g]]):int(wl.hap_off[wl.region_hap_off[g + 1]])]
                 for g in range(wl.n_regions)]
    pd1 = np.concatenate([region_pd[g] for g in range(wl.n_regions)
                          for _ in range(int(wl.region_read_off[g + 1] - wl.region_read_off[g]))])
    ref1 = O.pd_compute_workload(wl1, pd1)
    assert np.abs(engine.pd_compute(wl1, pd1) - ref1).max() <= 1e-3
    # regions without reads or without haplotypes among ordinary ones, over several pipelined chunks
    rng = np.random.default_rng(43)
    mixed = []
    for g in range(40):
        haps = [] if g % 7 == 3 else [bytes(rng.choice(list(b"ACGT"), size=int(rng.integers(30, 200))).astype(np.uint8))
                                      for _ in range(3)]
        reads = []
        if g % 5 != 2:
            for _ in range(int(rng.integers(1, 6))):
                n = int(rng.integers(10, 120))
                reads.append((bytes(rng.choice(list(b"ACGT"), size=n).astype(np.uint8)), rng.integers(10, 41, size=n),
                              np.full(n, 40), np.full(n, 40), np.full(n, 10)))
        mixed.append((haps, reads))
    wl2 = W.from_pairs(mixed)
    pd2 = W.pd_flags(wl2, 9)
    ref2 = O.pd_compute_workload(wl2, pd2)
    assert np.abs(engine.pd_compute(wl2, pd2) - ref2).max() <= 1e-3
    assert np.abs(engine64.pd_compute(wl2, pd2) - ref2).max() <= 1e-9
