"""Flat workloads: regions of reads and haplotypes laid out as contiguous planes.

``Workload`` is the in-memory form every entry point shares: the synthetic generator
(``generate``), the batch uploader (``as_flat``) and the test oracle all read the same arrays.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import native

# seeds of the five synthetic workloads
DEFAULT_SEEDS = {0: 0, 1: 1, 2: 2, 3: 3, 4: 4}


@dataclass
class Workload:
    region_read_off: np.ndarray  # int64 [G+1]
    region_hap_off: np.ndarray   # int64 [G+1]
    read_off: np.ndarray         # int64 [NR+1]
    bases: np.ndarray            # uint8 planes
    quals: np.ndarray
    ins: np.ndarray
    dels: np.ndarray
    gcp: np.ndarray
    hap_off: np.ndarray          # int64 [NH+1]
    hap_bases: np.ndarray        # uint8
    out_off: np.ndarray          # int64 [G+1]
    _keep: list = field(default_factory=list, repr=False)

    @property
    def n_regions(self) -> int:
        return len(self.region_read_off) - 1

    @property
    def n_reads(self) -> int:
        return len(self.read_off) - 1

    @property
    def n_haps(self) -> int:
        return len(self.hap_off) - 1

    @property
    def n_pairs(self) -> int:
        return int(self.out_off[-1])

    def read_lengths(self) -> np.ndarray:
        return np.diff(self.read_off)

    def hap_lengths(self) -> np.ndarray:
        return np.diff(self.hap_off)

    def cells(self) -> int:
        rl = self.read_lengths()
        hl = self.hap_lengths()
        tot = 0
        for g in range(self.n_regions):
            r0, r1 = self.region_read_off[g], self.region_read_off[g + 1]
            h0, h1 = self.region_hap_off[g], self.region_hap_off[g + 1]
            tot += int(rl[r0:r1].sum()) * int(hl[h0:h1].sum())
        return tot

    def cells_per_region(self) -> np.ndarray:
        rl = np.concatenate([[0], np.cumsum(self.read_lengths())])
        hl = np.concatenate([[0], np.cumsum(self.hap_lengths())])
        sr = rl[self.region_read_off[1:]] - rl[self.region_read_off[:-1]]
        sh = hl[self.region_hap_off[1:]] - hl[self.region_hap_off[:-1]]
        return sr.astype(np.int64) * sh.astype(np.int64)

    def pair_index(self):
        """Global (read, haplotype) index of every output slot, read-major per region."""
        pr = np.empty(self.n_pairs, dtype=np.int64)
        ph = np.empty(self.n_pairs, dtype=np.int64)
        for g in range(self.n_regions):
            r0, r1 = int(self.region_read_off[g]), int(self.region_read_off[g + 1])
            h0, h1 = int(self.region_hap_off[g]), int(self.region_hap_off[g + 1])
            o = int(self.out_off[g])
            nr, nh = r1 - r0, h1 - h0
            pr[o:o + nr * nh] = np.repeat(np.arange(r0, r1), nh)
            ph[o:o + nr * nh] = np.tile(np.arange(h0, h1), nr)
        return pr, ph

    def read(self, r: int):
        a, b = int(self.read_off[r]), int(self.read_off[r + 1])
        return (self.bases[a:b], self.quals[a:b], self.ins[a:b], self.dels[a:b], self.gcp[a:b])

    def hap(self, h: int):
        return self.hap_bases[int(self.hap_off[h]):int(self.hap_off[h + 1])]

    def subset(self, g0: int, g1: int) -> "Workload":
        """Regions [g0, g1) as a self-contained workload."""
        r0, r1 = int(self.region_read_off[g0]), int(self.region_read_off[g1])
        h0, h1 = int(self.region_hap_off[g0]), int(self.region_hap_off[g1])
        b0, b1 = int(self.read_off[r0]), int(self.read_off[r1])
        c0, c1 = int(self.hap_off[h0]), int(self.hap_off[h1])
        return Workload(
            region_read_off=self.region_read_off[g0:g1 + 1] - r0,
            region_hap_off=self.region_hap_off[g0:g1 + 1] - h0,
            read_off=self.read_off[r0:r1 + 1] - b0,
            bases=self.bases[b0:b1].copy(), quals=self.quals[b0:b1].copy(), ins=self.ins[b0:b1].copy(),
            dels=self.dels[b0:b1].copy(), gcp=self.gcp[b0:b1].copy(),
            hap_off=self.hap_off[h0:h1 + 1] - c0, hap_bases=self.hap_bases[c0:c1].copy(),
            out_off=self.out_off[g0:g1 + 1] - self.out_off[g0])

    def read_slice(self, read_begin: int, read_end: int) -> "Workload":
        """Reads [read_begin, read_end) (numbered across regions in order) as a self-contained workload: every
        region that overlaps the range, restricted to its reads in the range, with all its haplotypes.  Its
        read-major outputs are the slice of this workload's outputs that those reads own."""
        rro = self.region_read_off
        g0 = int(np.searchsorted(rro, read_begin, side="right")) - 1
        g1 = int(np.searchsorted(rro, read_end, side="left"))
        g0 = max(g0, 0)
        g1 = max(g1, g0)
        sub = self.subset(g0, g1) if g1 > g0 else self.subset(g0, g0)
        if g1 == g0:
            return sub
        # trim the first region's leading reads and the last region's trailing reads
        lead = read_begin - int(rro[g0])
        trail = int(rro[g1]) - read_end
        n_reads = read_end - read_begin
        nr = np.diff(sub.region_read_off).copy()
        nr[0] -= lead
        nr[-1] -= trail
        b0 = int(sub.read_off[lead])
        b1 = int(sub.read_off[lead + n_reads])
        nh = np.diff(sub.region_hap_off)
        return Workload(
            region_read_off=np.concatenate([[0], np.cumsum(nr)]).astype(np.int64),
            region_hap_off=sub.region_hap_off, read_off=sub.read_off[lead:lead + n_reads + 1] - b0,
            bases=sub.bases[b0:b1].copy(), quals=sub.quals[b0:b1].copy(), ins=sub.ins[b0:b1].copy(),
            dels=sub.dels[b0:b1].copy(), gcp=sub.gcp[b0:b1].copy(), hap_off=sub.hap_off, hap_bases=sub.hap_bases,
            out_off=np.concatenate([[0], np.cumsum(nr * nh)]).astype(np.int64))

    def as_flat(self) -> native.Flat:
        p = lambda a, t: a.ctypes.data_as(t)
        f = native.Flat(self.n_regions, p(self.region_read_off, native._i64p), p(self.region_hap_off, native._i64p),
                        p(self.read_off, native._i64p), p(self.bases, native._u8p), p(self.quals, native._u8p),
                        p(self.ins, native._u8p), p(self.dels, native._u8p), p(self.gcp, native._u8p),
                        p(self.hap_off, native._i64p), p(self.hap_bases, native._u8p), p(self.out_off, native._i64p))
        return f

    def as_regions(self):
        """ghmm_region array with per-read pointers into the planes (the JNI-shaped input)."""
        NR = self.n_reads
        assert ctypes.sizeof(native.Read) == 48 and ctypes.sizeof(native.Hap) == 16
        assert ctypes.sizeof(native.Region) == 32
        rd = np.zeros((max(NR, 1), 6), dtype=np.uint64)  # five plane pointers, then length and padding
        o = self.read_off[:-1].astype(np.uint64)
        for k, plane in enumerate((self.bases, self.quals, self.ins, self.dels, self.gcp)):
            np.add(o, np.uint64(plane.ctypes.data), out=rd[:NR, k])
        rd.view(np.int32)[:NR, 10] = np.diff(self.read_off)
        return _region_table(self, rd, 48)


def _region_table(wl: Workload, rd: np.ndarray, read_size: int):
    """ghmm_region-shaped array (reads pointer, count, haplotypes pointer, count) over the per-read table rd."""
    NH, G = wl.n_haps, wl.n_regions
    hp = np.zeros((max(NH, 1), 2), dtype=np.uint64)
    np.add(wl.hap_off[:-1].astype(np.uint64), np.uint64(wl.hap_bases.ctypes.data), out=hp[:NH, 0])
    hp.view(np.int32)[:NH, 2] = np.diff(wl.hap_off)
    rg = np.zeros((max(G, 1), 4), dtype=np.uint64)
    rg[:G, 0] = np.uint64(rd.ctypes.data) + wl.region_read_off[:-1].astype(np.uint64) * np.uint64(read_size)
    rg.view(np.int32)[:G, 2] = np.diff(wl.region_read_off)
    rg[:G, 2] = np.uint64(hp.ctypes.data) + wl.region_hap_off[:-1].astype(np.uint64) * np.uint64(16)
    rg.view(np.int32)[:G, 6] = np.diff(wl.region_hap_off)
    wl._keep.append((rd, hp, rg))
    return rg.ctypes.data_as(ctypes.POINTER(native.Region))


def as_raw_regions(wl: Workload, mapq: np.ndarray, with_indel_quals: bool = True):
    """ghmm_raw_region array: the workload's bases and base qualities as raw reads with a mapping quality each;
    the insertion / deletion planes as BI / BD tags, or none (the library's 45) when with_indel_quals is False."""
    NR = wl.n_reads
    assert ctypes.sizeof(native.RawRead) == 40 and ctypes.sizeof(native.RawRegion) == 32
    rd = np.zeros((max(NR, 1), 5), dtype=np.uint64)  # four pointers, then length and mapping quality
    o = wl.read_off[:-1].astype(np.uint64)
    planes = (wl.bases, wl.quals, wl.ins, wl.dels) if with_indel_quals else (wl.bases, wl.quals)
    for k, plane in enumerate(planes):
        np.add(o, np.uint64(plane.ctypes.data), out=rd[:NR, k])
    i32 = rd.view(np.int32)
    i32[:NR, 8] = np.diff(wl.read_off)
    i32[:NR, 9] = np.asarray(mapq, dtype=np.int32)
    return ctypes.cast(_region_table(wl, rd, 40), ctypes.c_void_p).value


def as_pd_raw_regions(wl: Workload, hap_pd: np.ndarray, mapq: np.ndarray, with_indel_quals: bool = True):
    """ghmm_pd_raw_region array: the workload's reads as raw reads (as as_raw_regions) against its haplotypes with PD
    flags (as as_pd_regions)."""
    as_raw_regions(wl, mapq, with_indel_quals)
    rd = wl._keep[-1][0]
    as_pd_regions(wl, hap_pd)
    _, hp, _ = wl._keep[-1]
    G = wl.n_regions
    rg = np.zeros((max(G, 1), 4), dtype=np.uint64)
    rg[:G, 0] = np.uint64(rd.ctypes.data) + wl.region_read_off[:-1].astype(np.uint64) * np.uint64(40)
    rg.view(np.int32)[:G, 2] = np.diff(wl.region_read_off)
    rg[:G, 2] = np.uint64(hp.ctypes.data) + wl.region_hap_off[:-1].astype(np.uint64) * np.uint64(24)
    rg.view(np.int32)[:G, 6] = np.diff(wl.region_hap_off)
    wl._keep.append((rd, hp, rg))
    return rg.ctypes.data


def as_pd_regions(wl: Workload, hap_pd: np.ndarray):
    """ghmm_pd_region array for a workload whose haplotypes carry PD flags (hap_pd, parallel to hap_bases)."""
    NR, NH, G = wl.n_reads, wl.n_haps, wl.n_regions
    wl.as_regions()  # builds the per-read structs (kept alive in wl._keep)
    rd = wl._keep[-1][0]
    pd = np.ascontiguousarray(hap_pd, dtype=np.uint8)
    hp = np.zeros((max(NH, 1), 3), dtype=np.uint64)  # bases pointer, PD flags pointer, length and padding
    ho = wl.hap_off[:-1].astype(np.uint64)
    np.add(ho, np.uint64(wl.hap_bases.ctypes.data), out=hp[:NH, 0])
    np.add(ho, np.uint64(pd.ctypes.data), out=hp[:NH, 1])
    hp.view(np.int32)[:NH, 4] = np.diff(wl.hap_off)
    rg = np.zeros((max(G, 1), 4), dtype=np.uint64)
    rg[:G, 0] = np.uint64(rd.ctypes.data) + wl.region_read_off[:-1].astype(np.uint64) * np.uint64(48)
    rg.view(np.int32)[:G, 2] = np.diff(wl.region_read_off)
    rg[:G, 2] = np.uint64(hp.ctypes.data) + wl.region_hap_off[:-1].astype(np.uint64) * np.uint64(24)
    rg.view(np.int32)[:G, 6] = np.diff(wl.region_hap_off)
    wl._keep.append((pd, hp, rg))
    return rg.ctypes.data


def generate(workload: int, regions: int | None = None, seed: int | None = None, region_begin: int = 0,
             threads: int = 0) -> Workload:
    """Synthetic workload `workload` (0-4), regions [region_begin, region_begin + regions)."""
    L = native.synth_lib()
    if seed is None:
        seed = DEFAULT_SEEDS[workload]
    if regions is None:
        regions = int(L.ghmm_synth_default_regions(workload))
    h = ctypes.c_void_p()
    rc = L.ghmm_synth_generate(workload, seed, region_begin, region_begin + regions, threads, ctypes.byref(h))
    if rc != 0:
        raise ValueError(f"ghmm_synth_generate failed for workload {workload}")
    try:
        a = native.SynthArrays()
        L.ghmm_synth_view(h, ctypes.byref(a))

        def cp(ptr, n, dt):
            if n == 0:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt, copy=True)

        G, NR, NH = a.n_regions, a.n_reads, a.n_haps
        return Workload(
            region_read_off=cp(a.region_read_off, G + 1, np.int64), region_hap_off=cp(a.region_hap_off, G + 1, np.int64),
            read_off=cp(a.read_off, NR + 1, np.int64), bases=cp(a.bases, a.read_bytes, np.uint8),
            quals=cp(a.quals, a.read_bytes, np.uint8), ins=cp(a.ins, a.read_bytes, np.uint8),
            dels=cp(a.dels, a.read_bytes, np.uint8), gcp=cp(a.gcp, a.read_bytes, np.uint8),
            hap_off=cp(a.hap_off, NH + 1, np.int64), hap_bases=cp(a.hap_bases, a.hap_bytes, np.uint8),
            out_off=cp(a.out_off, G + 1, np.int64))
    finally:
        L.ghmm_synth_free(h)


def from_pairs(regions) -> Workload:
    """Build a workload from Python data: regions = [(haps, reads)], haps = [bytes], reads =
    [(bases, quals, ins, dels, gcp)] with byte strings or uint8 arrays (Phred values)."""
    rro, rho, ro, ho, oo = [0], [0], [0], [0], [0]
    planes = [[], [], [], [], []]
    hb = []
    for haps, reads in regions:
        for h in haps:
            h = bytes(h)
            hb.append(np.frombuffer(h, dtype=np.uint8))
            ho.append(ho[-1] + len(h))
        for rd in reads:
            arrs = [np.asarray(bytearray(x) if isinstance(x, (bytes, bytearray)) else x, dtype=np.uint8) for x in rd]
            n = len(arrs[0])
            if any(len(x) != n for x in arrs):
                raise ValueError("read arrays must have equal lengths")
            for k in range(5):
                planes[k].append(arrs[k])
            ro.append(ro[-1] + n)
        rro.append(rro[-1] + len(reads))
        rho.append(rho[-1] + len(haps))
        oo.append(oo[-1] + len(reads) * len(haps))
    cat = lambda xs: np.concatenate(xs).astype(np.uint8) if xs else np.zeros(0, dtype=np.uint8)
    return Workload(region_read_off=np.array(rro, dtype=np.int64), region_hap_off=np.array(rho, dtype=np.int64),
                    read_off=np.array(ro, dtype=np.int64), bases=cat(planes[0]), quals=cat(planes[1]),
                    ins=cat(planes[2]), dels=cat(planes[3]), gcp=cat(planes[4]), hap_off=np.array(ho, dtype=np.int64),
                    hap_bases=cat(hb), out_off=np.array(oo, dtype=np.int64))


# PartiallyDeterminedHaplotype flag bits (utils/haplotype/PartiallyDeterminedHaplotype.java:59-66)
PD_SNP, PD_DEL_START, PD_DEL_END = 1, 2, 4
PD_BASE_BIT = {ord("A"): 8, ord("C"): 16, ord("G"): 32, ord("T"): 64}


def pd_flags(wl: Workload, seed: int = 5, snps_per_hap=(1, 3), dels_per_hap=(0, 2), del_len=(1, 10)) -> np.ndarray:
    """Partially-determined-haplotype flags for every haplotype of a workload (a byte per haplotype base, parallel
    to hap_bases), as PartiallyDeterminedHaplotype.getAlternateBases gives them (PartiallyDeterminedHaplotype.java:
    170-205): an undetermined SNP site carries SNP plus the bit of its alternative base; an undetermined deletion
    marks its first base DEL_START and its last DEL_END (both on a single-base deletion).  Sites are drawn with a
    numpy PCG64 stream seeded per haplotype, so the flags are the same on every machine."""
    out = np.zeros(len(wl.hap_bases), dtype=np.uint8)
    for h in range(wl.n_haps):
        a, b = int(wl.hap_off[h]), int(wl.hap_off[h + 1])
        H = b - a
        if H < 4:
            continue
        rng = np.random.default_rng([seed, h])
        hb = wl.hap_bases[a:b]
        for _ in range(int(rng.integers(snps_per_hap[0], snps_per_hap[1] + 1))):
            j = int(rng.integers(0, H))
            alts = [c for c in b"ACGT" if c != hb[j]]
            out[a + j] |= PD_SNP | PD_BASE_BIT[alts[int(rng.integers(0, 3))]]
        for _ in range(int(rng.integers(dels_per_hap[0], dels_per_hap[1] + 1))):
            n = int(rng.integers(del_len[0], del_len[1] + 1))
            j = int(rng.integers(1, max(2, H - n)))
            out[a + j] |= PD_DEL_START
            out[a + min(j + n - 1, H - 1)] |= PD_DEL_END
    return out
