"""The per-read struct arrays the Python side builds with numpy (gatk_gb300/workload.py) read back through the
ctypes mirrors of include/ghmm.h: the same pointers, lengths and mapping qualities the library will see."""
import ctypes

import numpy as np

from gatk_gb300 import native, workload as W


def _wl():
    wl = W.generate(1, regions=3)
    mapq = np.arange(wl.n_reads, dtype=np.int64) % 60 + 3
    return wl, mapq


def test_raw_region_table_reads_back():
    wl, mapq = _wl()
    base = W.as_raw_regions(wl, mapq, True)
    regs = ctypes.cast(base, ctypes.POINTER(native.RawRegion))
    for g in range(wl.n_regions):
        rg = regs[g]
        r0 = int(wl.region_read_off[g])
        assert rg.n_reads == int(wl.region_read_off[g + 1] - r0)
        assert rg.n_haps == int(wl.region_hap_off[g + 1] - wl.region_hap_off[g])
        reads = ctypes.cast(rg.reads, ctypes.POINTER(native.RawRead))
        for k in (0, rg.n_reads - 1):
            rd, r = reads[k], r0 + k
            off = int(wl.read_off[r])
            assert rd.length == int(wl.read_off[r + 1] - off) and rd.mapping_quality == int(mapq[r])
            assert rd.bases == wl.bases.ctypes.data + off and rd.quals == wl.quals.ctypes.data + off
            assert rd.ins_quals == wl.ins.ctypes.data + off and rd.del_quals == wl.dels.ctypes.data + off
        haps = ctypes.cast(rg.haps, ctypes.POINTER(native.Hap))
        h0 = int(wl.region_hap_off[g])
        assert ctypes.cast(haps[0].bases, ctypes.c_void_p).value == wl.hap_bases.ctypes.data + int(wl.hap_off[h0])
        assert haps[0].length == int(wl.hap_off[h0 + 1] - wl.hap_off[h0])


def test_raw_table_without_tags_has_null_tag_pointers():
    wl, mapq = _wl()
    regs = ctypes.cast(W.as_raw_regions(wl, mapq, False), ctypes.POINTER(native.RawRegion))
    rd = ctypes.cast(regs[1].reads, ctypes.POINTER(native.RawRead))[0]
    assert rd.ins_quals is None and rd.del_quals is None


def test_region_table_reads_back():
    wl, _ = _wl()
    regs = wl.as_regions()
    for g in range(wl.n_regions):
        rg = regs[g]
        r0 = int(wl.region_read_off[g])
        rd = rg.reads[rg.n_reads - 1]
        r = r0 + rg.n_reads - 1
        off = int(wl.read_off[r])
        assert rd.length == int(wl.read_off[r + 1] - off)
        for name, plane in (("bases", wl.bases), ("quals", wl.quals), ("ins_gop", wl.ins), ("del_gop", wl.dels),
                            ("gcp", wl.gcp)):
            assert ctypes.cast(getattr(rd, name), ctypes.c_void_p).value == plane.ctypes.data + off


def test_pd_tables_read_back():
    wl, mapq = _wl()
    pd = W.pd_flags(wl, 3)
    for base, read_t in ((W.as_pd_regions(wl, pd), native.Read), (W.as_pd_raw_regions(wl, pd, mapq), native.RawRead)):
        regs = ctypes.cast(base, ctypes.POINTER(native.PdRegion))
        for g in range(wl.n_regions):
            rg = regs[g]
            h0 = int(wl.region_hap_off[g])
            hp = ctypes.cast(rg.haps, ctypes.POINTER(native.PdHap))[rg.n_haps - 1]
            h = h0 + rg.n_haps - 1
            assert hp.length == int(wl.hap_off[h + 1] - wl.hap_off[h])
            assert ctypes.cast(hp.pd_bases, ctypes.c_void_p).value is not None
            rd = ctypes.cast(rg.reads, ctypes.POINTER(read_t))[0]
            r0 = int(wl.region_read_off[g])
            assert rd.length == int(wl.read_off[r0 + 1] - wl.read_off[r0])
            if read_t is native.RawRead:
                assert rd.mapping_quality == int(mapq[r0])
