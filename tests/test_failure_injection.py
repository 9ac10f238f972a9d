"""Failure detection without a GPU fault: the host-side injection hooks of ghmm_debug_inject and the loader's
"unsupported" report.  Refused device allocations must come back as status codes with the context still usable;
forced FP64 reruns must give FP64 results; an unsupported machine must surface as HardwareFeatureException, the
exception GATK's fallback chain catches (VectorLoglessPairHMM.java:60-79, PairHMM.java:79-98)."""
import numpy as np
import pytest

from gatk_gb300 import native


def test_loader_reports_unsupported_hardware(monkeypatch):
    from gatk_gb300.pairhmm import CudaLoglessPairHMM, HardwareFeatureException

    monkeypatch.setenv("GHMM_REPORT_UNSUPPORTED", "1")
    assert native.lib().ghmm_load() == 0
    with pytest.raises(HardwareFeatureException):
        CudaLoglessPairHMM()


@pytest.mark.gpu
def test_loader_report_is_a_switch(monkeypatch):
    monkeypatch.setenv("GHMM_REPORT_UNSUPPORTED", "0")
    assert native.lib().ghmm_load() == 1
    monkeypatch.setenv("GHMM_REPORT_UNSUPPORTED", "yes")
    assert native.lib().ghmm_load() == 0


@pytest.mark.gpu
def test_refused_allocation_is_reported_and_the_context_survives():
    from gatk_gb300 import workload as W
    from gatk_gb300.pairhmm import Engine
    from oracle import oracle as O

    wl = W.generate(1, regions=3)
    e = Engine()
    try:
        native.check(e.L.ghmm_debug_inject(e.handle, native.INJECT_REFUSE_ALLOCATIONS, 1), e.handle)
        with pytest.raises(native.GhmmError) as err:
            e.compute(wl)
        assert err.value.code == native.GHMM_ERR_NOMEM
        native.check(e.L.ghmm_debug_inject(e.handle, native.INJECT_REFUSE_ALLOCATIONS, 0), e.handle)
        got = e.compute(wl)  # the same context, afterwards
        assert np.abs(got - O.compute_workload(wl)).max() <= 1e-3
    finally:
        e.L.ghmm_debug_inject(e.handle, native.INJECT_REFUSE_ALLOCATIONS, 0)
        e.close()


@pytest.mark.gpu
def test_forced_reruns_give_fp64_results():
    from gatk_gb300 import workload as W
    from gatk_gb300.pairhmm import Engine
    from oracle import oracle as O

    wl = W.generate(1, regions=4)
    ref = O.compute_workload(wl)
    e = Engine()
    try:
        native.check(e.L.ghmm_debug_inject(e.handle, native.INJECT_FP64_RERUN_EVERY, 5), e.handle)
        with e.batch(wl) as b:
            b.forward(native.MODE_FP32_RERUN)
            got = b.results()
            st = b.stats()
    finally:
        e.L.ghmm_debug_inject(e.handle, native.INJECT_FP64_RERUN_EVERY, 0)
        e.close()
    forced = np.arange(wl.n_pairs) % 5 == 0
    assert st["n_rerun"] >= int(forced.sum())
    assert np.abs(got[forced] - ref[forced]).max() <= 1e-9
    assert np.abs(got - ref).max() <= 1e-3


def test_injection_constants_match_the_header():
    import os
    import re

    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ghmm.h")).read()
    defs = dict(re.findall(r"#define (GHMM_INJECT_\w+) (\d+)", hdr))
    assert int(defs["GHMM_INJECT_REFUSE_ALLOCATIONS"]) == native.INJECT_REFUSE_ALLOCATIONS
    assert int(defs["GHMM_INJECT_FP64_RERUN_EVERY"]) == native.INJECT_FP64_RERUN_EVERY
