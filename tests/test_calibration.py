"""Gap-penalty calibration (workload 3: 4,096 read x haplotype pairs around short tandem repeats).

The forward log10 likelihoods and the hand-written backward (calib.cu) are checked against the FP64
oracle (oracle_grad.c: forward and adjoint gradient over full matrices, every pair) and against FP64 central
finite differences with step 1e-4 computed with the GPU's FP64 forward, on every entry of the 8 x 20 x 2 table
that a read position uses (the unused ones must have zero gradient); the tolerance on the gradient is 1e-3
relative (scaled by the largest component).
"""
import numpy as np
import pytest

from gatk_gb300 import calibration as C
from gatk_gb300 import workload as W
from oracle import oracle as O


def test_str_parameter_index_layout():
    idx = C.str_parameter_index(np.frombuffer(b"ACACACACGTTTTTGA", dtype=np.uint8))
    assert idx[-1] == -1
    assert ((idx[:-1] >= 0) & (idx[:-1] < C.MAX_PERIOD * C.MAX_REPEAT)).all()
    # inside the ACAC... run the best period is 2
    assert (idx[2:6] // C.MAX_REPEAT == 1).all()
    # the TTTTT homopolymer: period 1, 5 repeats
    assert idx[11] == 0 * C.MAX_REPEAT + (5 - 1)


def test_default_theta():
    torch = pytest.importorskip("torch")
    t = C.default_theta()
    assert tuple(t.shape) == (8, 20, 2)
    assert torch.all(t[..., 0] == -4.5)
    assert abs(float(t[0, 0, 1]) + 1.0) < 1e-6 and abs(float(t[2, 0, 1]) + 0.333) < 1e-6


def _oracle_pair(wl, cs, g, c, p, grad=False):
    pr, ph = wl.pair_index()
    r, h = int(pr[p]), int(ph[p])
    a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
    args = (wl.hap(h), wl.bases[a:b], wl.quals[a:b], g[a:b].astype(np.float64), c[a:b].astype(np.float64))
    return O.cont_grad(*args) if grad else O.cont_forward(*args)


@pytest.fixture(scope="module")
def calib():
    torch = pytest.importorskip("torch")
    from gatk_gb300.pairhmm import Engine

    e = Engine()
    wl = W.generate(3)
    cs = C.CalibrationSet(wl)
    yield torch, e, wl, cs
    e.close()


@pytest.mark.gpu
def test_forward_matches_oracle(calib):
    torch, e, wl, cs = calib
    theta = C.default_theta()
    g, c = cs.position_params(theta)
    ll32 = C.log10_likelihoods(theta, cs, e, precision=0).cpu().numpy()
    ll64 = C.log10_likelihoods(theta, cs, e, precision=1).cpu().numpy()
    gn, cn = g.cpu().numpy(), c.cpu().numpy()
    for p in range(0, cs.n_pairs, 64):
        ref = _oracle_pair(wl, cs, gn, cn, p)
        assert abs(ll64[p] - ref) <= 1e-9
        assert abs(ll32[p] - ref) <= 1e-3


@pytest.mark.gpu
def test_backward_matches_oracle_gradient(calib):
    torch, e, wl, cs = calib
    theta = C.default_theta()
    g, c = cs.position_params(theta)
    g = g.detach().requires_grad_(True)
    c = c.detach().requires_grad_(True)
    fn = C._function() if C._FN is None else C._FN
    for precision, tol in ((0, 1e-3), (1, 1e-6)):  # gradients are returned as float32
        g.grad = None
        c.grad = None
        ll = fn.apply(g, c, cs, e, precision)
        ll.sum().backward()
        gg, gc = g.grad.cpu().numpy(), c.grad.cpu().numpy()
        gn, cn = g.detach().cpu().numpy(), c.detach().cpu().numpy()
        pr, _ = wl.pair_index()
        for p in range(cs.n_pairs):  # every pair; each read has one pair here, so per-position gradients are per pair
            _, dg, dc = _oracle_pair(wl, cs, gn, cn, p, grad=True)
            r = int(pr[p])
            a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
            scale = max(np.abs(dg).max(), np.abs(dc).max())
            assert np.abs(gg[a:b] - dg).max() <= tol * scale + 1e-9, (p, precision)
            assert np.abs(gc[a:b] - dc).max() <= tol * scale + 1e-9, (p, precision)


@pytest.mark.gpu
def test_theta_gradient_matches_fp64_central_differences(calib):
    torch, e, wl, cs = calib
    theta = C.default_theta().to(cs.device).requires_grad_(True)
    s = C.log10_likelihoods(theta, cs, e, precision=0).sum()
    s.backward()
    grad = theta.grad.detach().cpu().numpy().reshape(-1, 2)
    # every table entry some read position uses; the others get exactly zero gradient
    used = np.bincount(cs.param_index_np[cs.param_index_np >= 0], minlength=160)
    order = np.nonzero(used)[0]
    assert len(order) > 8
    assert (grad[used == 0] == 0).all()
    h = 1e-4
    scale = np.abs(grad).max()
    with torch.no_grad():
        for k in order:
            for comp in (0, 1):
                tp = theta.detach().clone()
                tm = theta.detach().clone()
                tp.view(-1, 2)[k, comp] += h
                tm.view(-1, 2)[k, comp] -= h
                sp = float(C.log10_likelihoods(tp, cs, e, precision=1).sum())
                sm = float(C.log10_likelihoods(tm, cs, e, precision=1).sum())
                # the table is float32: divide by the step actually stored, not by 2h
                step = float(tp.view(-1, 2)[k, comp].double() - tm.view(-1, 2)[k, comp].double())
                fd = (sp - sm) / step
                assert abs(grad[k, comp] - fd) <= 1e-3 * max(abs(fd), 1e-2 * scale), (k, comp, grad[k, comp], fd)


def _long_read_workload():
    """Reads of one to four 256-row strips (and one short read in the same batch), some longer than their
    haplotype, sampled with 2-4 % substitutions so that the FP32 pass underflows for some and redoes them in FP64."""
    rng = np.random.default_rng(17)
    regions = []
    # (the reads stay within a few hundred decades of likelihood: far below that the oracle's unscaled FP64 adjoints
    # underflow, while the kernel's, seeded with w / L, do not)
    for R, H, sub in ((300, 420, 0.02), (513, 600, 0.03), (330, 300, 0.02), (1000, 1200, 0.04), (257, 257, 0.02),
                      (256, 500, 0.02), (150, 900, 0.02), (2, 40, 0.0)):
        base = rng.choice(list(b"ACGT"), size=H).astype(np.uint8)
        start = int(rng.integers(0, max(1, H - R + 1)))
        rd = np.concatenate([base[start:start + R], rng.choice(list(b"ACGT"), size=max(0, R - H)).astype(np.uint8)])[:R]
        flip = rng.random(R) < sub
        rd[flip] = rng.choice(list(b"ACGT"), size=int(flip.sum())).astype(np.uint8)
        regions.append(([base.tobytes()], [(rd, rng.integers(10, 41, size=R), np.full(R, 45), np.full(R, 45),
                                             np.full(R, 10))]))
    return W.from_pairs(regions)


@pytest.mark.gpu
def test_reads_longer_than_one_strip_match_the_oracle(calib):
    # the strips of a long read pass their last row down (forward) and their first row's adjoints up (backward)
    torch, e, _, _ = calib
    wl = _long_read_workload()
    cs = C.CalibrationSet(wl)
    assert cs.max_read_len == 1000
    theta = C.default_theta()
    g, c = cs.position_params(theta)
    g = g.detach().requires_grad_(True)
    c = c.detach().requires_grad_(True)
    fn = C._function() if C._FN is None else C._FN
    gn, cn = g.detach().cpu().numpy(), c.detach().cpu().numpy()
    pr, _ = wl.pair_index()
    refs = [_oracle_pair(wl, cs, gn, cn, p, grad=True) for p in range(cs.n_pairs)]
    for precision, tol_l, tol_g in ((0, 1e-3, 1e-3), (1, 1e-9, 1e-6)):
        g.grad = None
        c.grad = None
        ll = fn.apply(g, c, cs, e, precision)
        ll.sum().backward()
        lln = ll.detach().cpu().numpy()
        gg, gc = g.grad.cpu().numpy(), c.grad.cpu().numpy()
        for p in range(cs.n_pairs):
            lref, dg, dc = refs[p]
            assert abs(lln[p] - lref) <= tol_l, (p, precision, lln[p], lref)
            r = int(pr[p])
            a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
            scale = max(np.abs(dg).max(), np.abs(dc).max())
            assert np.abs(gg[a:b] - dg).max() <= tol_g * scale + 1e-9, (p, precision)
            assert np.abs(gc[a:b] - dc).max() <= tol_g * scale + 1e-9, (p, precision)


@pytest.mark.gpu
def test_long_reads_forward_only_first_and_under_a_one_block_scratch_budget(monkeypatch):
    # A fresh context's first calibration call is a forward without backward over reads of several strips: their
    # boundary rows pass through scratch that this call itself has to reserve.  Then a scratch budget below one
    # warp's need leaves a single block of two warps, which takes all eight pairs in turn, reusing its scratch.
    torch = pytest.importorskip("torch")
    from gatk_gb300.pairhmm import Engine

    wl = _long_read_workload()
    cs = C.CalibrationSet(wl)
    theta = C.default_theta()
    g, c = cs.position_params(theta)
    gn, cn = g.detach().cpu().numpy(), c.detach().cpu().numpy()
    refs = [_oracle_pair(wl, cs, gn, cn, p, grad=True) for p in range(cs.n_pairs)]
    pr, _ = wl.pair_index()
    e = Engine()
    try:
        with torch.no_grad():
            for precision, tol in ((0, 1e-3), (1, 1e-9)):
                ll = C.log10_likelihoods(theta, cs, e, precision=precision).cpu().numpy()
                for p in range(cs.n_pairs):
                    assert abs(ll[p] - refs[p][0]) <= tol, (p, precision, ll[p], refs[p][0])
        monkeypatch.setenv("GHMM_CALIB_SCRATCH_BYTES", "1")
        fn = C._function() if C._FN is None else C._FN
        for precision, tol_l, tol_g in ((0, 1e-3, 1e-3), (1, 1e-9, 1e-6)):
            gg = g.detach().clone().requires_grad_(True)
            cc = c.detach().clone().requires_grad_(True)
            ll = fn.apply(gg, cc, cs, e, precision)
            ll.sum().backward()
            lln = ll.detach().cpu().numpy()
            dgn, dcn = gg.grad.cpu().numpy(), cc.grad.cpu().numpy()
            for p in range(cs.n_pairs):
                lref, dg, dc = refs[p]
                assert abs(lln[p] - lref) <= tol_l, (p, precision)
                r = int(pr[p])
                a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
                scale = max(np.abs(dg).max(), np.abs(dc).max())
                assert np.abs(dgn[a:b] - dg).max() <= tol_g * scale + 1e-9, (p, precision)
                assert np.abs(dcn[a:b] - dc).max() <= tol_g * scale + 1e-9, (p, precision)
    finally:
        e.close()


@pytest.mark.gpu
def test_fit_increases_likelihood(calib):
    torch, e, wl, cs = calib
    theta, hist = C.fit(cs, e, steps=8, lr=0.05)
    assert hist[-1] > hist[0]
    assert torch.isfinite(theta).all()
