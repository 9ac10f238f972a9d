"""Gap-penalty calibration: a differentiable PairHMM over the DRAGstr (period, repeat) parameter table.

GATK's DRAGstr mode gives every read position the gap-open (GOP) and gap-continuation (GCP) penalties of
the short tandem repeat it sits in: DragstrReadSTRAnalyzer finds each position's most repeated period and
its repeat count (DragstrReadSTRAnalyzer.java:110-136), DragstrParams looks the pair up in 8 x 20 tables
(DragstrParams.java:194-220) and DragstrPairHMMInputScoreImputator feeds them to the PairHMM with the last
position fixed at 45 / 10 (DragstrPairHMMInputScoreImputator.java:54-88).

Here the table is a [8, 20, 2] tensor theta of log10 probabilities (theta[p-1, r-1, 0] = gap open,
[..., 1] = gap continuation) and the likelihood is differentiable in it: the forward and the hand-written
backward run in libghmm.so (calib.cu) and are exposed as a torch.autograd.Function, so the penalties can be
fitted by maximum likelihood.  All computation is on the GPU; torch supplies device memory and autograd.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native
from .workload import Workload

MAX_PERIOD = 8
MAX_REPEAT = 20
LAST_GAP_OPEN = -4.5  # Phred 45 (DragstrPairHMMInputScoreImputator.java:22)
LAST_GAP_CONT = -1.0  # Phred 10 (:23)


def str_parameter_index(bases: np.ndarray) -> np.ndarray:
    """Per read position: index (period-1)*20 + (repeats-1) into the flattened table, clamped to the
    table's 8 x 20 (DragstrParams.lookup, DragstrParams.java:194-199); the last position is -1 (fixed)."""
    b = np.ascontiguousarray(bases, dtype=np.uint8)
    n = len(b)
    bp = np.zeros(n, dtype=np.int32)
    br = np.zeros(n, dtype=np.int32)
    if n:
        rc = native.lib().ghmm_str_analyze(b.ctypes.data_as(native._u8p), n, MAX_PERIOD,
                                           bp.ctypes.data_as(native._i32p), br.ctypes.data_as(native._i32p), None)
        if rc != 0:
            raise ValueError("ghmm_str_analyze failed")
    idx = (np.minimum(bp, MAX_PERIOD) - 1) * MAX_REPEAT + (np.minimum(np.maximum(br, 1), MAX_REPEAT) - 1)
    idx = idx.astype(np.int64)
    if n:
        idx[-1] = -1
    return idx


def default_theta():
    """A starting table: gap open Phred 45 everywhere, gap continuation round(1000/period)/100 as DRAGstr's
    default GCP (DragstrParams.java:114-117), both as log10 probabilities."""
    import torch

    t = torch.empty(MAX_PERIOD, MAX_REPEAT, 2, dtype=torch.float32)
    t[..., 0] = -4.5
    for p in range(1, MAX_PERIOD + 1):
        t[p - 1, :, 1] = -(round(1000.0 / p) / 100.0) / 10.0
    return t


class CalibrationSet:
    """Every (read, haplotype) pair of a workload on the GPU, with each read position's table index."""

    def __init__(self, wl: Workload, device: str = "cuda:0"):
        import torch

        self.wl = wl
        self.device = torch.device(device)
        pr, ph = wl.pair_index()
        idx = np.empty(len(wl.bases), dtype=np.int64)
        for r in range(wl.n_reads):
            a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
            idx[a:b] = str_parameter_index(wl.bases[a:b])
        self.param_index_np = idx
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).astype(dt)).to(self.device)
        self.bases = t(wl.bases, np.uint8)
        self.quals = t(wl.quals, np.uint8)
        self.read_off = t(wl.read_off, np.int64)
        self.hap_bases = t(wl.hap_bases, np.uint8)
        self.hap_off = t(wl.hap_off, np.int64)
        self.pair_read = t(pr, np.int32)
        self.pair_hap = t(ph, np.int32)
        self.param_index = t(idx, np.int64)
        self.n_pairs = len(pr)
        self.max_read_len = int(wl.read_lengths().max()) if wl.n_reads else 1
        self.max_hap_len = int(wl.hap_lengths().max()) if wl.n_haps else 1
        self.cells = wl.cells()
        self._ii = None

    def position_params(self, theta):
        """(gap_open, gap_cont) per read position from the [8, 20, 2] table (differentiable in theta)."""
        import torch

        # gathered in FP64 so that the backward's index_add sums the 10^5-10^6 per-position gradients into the
        # table in FP64 (index_select's backward is an atomic index_add; advanced indexing's sorts the
        # positions and costs tens of milliseconds)
        flat = theta.reshape(-1, 2).to(self.device, torch.float64)
        if self._ii is None:
            self._ii = self.param_index.clamp(min=0)
            self._fixed = self.param_index < 0
            self._last = (torch.full_like(self._ii, 0, dtype=torch.float64) + LAST_GAP_OPEN,
                          torch.full_like(self._ii, 0, dtype=torch.float64) + LAST_GAP_CONT)
        g = torch.where(self._fixed, self._last[0], torch.index_select(flat[:, 0], 0, self._ii))
        c = torch.where(self._fixed, self._last[1], torch.index_select(flat[:, 1], 0, self._ii))
        return g.float().contiguous(), c.float().contiguous()

    def batch(self, gap_open, gap_cont) -> native.CalibBatch:
        return native.CalibBatch(self.bases.data_ptr(), self.quals.data_ptr(), self.read_off.data_ptr(),
                                 self.hap_bases.data_ptr(), self.hap_off.data_ptr(), self.pair_read.data_ptr(),
                                 self.pair_hap.data_ptr(), gap_open.data_ptr(), gap_cont.data_ptr(), self.n_pairs,
                                 self.max_read_len, self.max_hap_len)


def _function():
    import torch

    class PairHMMLog10Likelihood(torch.autograd.Function):
        """log10 L of every pair as a function of per-position (gap_open, gap_cont); backward through the
        hand-written adjoint kernel (ghmm_calib_backward)."""

        @staticmethod
        def forward(ctx, gap_open, gap_cont, cs, engine, precision):
            out = torch.empty(cs.n_pairs, dtype=torch.float64, device=cs.device)
            b = cs.batch(gap_open, gap_cont)
            torch.cuda.synchronize(cs.device)
            native.check(engine.L.ghmm_calib_forward(engine.handle, ctypes.byref(b), precision, out.data_ptr()),
                         engine.handle)
            ctx.save_for_backward(gap_open, gap_cont)
            ctx.cs, ctx.engine, ctx.precision = cs, engine, precision
            return out

        @staticmethod
        def backward(ctx, grad_out):
            gap_open, gap_cont = ctx.saved_tensors
            cs, engine = ctx.cs, ctx.engine
            w = grad_out.detach().to(torch.float64).contiguous()
            go = torch.zeros_like(gap_open)
            gc = torch.zeros_like(gap_cont)
            ll = torch.empty(cs.n_pairs, dtype=torch.float64, device=cs.device)
            b = cs.batch(gap_open, gap_cont)
            torch.cuda.synchronize(cs.device)
            native.check(engine.L.ghmm_calib_backward(engine.handle, ctypes.byref(b), ctx.precision, w.data_ptr(),
                                                      ll.data_ptr(), go.data_ptr(), gc.data_ptr()), engine.handle)
            return go, gc, None, None, None

    return PairHMMLog10Likelihood


_FN = None


def log10_likelihoods(theta, cs: CalibrationSet, engine, precision: int = 0):
    """Per-pair log10 likelihood under the table theta (differentiable)."""
    global _FN
    if _FN is None:
        _FN = _function()
    g, c = cs.position_params(theta)
    return _FN.apply(g, c, cs, engine, precision)


def fit(cs: CalibrationSet, engine, theta0=None, steps: int = 50, lr: float = 0.05):
    """Maximum-likelihood fit of the table by Adam on -sum log10 L; returns (theta, history of sum log10 L)."""
    import torch

    theta = (default_theta() if theta0 is None else theta0.clone()).to(cs.device).requires_grad_(True)
    opt = torch.optim.Adam([theta], lr=lr)
    hist = []
    for _ in range(steps):
        opt.zero_grad()
        s = log10_likelihoods(theta, cs, engine).sum()
        (-s).backward()
        opt.step()
        with torch.no_grad():  # log10 probabilities of gap events stay below log10(1/2)
            theta.clamp_(max=-0.31)
        hist.append(float(s.detach()))
    return theta.detach(), hist
