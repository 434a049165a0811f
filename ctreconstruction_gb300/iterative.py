"""Iterative reconstruction drivers on the GB300 projectors.

Each driver restates one of the reference's scripts, with the same parameters
and the same update formulas (including where the reference places eps):

* ``sart``      python/SART.py:27-59   (all views per update, SIRT-like)
* ``mlem``      python/EM.py:20-44
* ``asd_pocs``  python/ASD_POCS.py:137-201 (POCS + TV descent, adaptive steps)
* ``os_sart``   ordered subsets of views (no reference counterpart)

The scripts call ``Reconstruction.forward()``/``backward()``; here those are
the device projectors (``Projector.forward`` / ``Projector.backproject_fdk``,
which is the reference's FDK-weighted backward()).  ``matched=True`` uses the
exact adjoint instead.  All arithmetic runs in libctgb kernels on device
tensors; the host only reads back the scalars the scripts branch on.
"""
import ctypes
import math

import torch

from . import _lib
from .geometry import ReconstructionParams
from .projector import Projector, _ptr, _stream


def _n(t):
    return int(t.numel())


class _Scratch:
    """Device work arrays of one driver run (allocated once, through torch)."""

    def __init__(self, P, device):
        self.P = P
        vshape, pshape = P.volume_shape, P.proj_shape()
        self.proj = torch.empty(pshape, dtype=torch.float32, device=device)
        self.res = torch.empty(pshape, dtype=torch.float32, device=device)
        self.bp = torch.empty(vshape, dtype=torch.float32, device=device)
        cnt = ctypes.c_int32(0)
        _lib.call("ctgb_partials_count", max(_n(self.bp), _n(self.proj)), ctypes.byref(cnt))
        self.partials = torch.empty(cnt.value, dtype=torch.float64, device=device)
        self.scalar = torch.empty(1, dtype=torch.float64, device=device)


def _sqdist(S, a, b=None):
    _lib.call("ctgb_sqdist", _ptr(a), _ptr(b) if b is not None else None, _n(a), _ptr(S.partials), _ptr(S.scalar),
              _stream())
    return S.scalar


def _backproject(P, proj, out, matched):
    if matched:
        return P.backproject_matched(proj, out=out)
    return P.backproject_fdk(proj, out=out)


def _rmse(S, x, phantom):
    return math.sqrt(_sqdist(S, x, phantom).item() / _n(x))


def normalisers(P, matched=False):
    """norm1 = backward(ones) (SART.py:31-35), norm2 = forward(ones) (:36-38)."""
    dev = P.device
    ones_p = torch.ones(P.proj_shape(), dtype=torch.float32, device=dev)
    norm1 = _backproject(P, ones_p, None, matched)
    norm2 = P.forward(torch.ones(P.volume_shape, dtype=torch.float32, device=dev))
    return norm1, norm2


class _Solver:
    """An iterative solver whose device state (iterate, normalisers, scratch)
    lives in tensors allocated once, so that one iteration is a fixed
    sequence of stream-ordered launches: ``step()`` issues it eagerly,
    ``capture()`` records it into a CUDA graph and ``run(n)`` replays that
    graph n times (one graph launch per iteration)."""

    graph = None

    def step(self):
        raise NotImplementedError

    def capture(self):
        """Record one iteration into a CUDA graph.  Runs one eager iteration
        first (it allocates the projectors' lazy buffers and sets kernel
        attributes outside the capture) — the state advances by it."""
        self.step()
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step()
        self.graph = g
        return g

    def run(self, niter, phantom=None):
        rmse = []
        for _ in range(niter):
            if self.graph is not None:
                self.graph.replay()
            else:
                self.step()
            if phantom is not None:
                rmse.append(_rmse(self.S, self.x, phantom))
        return rmse


class SART(_Solver):
    """SART.py:44-59: x <- x - alpha * (B((Ax - p0) / (A1 + eps)) / norm1 + eps).
    x0 defaults to zeros, as in the script."""

    def __init__(self, P, proj0, alpha=1.0, eps=1e-5, x0=None, matched=False, norms=None):
        self.P = P if isinstance(P, Projector) else Projector(P)
        self.device = dev = self.P.device
        self.S = _Scratch(self.P, dev)
        self.norm1, self.norm2 = norms if norms is not None else normalisers(self.P, matched)
        self.proj0, self.alpha, self.eps, self.matched = proj0, float(alpha), float(eps), matched
        self.x = torch.zeros(self.P.volume_shape, dtype=torch.float32, device=dev) if x0 is None else x0.clone()

    def step(self):
        S, x = self.S, self.x
        self.P.forward(x, out=S.proj)
        _lib.call("ctgb_sart_residual", _ptr(S.proj), _ptr(self.proj0), _ptr(self.norm2), self.eps, _ptr(S.res),
                  _n(S.proj), _stream())
        _backproject(self.P, S.res, S.bp, self.matched)
        # element-wise update, in place (each element reads only itself)
        _lib.call("ctgb_sart_update", _ptr(x), _ptr(S.bp), _ptr(self.norm1), self.alpha, self.eps, _ptr(x), _n(x),
                  _stream())


class MLEM(_Solver):
    """EM.py:32-44: x <- x * B(p0 / Ax) / B(1) with the script's zero guards.
    proj0 is modified in place where Ax == 0 (the script's proj0 aliases its
    measured data).  x0 defaults to ones, as in the script."""

    def __init__(self, P, proj0, eps=1e-5, x0=None, matched=False, norm=None):
        self.P = P if isinstance(P, Projector) else Projector(P)
        self.device = dev = self.P.device
        self.S = _Scratch(self.P, dev)
        if norm is None:
            norm = _backproject(self.P, torch.ones(self.P.proj_shape(), dtype=torch.float32, device=dev), None,
                                matched)
        self.norm, self.proj0, self.eps, self.matched = norm, proj0, float(eps), matched
        self.x = torch.ones(self.P.volume_shape, dtype=torch.float32, device=dev) if x0 is None else x0.clone()

    def step(self):
        S, x = self.S, self.x
        self.P.forward(x, out=S.proj)
        _lib.call("ctgb_em_ratio", _ptr(self.proj0), _ptr(S.proj), self.eps, _ptr(S.res), _n(S.proj), _stream())
        _backproject(self.P, S.res, S.bp, self.matched)
        _lib.call("ctgb_em_update", _ptr(x), _ptr(S.bp), _ptr(self.norm), _ptr(x), _n(x), _stream())


class OSSART(_Solver):
    """Ordered-subsets SART (no reference counterpart).

    Subset s holds views s, s + nsubsets, s + 2 nsubsets, ... — itself a
    regular scan (StartAngle + s * dtheta, the same angular span,
    NumberOfViews / nsubsets views), so each subset gets its own Projector.
    Each sub-iteration applies
        x <- max(0, x + lam * B_s((p0_s - A_s x) / (A_s 1 + eps)) / (B_s 1 + eps))
    with rows/voxels whose normaliser is zero left untouched; one step() is
    one pass over all subsets."""

    def __init__(self, P, proj0, nsubsets=10, lam=0.8, eps=1e-5, x0=None, matched=True):
        P = P if isinstance(P, Projector) else Projector(P)
        self.P, self.device = P, P.device
        dev = P.device
        base = P.params
        nv = base.NumberOfViews
        if nsubsets < 1 or nv % nsubsets:
            raise ValueError("NumberOfViews (%d) must be divisible by nsubsets (%d)" % (nv, nsubsets))
        span = base.EndAngle - base.StartAngle
        dth = span / nv
        vol_ones = torch.ones(P.volume_shape, dtype=torch.float32, device=dev)
        self.subsets = []
        for s in range(nsubsets):
            d = base.as_dict()
            d['StartAngle'] = base.StartAngle + s * dth
            d['EndAngle'] = d['StartAngle'] + span
            d['NumberOfViews'] = nv // nsubsets
            Ps = Projector(ReconstructionParams.from_dict(d, base.flavour), device=dev)
            ps0 = proj0[s::nsubsets].contiguous()
            a1 = Ps.forward(vol_ones)
            b1 = _backproject(Ps, torch.ones_like(ps0), None, matched)
            self.subsets.append((Ps, ps0, a1, b1))
        self.x = torch.zeros(P.volume_shape, dtype=torch.float32, device=dev) if x0 is None else x0.clone()
        self.S = _Scratch(self.subsets[0][0], dev)
        self.lam, self.eps, self.matched = float(lam), float(eps), matched

    def step(self):
        S, x = self.S, self.x
        for Ps, ps0, a1, b1 in self.subsets:
            Ps.forward(x, out=S.proj)
            _lib.call("ctgb_pocs_residual", _ptr(ps0), _ptr(S.proj), _ptr(a1), self.eps, _ptr(S.res), _n(S.res),
                      _stream())
            _backproject(Ps, S.res, S.bp, self.matched)
            _lib.call("ctgb_pocs_update", _ptr(x), _ptr(S.bp), _ptr(b1), self.lam, self.eps, _ptr(x), _n(x),
                      _stream())


class SolverBatch:
    """Many solvers (scans of uneven sizes) advanced together: one CUDA graph
    holds one iteration of every solver, so a batch iteration is a single
    graph launch.  Each solver's launches go to a stream of its own, forked
    from and joined back to the current stream (in the graph: independent
    branches), so the scans run concurrently — one small scan's launches
    alone do not fill the GPU."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        self.device = self.solvers[0].device
        self.graph = None
        self._side = None

    def step(self):
        main = torch.cuda.current_stream(self.device)
        if self._side is None:
            self._side = [torch.cuda.Stream(device=self.device) for _ in self.solvers]
        for s, st in zip(self.solvers, self._side):
            st.wait_stream(main)
            with torch.cuda.stream(st):
                s.step()
        for st in self._side:
            main.wait_stream(st)

    def capture(self):
        self.step()
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step()
        self.graph = g
        return g

    def run(self, niter):
        for _ in range(niter):
            if self.graph is not None:
                self.graph.replay()
            else:
                self.step()


def sart(P, proj0, niter=10, alpha=1.0, eps=1e-5, x0=None, phantom=None, matched=False, norms=None, graph=False):
    """SART.py:44-59; returns (x, rmse list)."""
    s = SART(P, proj0, alpha, eps, x0, matched, norms)
    if graph and niter > 0:
        x_start = s.x.clone()
        s.capture()                 # advances the state by one (eager warm-up) iteration
        s.x.copy_(x_start)
    return s.x, s.run(niter, phantom)


def mlem(P, proj0, niter=10, eps=1e-5, x0=None, phantom=None, matched=False, norm=None):
    """EM.py:32-44; returns (x, rmse list)."""
    s = MLEM(P, proj0, eps, x0, matched, norm)
    return s.x, s.run(niter, phantom)


def tv_descent(x, step, ng, eps=1e-7):
    """ng steps of x <- x - step * tv_grad(x) (ASD_POCS.py:188-190; tv_grad
    :55-77).  Returns a new tensor; x is not modified."""
    nz, ny, nx = x.shape
    cnt = ctypes.c_int32(0)
    _lib.call("ctgb_partials_count", _n(x), ctypes.byref(cnt))
    partials = torch.empty(cnt.value, dtype=torch.float64, device=x.device)
    bufs = (torch.empty_like(x), torch.empty_like(x))
    a = x
    for i in range(ng):
        out = bufs[i % 2]
        _lib.call("ctgb_tv_step", _ptr(a), _ptr(out), nz, ny, nx, eps, float(step), _ptr(partials), _stream())
        a = out
    return a.clone() if ng == 0 else a


def asd_pocs(P, proj0, niter=20, beta=1.0, beta_red=0.999, na=5, ng=20, alpha=0.007, r_max=0.99, alpha_red=0.95,
             eps=1e-7, x0=None, phantom=None, matched=False, norms=None, filter_type=None, cutoff=None, prox=None,
             on_tv=None, times=None):
    """ASD_POCS.py:137-201.  x0 defaults to the script's FBP start
    (Filtering() then backward() of proj0).  Returns (x, rmse list, log).

    prox: optional replacement of the TV-descent step (ASD_POCS.py:186-190):
    called as prox(x, plain) where plain() runs the script's ng TV steps on
    a copy and returns it; prox returns the new volume (it may return
    plain(), e.g. as a fallback).  on_tv(pre, post): called with the volume
    before and after each TV step (training pairs for a learned prox).
    times: optional list that receives the wall time (s, device-synchronised)
    at the end of every iteration."""
    import time as _time
    P = P if isinstance(P, Projector) else Projector(P)
    dev = P.device
    S = _Scratch(P, dev)
    norm1, norm2 = norms if norms is not None else normalisers(P, matched)
    if x0 is None:
        q = proj0.clone()
        P.filter(q, filter_type, cutoff)
        x = P.backproject_fdk(q)
    else:
        x = x0.clone()
    xn = torch.empty_like(x)
    f0 = torch.empty_like(x)
    tv_a, tv_b = torch.empty_like(x), torch.empty_like(x)
    n_p, n_v = _n(S.proj), _n(x)
    rmse, log = [], []
    nz, ny, nx = x.shape
    t0 = _time.perf_counter()
    for _ in range(niter):
        f0.copy_(x)
        for _a in range(na):
            P.forward(x, out=S.proj)
            _lib.call("ctgb_pocs_residual", _ptr(proj0), _ptr(S.proj), _ptr(norm2), eps, _ptr(S.res), n_p, _stream())
            _backproject(P, S.res, S.bp, matched)
            _lib.call("ctgb_pocs_update", _ptr(x), _ptr(S.bp), _ptr(norm1), beta, eps, _ptr(xn), n_v, _stream())
            x, xn = xn, x
        dp = math.sqrt(_sqdist(S, x, f0).item())
        dtvg = alpha * dp
        f0.copy_(x)

        def plain(src=x, step=dtvg):
            a, b = src, tv_a
            for _g in range(ng):
                _lib.call("ctgb_tv_step", _ptr(a), _ptr(b), nz, ny, nx, eps, float(step), _ptr(S.partials),
                          _stream())
                a, b = b, (tv_b if b is tv_a else tv_a)
            return a

        new = plain() if prox is None else prox(x, plain)
        if on_tv is not None:
            on_tv(f0, new)
        if new is not x:
            x.copy_(new)
        dg = math.sqrt(_sqdist(S, x, f0).item())
        if dg > r_max * dp:
            alpha *= alpha_red
        beta *= beta_red
        log.append({"dtvg": dtvg, "beta": beta, "dp": dp, "dg": dg, "alpha": alpha})
        if phantom is not None:
            rmse.append(_rmse(S, x, phantom))
        if times is not None:
            torch.cuda.synchronize(dev)
            times.append(_time.perf_counter() - t0)
    return x, rmse, log


def os_sart(P, proj0, nsubsets=10, niter=20, lam=0.8, eps=1e-5, x0=None, phantom=None, matched=True):
    """OSSART run for niter passes; returns (x, rmse list)."""
    s = OSSART(P, proj0, nsubsets, lam, eps, x0, matched)
    return s.x, s.run(niter, phantom)
