"""Iterative drivers over many cone-beam scans in single persistent launches.

The reference's iterative scripts (python/SART.py, python/EM.py,
python/ASD_POCS.py) advance one scan, one projector call and one element-wise
line at a time.  ``BatchedSolver`` advances many scans of uneven volume and
detector sizes together: one update is, per ordered subset, one batched
forward projection (``ctgb_batch_forward``: a transpose launch and one
persistent launch per dominant axis over every (scan, view, detector tile)
item), with the driver's residual line fused into the projector's store, and
one batched backprojection (``ctgb_batch_backproject``: an integration launch
and one persistent launch over every (scan, voxel-column block) item), with
the driver's update line fused into the backprojector's store.  The plans
(per-scan descriptors, view lists, TMA tensor maps) are built once on the host
and copied to the device; a step is launches only, so it captures into a CUDA
graph.  The persistent grid sizes (CTAs per SM) are chosen by a
``TileAutotuner`` (CUDA-event timing of the candidates, cached per batch
signature).

The per-scan state (iterate, normalisers, subset projectors, scratch) is the
single-scan solvers' (``iterative.SART``, ``MLEM``, ``OSSART``), so a batched
run and the solvers run one by one give the same bits.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .fanbeam import TileAutotuner
from .iterative import MLEM, OSSART, SART
from .projector import _ptr, _stream

# Persistent CTAs per SM tried by the autotuner: the forward kernel runs one
# warp per CTA (up to 16 or 24 resident), the batched backprojectors 128
# threads (up to 4 resident).
FWD_CTAS = (4, 8, 16)
BP_CTAS = (2, 3, 4)
FWD_TUNER = TileAutotuner(candidates=FWD_CTAS, reps=2)
BP_TUNER = TileAutotuner(candidates=BP_CTAS, reps=2)


class Plan:
    """One batched launch: the plan's host bytes (launch sizes) and their
    device copy (the jobs the kernels read), built once."""

    def __init__(self, kind, jobs, device, matched=False):
        if kind not in ("forward", "backproject"):
            raise ValueError("kind must be 'forward' or 'backproject'")
        self.kind, self.matched = kind, bool(matched)
        cls = _lib.CtgbFwdJob if kind == "forward" else _lib.CtgbBpJob
        arr = (cls * len(jobs))(*jobs)
        n = ctypes.c_size_t(0)
        if kind == "forward":
            _lib.call("ctgb_batch_forward_plan_bytes", arr, len(jobs), ctypes.byref(n))
        else:
            _lib.call("ctgb_batch_backproject_plan_bytes", arr, len(jobs), ctypes.byref(n))
        raw = np.zeros(n.value + 128, dtype=np.uint8)          # 128-byte aligned host copy
        off = (-raw.ctypes.data) % 128
        self.host = raw[off:off + n.value]
        hp = ctypes.c_void_p(self.host.ctypes.data)
        if kind == "forward":
            _lib.call("ctgb_batch_forward_plan", arr, len(jobs), hp, n.value)
        else:
            _lib.call("ctgb_batch_backproject_plan", arr, len(jobs), int(self.matched), hp, n.value)
        self.dev = torch.from_numpy(self.host.copy()).to(device)
        if self.dev.data_ptr() % 128:
            raise RuntimeError("device plan not 128-byte aligned")

    def launch(self, ctas_per_sm):
        fn = "ctgb_batch_forward" if self.kind == "forward" else "ctgb_batch_backproject"
        _lib.call(fn, ctypes.c_void_p(self.host.ctypes.data), _ptr(self.dev), int(ctas_per_sm), _stream())


def _vp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _workspace(P, nviews, device):
    n = ctypes.c_size_t(0)
    _lib.call("ctgb_backproject_fdk_workspace_bytes", ctypes.byref(P.c), int(nviews), ctypes.byref(n))
    return torch.empty((n.value + 3) // 4, dtype=torch.float32, device=device), n.value


class BatchedSolver:
    """One iteration of many single-scan solvers (all SART, all MLEM or all
    OSSART) as batched, fused launches.  ``step()`` issues it; ``capture()``
    records it into a CUDA graph (after one eager step, which tunes the
    persistent grids and advances the state) and ``run(n)`` replays it."""

    def __init__(self, solvers, fwd_tuner=FWD_TUNER, bp_tuner=BP_TUNER):
        self.solvers = list(solvers)
        kinds = {type(s) for s in self.solvers}
        if len(kinds) != 1 or kinds.pop() not in (SART, MLEM, OSSART):
            raise ValueError("a batch holds solvers of one kind: SART, MLEM or OSSART")
        self.device = self.solvers[0].device
        self.graph = None
        self._keep = []                 # per-scan buffers the plans point at
        self.fwd_tuner, self.bp_tuner = fwd_tuner, bp_tuner
        self.fwd_ctas = self.bp_ctas = None
        s0 = self.solvers[0]
        if isinstance(s0, OSSART):
            nsub = len(s0.subsets)
            self.plans = [self._plans_ossart(k) for k in range(nsub)]
        else:
            self.plans = [self._plans_full()]

    # -- plans ---------------------------------------------------------------------
    def _scan_buffers(self, s, P, nviews):
        nz, ny, nx = P.volume_shape
        xzy = torch.empty((nz, nx, ny), dtype=torch.float32, device=self.device)
        ws, wsb = _workspace(P, nviews, self.device)
        self._keep += [xzy, ws]
        return xzy, ws, wsb

    def _plans_ossart(self, k):
        fj, bj = [], []
        for s in self.solvers:
            Ps, ps0, a1, b1 = s.subsets[k]
            if not hasattr(s, "_batch_bufs"):
                s._batch_bufs = self._scan_buffers(s, Ps, ps0.shape[0])
            xzy, ws, wsb = s._batch_bufs
            nv = ps0.shape[0]
            fj.append(_lib.CtgbFwdJob(ctypes.pointer(Ps.c), _vp(Ps.table), _vp(s.x), _vp(xzy), _vp(s.S.res), 0, nv,
                                      _lib.FWD_POCS_RESIDUAL, s.eps, _vp(ps0), _vp(a1)))
            bj.append(_lib.CtgbBpJob(ctypes.pointer(Ps.c), _vp(Ps.table), _vp(s.S.res), None, _vp(ws), wsb, 0, nv,
                                     1.0, 0, _lib.BP_POCS_UPDATE, s.lam, s.eps, _vp(s.x), _vp(b1)))
        return (Plan("forward", fj, self.device), Plan("backproject", bj, self.device, matched=s.matched))

    def _plans_full(self):
        fj, bj = [], []
        for s in self.solvers:
            P = s.P
            nv = P.params.NumberOfViews
            xzy, ws, wsb = self._scan_buffers(s, P, nv)
            scale = 1.0 if s.matched else P.params.dtheta      # backward(): dtheta; matched: A^T
            if isinstance(s, SART):
                fj.append(_lib.CtgbFwdJob(ctypes.pointer(P.c), _vp(P.table), _vp(s.x), _vp(xzy), _vp(s.S.res), 0, nv,
                                          _lib.FWD_SART_RESIDUAL, s.eps, _vp(s.proj0), _vp(s.norm2)))
                bj.append(_lib.CtgbBpJob(ctypes.pointer(P.c), _vp(P.table), _vp(s.S.res), None, _vp(ws), wsb, 0, nv,
                                         scale, 0, _lib.BP_SART_UPDATE, s.alpha, s.eps, _vp(s.x), _vp(s.norm1)))
            else:
                fj.append(_lib.CtgbFwdJob(ctypes.pointer(P.c), _vp(P.table), _vp(s.x), _vp(xzy), _vp(s.S.res), 0, nv,
                                          _lib.FWD_EM_RATIO, s.eps, _vp(s.proj0), None))
                bj.append(_lib.CtgbBpJob(ctypes.pointer(P.c), _vp(P.table), _vp(s.S.res), None, _vp(ws), wsb, 0, nv,
                                         scale, 0, _lib.BP_EM_UPDATE, 0.0, 0.0, _vp(s.x), _vp(s.norm)))
        return (Plan("forward", fj, self.device), Plan("backproject", bj, self.device, matched=s.matched))

    # -- tuning, stepping, graphs ---------------------------------------------------
    def signature(self):
        return (type(self.solvers[0]).__name__,
                tuple((s.P.volume_shape, s.P.proj_shape()) for s in self.solvers))

    def tune(self):
        """Choose the persistent grids (CTAs per SM) by timing the first
        subset's launches; the iterates are restored afterwards."""
        if self.fwd_ctas is not None:
            return
        saved = [s.x.clone() for s in self.solvers]
        fp, bp = self.plans[0]
        self.fwd_ctas = self.fwd_tuner.best(("fwd",) + self.signature(), fp.launch)
        self.bp_ctas = self.bp_tuner.best(("bp",) + self.signature(), bp.launch)
        for s, x in zip(self.solvers, saved):
            s.x.copy_(x)
        torch.cuda.synchronize(self.device)

    def step(self):
        self.tune()
        for fp, bp in self.plans:
            fp.launch(self.fwd_ctas)
            bp.launch(self.bp_ctas)

    def launches_per_step(self):
        """Kernel launches one step() makes."""
        n = 0
        for fp, bp in self.plans:
            head = fp.host[:64].view(np.int32)
            ngroups, ntrans = int(head[1]), int(head[2])
            n += ngroups + (1 if ntrans > 0 else 0) + 2
        return n

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


def batched_os_sart(scans, nsubsets=10, lam=0.8, eps=1e-5):
    """OS-SART (iterative.OSSART) over many (projector, projections) scans."""
    return BatchedSolver([OSSART(P, p, nsubsets=nsubsets, lam=lam, eps=eps) for P, p in scans])


def batched_mlem(scans, eps=1e-5, matched=False):
    """MLEM (EM.py, iterative.MLEM) over many (projector, projections) scans."""
    return BatchedSolver([MLEM(P, p, eps=eps, matched=matched) for P, p in scans])


def batched_sart(scans, alpha=1.0, eps=1e-5, matched=False):
    """SART (SART.py, iterative.SART) over many (projector, projections) scans."""
    return BatchedSolver([SART(P, p, alpha=alpha, eps=eps, matched=matched) for P, p in scans])
