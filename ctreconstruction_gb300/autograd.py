"""The DD projector as a differentiable torch operation.

``dd_project(vol, projector)`` returns A vol; its gradient is the matched
backprojector A^T (``ctgb_backproject_matched``), the exact adjoint of the
forward kernel, so autograd through reconstruction losses is consistent with
the forward to float32 rounding.  ``dd_backproject`` is the adjoint
operation, whose gradient is A.  Both accept a single volume [nz, ny, nx] /
projection stack [nviews, nv, nu] or a batch with a leading dimension.
"""
import torch

from .projector import Projector


class _DDProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vol, projector):
        ctx.projector = projector
        return _apply(projector.forward, vol, projector.volume_shape)

    @staticmethod
    def backward(ctx, grad):
        P = ctx.projector
        return _apply(P.backproject_matched, grad, P.proj_shape()), None


class _DDBackprojection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, proj, projector):
        ctx.projector = projector
        return _apply(projector.backproject_matched, proj, projector.proj_shape())

    @staticmethod
    def backward(ctx, grad):
        P = ctx.projector
        return _apply(P.forward, grad, P.volume_shape), None


def _apply(fn, t, shape):
    t = t.contiguous()
    if t.dim() == len(shape):
        return fn(t)
    if t.dim() == len(shape) + 1:
        return torch.stack([fn(t[i].contiguous()) for i in range(t.shape[0])])
    raise ValueError("expected shape %s or a batch of it, got %s" % (tuple(shape), tuple(t.shape)))


def dd_project(vol, projector):
    """A vol, differentiable (gradient: matched backprojection)."""
    if not isinstance(projector, Projector):
        projector = Projector(projector)
    return _DDProjection.apply(vol, projector)


def dd_backproject(proj, projector):
    """A^T proj, differentiable (gradient: forward projection)."""
    if not isinstance(projector, Projector):
        projector = Projector(projector)
    return _DDBackprojection.apply(proj, projector)
