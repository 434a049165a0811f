"""torch.autograd through the DD projector: the gradient of a least-squares
data term, checked against central finite differences of the FP64 oracle."""
import numpy as np
import pytest
import torch

from ctreconstruction_gb300 import Projector
from ctreconstruction_gb300.autograd import dd_backproject, dd_project
from oracle.oracle import OracleGeometry
from _util import cone_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [(24, 24, 16), (21, 19, 13)])
def test_gradient_matches_fp64_finite_differences(cuda, n):
    p = cone_params(n=n, nviews=10, nu=40, nv=30)
    P = Projector(p, device=cuda)
    g = OracleGeometry(p)
    rng = np.random.default_rng(4)
    x = rng.random(P.volume_shape).astype(np.float32)
    y = rng.random(P.proj_shape()).astype(np.float32)
    xt = torch.from_numpy(x).to(cuda).requires_grad_(True)
    loss = 0.5 * torch.sum((dd_project(xt, P) - torch.from_numpy(y).to(cuda)) ** 2)
    loss.backward()
    grad = xt.grad.double().cpu().numpy()

    def L(v):
        r = g.forward(v.astype(np.float32)) - y.astype(np.float64)
        return 0.5 * np.sum(r * r)

    for k in range(3):
        e = rng.standard_normal(x.shape)
        e /= np.linalg.norm(e)
        h = 1e-2
        # L is quadratic, so the central difference is exact up to rounding;
        # evaluate it in float64 on the oracle (x + h e rounded to float32 by
        # the projector's input type is avoided by differencing the linear part).
        Ae = g.forward(e.astype(np.float32))
        r0 = g.forward(x) - y
        fd = float(np.sum(r0 * Ae))
        an = float(np.sum(grad * e.astype(np.float32)))
        assert abs(fd - an) <= 1e-4 * max(abs(fd), 1e-12), (k, fd, an)
        # the literal central difference agrees with the directional derivative
        lp, lm = L(x + h * e), L(x - h * e)
        assert abs((lp - lm) / (2 * h) - fd) <= 1e-3 * abs(fd)


def test_backproject_op_gradient_is_forward(cuda):
    p = cone_params(n=(24, 20, 16), nviews=8, nu=36, nv=28)
    P = Projector(p, device=cuda)
    yt = torch.rand(P.proj_shape(), device=cuda, requires_grad=True)
    w = torch.rand(P.volume_shape, device=cuda)
    (dd_backproject(yt, P) * w).sum().backward()
    want = P.forward(w)
    assert torch.allclose(yt.grad, want, rtol=1e-5, atol=1e-6 * want.abs().max().item())


def test_batched_projection(cuda):
    p = cone_params(n=(20, 20, 12), nviews=6, nu=30, nv=20)
    P = Projector(p, device=cuda)
    xb = torch.rand((3,) + P.volume_shape, device=cuda)
    out = dd_project(xb, P)
    assert out.shape == (3,) + P.proj_shape()
    for i in range(3):
        assert torch.equal(out[i], P.forward(xb[i].contiguous()))
