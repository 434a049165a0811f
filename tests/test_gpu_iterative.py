"""Iterative drivers (SART.py, EM.py, ASD_POCS.py restated) on the GPU
against the same loops over the FP64 oracle, a few iterations each.
Bar: max|gpu - oracle| / max|oracle| <= 1e-4 on the volume."""
import numpy as np
import pytest
import torch

from ctreconstruction_gb300 import Projector, iterative
from oracle import oracle as ora
from oracle.oracle import OracleGeometry
from _util import RTOL, cone_params, rel_err

pytestmark = pytest.mark.gpu

GEOM = cone_params(n=(20, 16, 12), nviews=12, nu=44, nv=36, du=1.0, dv=1.0, dx=1.0)


def _phantom(shape, seed=0):
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.linspace(-1, 1, nz), np.linspace(-1, 1, ny), np.linspace(-1, 1, nx), indexing="ij")
    v = np.zeros(shape, np.float32)
    for _ in range(4):
        c = rng.uniform(-0.4, 0.4, 3)
        a = rng.uniform(0.2, 0.5, 3)
        v += rng.uniform(0.2, 1.0) * ((((x - c[0]) / a[0]) ** 2 + ((y - c[1]) / a[1]) ** 2 +
                                        ((z - c[2]) / a[2]) ** 2) <= 1)
    return v.astype(np.float32)


@pytest.fixture(scope="module")
def setup(cuda):
    g = OracleGeometry(GEOM)
    P = Projector(GEOM, device=cuda)
    ph = _phantom((g.nz, g.ny, g.nx))
    proj0 = g.forward(ph).astype(np.float32)
    return g, P, ph, proj0


def test_sart_matches_oracle(setup, cuda):
    g, P, ph, proj0 = setup
    want = ora.sart(g, proj0.copy(), 3)
    x, _ = iterative.sart(P, torch.from_numpy(proj0).to(cuda), niter=3)
    assert rel_err(x.cpu().numpy(), want) < RTOL


def test_mlem_matches_oracle(setup, cuda):
    g, P, ph, proj0 = setup
    p_host = proj0.copy()
    want = ora.mlem(g, p_host, 3)
    p_dev = torch.from_numpy(proj0.copy()).to(cuda)
    x, _ = iterative.mlem(P, p_dev, niter=3)
    assert rel_err(x.cpu().numpy(), want) < RTOL
    # the script zeroes measured data where the forward projection is zero, in place
    assert np.array_equal(p_dev.cpu().numpy() == 0, p_host == 0)


def test_tv_step_matches_tv_grad(cuda):
    rng = np.random.default_rng(5)
    x = rng.random((9, 11, 13), dtype=np.float32)
    want = x - np.float32(0.05) * ora.tv_grad(x)
    got = iterative.tv_descent(torch.from_numpy(x).to(cuda), 0.05, 1)
    assert rel_err(got.cpu().numpy(), want) < 1e-5
    want3 = x.copy()
    for _ in range(3):
        want3 = want3 - np.float32(0.02) * ora.tv_grad(want3)
    got3 = iterative.tv_descent(torch.from_numpy(x).to(cuda), 0.02, 3)
    assert rel_err(got3.cpu().numpy(), want3) < 1e-5


@pytest.mark.parametrize("ng", [0, 3])
def test_asd_pocs_matches_oracle(setup, cuda, ng):
    """ASD-POCS (2 outer iterations, 2 POCS sub-steps, ng TV steps) against
    the same loop over the FP64 oracle, at the common bar."""
    g, P, ph, proj0 = setup
    want, log_o = ora.asd_pocs(g, proj0.copy(), 2, na=2, ng=ng)
    x, _, log_g = iterative.asd_pocs(P, torch.from_numpy(proj0).to(cuda), niter=2, na=2, ng=ng)
    err = rel_err(x.cpu().numpy(), want)
    print("ASD-POCS ng=%d rel err %.3e" % (ng, err))
    assert err < RTOL
    for a, b in zip(log_g, log_o):
        assert a["alpha"] == b["alpha"] and abs(a["dp"] - b["dp"]) <= 1e-3 * b["dp"]


@pytest.mark.parametrize("nsubsets,niter", [(4, 3), (3, 2), (12, 1)])
def test_os_sart_matches_oracle(setup, cuda, nsubsets, niter):
    """OS-SART with several subsets against the same loop over the FP64
    oracle projectors (oracle.os_sart)."""
    g, P, ph, proj0 = setup
    want = ora.os_sart(GEOM, proj0.copy(), nsubsets, niter, lam=0.8)
    x, _ = iterative.os_sart(P, torch.from_numpy(proj0).to(cuda), nsubsets=nsubsets, niter=niter, lam=0.8)
    err = rel_err(x.cpu().numpy(), want)
    print("OS-SART nsubsets=%d niter=%d rel err %.3e" % (nsubsets, niter, err))
    assert err < RTOL


def test_os_sart_reduces_error(setup, cuda):
    g, P, ph, proj0 = setup
    x, rmse = iterative.os_sart(P, torch.from_numpy(proj0).to(cuda), nsubsets=4, niter=6, lam=0.8,
                                phantom=torch.from_numpy(ph).to(cuda))
    assert rmse[-1] < 0.7 * rmse[0]
    assert np.all(x.cpu().numpy() >= 0)


def test_os_sart_one_subset_is_one_pocs_step(setup, cuda):
    """nsubsets=1 and niter=1 from zero equals the POCS formula with the matched pair."""
    g, P, ph, proj0 = setup
    x, _ = iterative.os_sart(P, torch.from_numpy(proj0).to(cuda), nsubsets=1, niter=1, lam=0.8)
    a1 = g.forward(np.ones((g.nz, g.ny, g.nx), np.float32))
    b1 = g.backward_matched(np.ones((g.nviews, g.nv, g.nu), np.float32))
    r = np.where(a1 == 0, 0, proj0 / (a1 + 1e-5))
    b = g.backward_matched(r.astype(np.float32))
    want = np.maximum(0.8 * np.where(b1 == 0, 0, b) / (b1 + 1e-5), 0)
    assert rel_err(x.cpu().numpy(), want) < RTOL


def test_graph_replay_matches_eager(setup, cuda):
    """One iteration captured in a CUDA graph and replayed gives the same
    bits as the same iterations issued eagerly (SART, MLEM, OS-SART)."""
    g, P, ph, proj0 = setup
    p = torch.from_numpy(proj0).to(cuda)
    for make in (lambda: iterative.SART(P, p.clone()), lambda: iterative.MLEM(P, p.clone().clamp_(min=0)),
                 lambda: iterative.OSSART(P, p.clone(), nsubsets=4)):
        eager, graphed = make(), make()
        eager.run(4)                      # capture() runs one eager warm-up iteration; recording runs nothing
        graphed.capture()
        graphed.run(3)
        torch.cuda.synchronize()
        assert torch.equal(eager.x, graphed.x), type(eager).__name__


def test_solver_batch_single_graph(cuda):
    """Scans of uneven sizes advanced by one graph launch per iteration match
    the solvers run one by one."""
    scans = []
    for n, nv, seed in ((12, 8, 1), (16, 12, 2), (20, 8, 3)):
        geom = cone_params(n=n, nviews=nv, nu=2 * n + 4, nv=2 * n, dx=1.0)
        P = Projector(geom, device=cuda)
        x = torch.from_numpy(_phantom((n, n, n), seed)).to(cuda)
        scans.append((geom, P.forward(x)))
    ref = [iterative.OSSART(Projector(geom, device=cuda), p, nsubsets=4) for geom, p in scans]
    for s in ref:
        s.run(3)
    batch = iterative.SolverBatch([iterative.OSSART(Projector(geom, device=cuda), p, nsubsets=4) for geom, p in scans])
    batch.capture()
    batch.run(2)
    torch.cuda.synchronize()
    for a, b in zip(ref, batch.solvers):
        assert torch.equal(a.x, b.x)
