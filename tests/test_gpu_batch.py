"""Batched, fused iterative drivers (ctreconstruction_gb300.batch): many scans
of uneven sizes advanced by single persistent launches with the drivers'
residual and update lines fused into the projectors' stores, against the same
single-scan solvers run one by one with separate element-wise kernels.  The
fused epilogues evaluate the same expressions, so the iterates agree bit for
bit (to float rounding where a single scan's backprojection runs over the
rotation orbits of a quarter-turn-symmetric scan)."""
import numpy as np
import pytest
import torch

from ctreconstruction_gb300 import Projector, batch, iterative
from _util import cone_params

pytestmark = pytest.mark.gpu


def _phantom(shape, seed):
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.linspace(-1, 1, nz), np.linspace(-1, 1, ny), np.linspace(-1, 1, nx), indexing="ij")
    v = np.zeros(shape, np.float32)
    for _ in range(4):
        c = rng.uniform(-0.4, 0.4, 3)
        a = rng.uniform(0.2, 0.5, 3)
        v += rng.uniform(0.2, 1.0) * ((((x - c[0]) / a[0]) ** 2 + ((y - c[1]) / a[1]) ** 2 +
                                        ((z - c[2]) / a[2]) ** 2) <= 1)
    return v


# Uneven scans: cubes and boxes, sides that are and are not multiples of 4
# (the TMA and the global-load forward paths), different detectors.
SCANS = [((16, 16, 16), 12, 36, 32, 1), ((20, 24, 12), 12, 44, 30, 2), ((18, 14, 10), 12, 30, 24, 3)]


@pytest.fixture(scope="module")
def scans(cuda):
    out = []
    for shape, nviews, nu, nv, seed in SCANS:
        nx, ny, nz = shape
        geom = cone_params(n=(nx, ny, nz), nviews=nviews, nu=nu, nv=nv, dx=1.0)
        P = Projector(geom, device=cuda)
        ph = torch.from_numpy(_phantom((nz, ny, nx), seed)).to(cuda)
        out.append((geom, P.forward(ph).clamp_(min=0)))
    return out


def _fresh(scans, cuda):
    return [(Projector(g, device=cuda), p.clone()) for g, p in scans]


@pytest.mark.parametrize("kind", ["ossart", "mlem", "sart"])
def test_batched_solver_matches_solvers_one_by_one(cuda, scans, kind):
    make = {"ossart": lambda P, p: iterative.OSSART(P, p, nsubsets=4, lam=0.8),
            "mlem": lambda P, p: iterative.MLEM(P, p),
            "sart": lambda P, p: iterative.SART(P, p)}[kind]
    ref = [make(P, p) for P, p in _fresh(scans, cuda)]
    for s in ref:
        s.run(3)
    b = batch.BatchedSolver([make(P, p) for P, p in _fresh(scans, cuda)])
    b.run(3)
    torch.cuda.synchronize()
    for a, c in zip(ref, b.solvers):
        if kind != "ossart" and a.P.orbit_size() == 4:
            # a single scan on a quarter-turn-symmetric orbit backprojects by
            # the row walk, the batch by integrated projections: the same sums
            # in another float order
            err = float((a.x - c.x).abs().max() / a.x.abs().max())
            assert err < 1e-5, (kind, err)
            continue
        assert torch.equal(a.x, c.x), kind
        if kind == "mlem":   # EM.py zeroes measured data where A x == 0, in place
            assert torch.equal(a.proj0, c.proj0)


def test_batched_os_sart_graph_replay(cuda, scans):
    """One batched iteration captured in a CUDA graph and replayed gives the
    same bits as the same iterations issued eagerly; the whole iteration is a
    handful of launches (per subset: transpose, one forward launch per
    dominant axis, integration, backprojection)."""
    eager = batch.batched_os_sart(_fresh(scans, cuda), nsubsets=4)
    graphed = batch.batched_os_sart(_fresh(scans, cuda), nsubsets=4)
    eager.run(4)
    graphed.capture()          # one eager step first
    graphed.run(3)
    torch.cuda.synchronize()
    for a, c in zip(eager.solvers, graphed.solvers):
        assert torch.equal(a.x, c.x)
    assert graphed.launches_per_step() <= 4 * 5


def test_batched_mlem_matched_backprojector(cuda, scans):
    ref = [iterative.MLEM(P, p, matched=True) for P, p in _fresh(scans, cuda)]
    for s in ref:
        s.run(2)
    b = batch.batched_mlem(_fresh(scans, cuda), matched=True)
    b.run(2)
    torch.cuda.synchronize()
    for a, c in zip(ref, b.solvers):
        if a.P.orbit_size() == 4:
            # single scan: the quarter-turn orbit kernel (shared set-ups, the
            # same float expressions otherwise); batch: one column per thread
            err = float((a.x - c.x).abs().max() / a.x.abs().max())
            assert err < 1e-5, err
            continue
        assert torch.equal(a.x, c.x)


def test_device_status_clean_after_batches(cuda):
    import ctypes
    from ctreconstruction_gb300 import _lib
    st = ctypes.c_int32(-1)
    _lib.call("ctgb_device_status", ctypes.byref(st), 1)
    assert st.value == 0
