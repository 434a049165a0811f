"""Parity at the benchmarks' full sizes.

The small-geometry parity tests cannot show errors that grow with the
problem: float32 running sums over 768 detector rows in the integrated
projections, the filter's FFT at 2048 points, tile choices that only large
detectors select.  These tests run the exact benchmark geometries on the GPU
and compare with the FP64 oracle on what the oracle can afford: a spread of
views for the 512^3 forward projection, z slabs of the full-volume
backprojections, every voxel and view of the 128^3 FDK reconstruction.  The
adjoint test runs on the whole 512^3 / 720-view problem with float64 sums.

Bars: max|gpu - oracle| / max|oracle| <= 1e-4 per projection stack, slab and
volume (RTOL); adjoint 1e-5 relative.  Each test prints its errors.
"""
import numpy as np
import pytest
import torch

from ctreconstruction_gb300 import Projector, phantoms
from ctreconstruction_gb300.autograd import dd_project
from ctreconstruction_gb300.parallel import slab_params
from oracle.oracle import OracleGeometry
from _util import RTOL, cfg1_params, cfg3_params, rel_err

pytestmark = pytest.mark.gpu

# Views spread over the orbit: both dominant axes (the axis changes at 45
# degrees, view 90 of 720), the first and last quarter turns.
VIEWS = (0, 37, 90, 180, 359, 540)
SLAB = 16
# The central slab, and one 80 mm above the centre: its footprints reach
# detector rows far from the central row, where the running row sums of the
# integrated projections are large.
SLABS = (248, 96)


def _report(name, errs):
    print("FULLSIZE %s %s" % (name, " ".join("%s=%.3e" % kv for kv in errs.items())))


@pytest.fixture(scope="module")
def cfg3(cuda):
    p = cfg3_params()
    P = Projector(p, device=cuda)
    vol = phantoms.random_ellipsoids((512, 512, 512), n=30, seed=1, device=cuda)
    return p, P, vol


def test_cfg3_forward_views(cfg3):
    p, P, vol = cfg3
    g = OracleGeometry(p)
    x = vol.cpu().numpy()
    errs = {}
    for v in VIEWS:
        got = P.forward(vol, view0=v, nviews=1).cpu().numpy()
        errs["view%d" % v] = rel_err(got, g.forward(x, v, 1))
    # one launch over a run of views that crosses the change of dominant axis
    got = P.forward(vol, view0=84, nviews=12).cpu().numpy()
    errs["views84-95"] = rel_err(got, g.forward(x, 84, 12))
    _report("forward", errs)
    assert max(errs.values()) <= RTOL, errs


def _slab_oracles(p):
    return {z0: OracleGeometry(slab_params(p, z0, SLAB).as_dict()) for z0 in SLABS}


def test_cfg3_fdk_backprojection_slabs(cfg3):
    """FDK-weighted backprojection of the phantom's own projections (positive,
    so the running row sums are as large as the benchmark's), one view per
    launch and a 12-view launch, on the full 512^3 grid; the oracle computes
    two 16-voxel z slabs."""
    p, P, vol = cfg3
    oracles = _slab_oracles(p)
    errs = {}
    cases = [(v, 1) for v in VIEWS] + [(84, 12)]
    for v0, nv in cases:
        proj = P.forward(vol, view0=v0, nviews=nv)
        got = P.backproject_fdk(proj, view0=v0, nviews=nv).cpu().numpy()
        host = proj.cpu().numpy()
        for z0, g in oracles.items():
            want = g.backward_fdk(host, v0, nv)
            errs["v%d+%d_z%d" % (v0, nv, z0)] = rel_err(got[z0:z0 + SLAB], want)
    _report("backproject_fdk", errs)
    assert max(errs.values()) <= RTOL, errs


def test_cfg3_fdk_walk_full_orbit(cfg3):
    """The benchmark's backward(): one row-walk launch over all 720 views
    sharing each set-up between the four columns of a quarter-turn orbit.  The
    whole volume against the integrated-projection kernel (pinned per view
    above), and the central 8-slice slab against the FP64 oracle over all 720
    views."""
    p, P, vol = cfg3
    assert P.orbit_size() == 4
    proj = P.forward(vol)
    got = P.backproject_fdk(proj)
    integ = P.integrate(proj)
    ref = P.backproject_fdk_integrated(integ)
    errs = {"vs_integrated": float((got - ref).abs().max() / ref.abs().max())}
    del integ, ref
    z0 = 252
    g = OracleGeometry(slab_params(p, z0, 8).as_dict())
    want = g.backward_fdk(proj.cpu().numpy())
    errs["vs_oracle_z%d" % z0] = rel_err(got[z0:z0 + 8].cpu().numpy(), want)
    _report("backproject_fdk_walk", errs)
    assert max(errs.values()) <= RTOL, errs


# Single-view matched backprojections at oblique views carry the float32
# rounding of the detector columns' transverse footprint positions: on a
# 512-voxel grid a boundary ray's position (a difference of two terms near
# 2000 voxel units) is rounded to ~1e-4 voxel, which a single view's
# backprojection shows as ~2e-4 of a voxel's value.  The forward projector
# evaluates the same positions (its adjoint agrees to 2e-6), and sums over
# views average the rounding out (12 views: 6e-5).
SINGLE_VIEW_MATCHED_TOL = 3e-4


def test_cfg3_matched_backprojection_slabs(cfg3):
    """Matched (adjoint) backprojection of seeded cotangents: uniform on
    [0, 1), against max|oracle|; and Gaussian, whose backprojection is a
    cancelling sum of a few terms per voxel and view, against the scale of
    those terms, max of the oracle's backprojection of |y| (the bound any
    floating-point evaluation of a signed sum is held to).  Bars: RTOL for
    the 12-view launch, SINGLE_VIEW_MATCHED_TOL for one view."""
    p, P, _ = cfg3
    oracles = _slab_oracles(p)
    gen = torch.Generator(device=P.device).manual_seed(1)
    errs = {}
    for v0, nv in [(v, 1) for v in VIEWS[:4]] + [(84, 12)]:
        for kind in ("unif", "gauss"):
            y = (torch.rand if kind == "unif" else torch.randn)((nv, 768, 1024), device=P.device, generator=gen)
            got = P.backproject_matched(y, view0=v0, nviews=nv).cpu().numpy()
            host = y.cpu().numpy()
            for z0, g in oracles.items():
                want = g.backward_matched(host, v0, nv)
                scale = np.abs(want).max() if kind == "unif" else g.backward_matched(np.abs(host), v0, nv).max()
                errs["%s_v%d+%d_z%d" % (kind, v0, nv, z0)] = float(np.abs(got[z0:z0 + SLAB] - want).max() / scale)
    _report("backproject_matched", errs)
    assert max(v for k, v in errs.items() if "+12_" in k) <= RTOL, errs
    assert max(v for k, v in errs.items() if "+1_" in k) <= SINGLE_VIEW_MATCHED_TOL, errs


def _dot(a, b, chunk=60):
    """<a, b> in float64, a view chunk at a time."""
    s = 0.0
    for i in range(0, a.shape[0], chunk):
        s += torch.sum(a[i:i + chunk].double() * b[i:i + chunk].double()).item()
    return s


@pytest.mark.parametrize("kind", ["gauss", "unif"])
def test_cfg3_adjoint_full_size(cfg3, kind):
    """<A x, y> = <x, A^T y> over the whole 512^3 volume and all 720 views,
    x and y seeded Gaussian or uniform on [0, 1), float64 sums."""
    _, P, _ = cfg3
    gen = torch.Generator(device=P.device).manual_seed(1)
    draw = torch.randn if kind == "gauss" else torch.rand
    x = draw(P.volume_shape, device=P.device, generator=gen)
    y = draw(P.proj_shape(), device=P.device, generator=gen)
    ax = P.forward(x)
    lhs = _dot(ax, y)
    del ax
    aty = P.backproject_matched(y)
    rhs = _dot(x, aty)
    err = abs(lhs - rhs) / max(abs(lhs), abs(rhs))
    _report("adjoint_" + kind, {"rel": err, "lhs": lhs, "rhs": rhs})
    assert err <= 1e-5


def test_cfg3_matched_orbit_full(cfg3):
    """The matched backprojection of all 720 views by the quarter-turn orbit
    kernel against the view-chunked kernel (a workspace of 360 views), over
    the whole volume; the orbit kernel's adjoint identity is checked above."""
    import ctypes
    from ctreconstruction_gb300 import _lib
    _, P, _ = cfg3
    gen = torch.Generator(device=P.device).manual_seed(3)
    y = torch.rand(P.proj_shape(), device=P.device, generator=gen)
    got = P.backproject_matched(y)
    n = ctypes.c_size_t(0)
    _lib.call("ctgb_backproject_fdk_workspace_bytes", ctypes.byref(P.c), 360, ctypes.byref(n))
    ws = torch.empty(n.value // 4, device=P.device)
    ref = torch.empty_like(got)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("ctgb_backproject_matched_ws", ctypes.byref(P.c), ctypes.c_void_p(P.table.data_ptr()),
              ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(ref.data_ptr()), 0, 720, 1.0, 0,
              ctypes.c_void_p(ws.data_ptr()), n.value, stream)
    err = float((got - ref).abs().max() / ref.abs().max())
    _report("matched_orbit", {"vs_chunked": err})
    assert err <= 1e-5


@pytest.mark.parametrize("width", [1024, 256])
def test_filter_full_width(cfg3, width):
    """Filtering() at the benchmark detector widths (zero-padded FFTs of 2048
    and 512 points) for all five windows and two cutoffs, on projections of
    the phantom."""
    p, P, vol = cfg3
    if width == 256:
        p = cfg1_params()
        P = Projector(p, device=vol.device)
        src = phantoms.shepp_logan_3d((128, 128, 128), device=vol.device) * 0.02
    else:
        src = vol
    g = OracleGeometry(p)
    proj = P.forward(src, view0=30, nviews=4)
    host = proj.cpu().numpy()
    errs = {}
    for ft in ("ram-lak", "shepp-logan", "cosine", "hamming", "hann"):
        for co in (1.0, 0.5):
            q = proj.clone()
            P.filter(q, ft, co)
            errs["%s_%g" % (ft, co)] = rel_err(q.cpu().numpy(), g.filtering(host, ft, co))
    _report("filter_nu%d" % width, errs)
    assert max(errs.values()) <= RTOL, errs


def test_cfg1_fdk_reconstruction(cuda):
    """Filtering() + backward() of the 128^3 / 360-view FDK benchmark
    (modified Shepp-Logan, Poisson noise at I0 = 1e5), every voxel and view,
    against the oracle's filter and backprojection in float64."""
    p = cfg1_params()
    P = Projector(p, device=cuda)
    g = OracleGeometry(p)
    ph = phantoms.shepp_logan_3d((128, 128, 128), device=cuda) * 0.02
    clean = P.forward(ph)
    gen = torch.Generator(device=cuda).manual_seed(0)
    counts = torch.poisson(1e5 * torch.exp(-clean), generator=gen)
    proj = -torch.log(torch.clamp(counts, min=1.0) / 1e5)
    host = proj.cpu().numpy()
    q = proj.clone()
    P.filter(q)
    recon = P.backproject_fdk(q).cpu().numpy()
    filt = g.filtering(host)
    errs = {"filter": rel_err(q.cpu().numpy(), filt),
            "recon": rel_err(recon, g.backward_fdk(filt.astype(np.float32)))}
    _report("cfg1_fdk", errs)
    assert max(errs.values()) <= RTOL, errs


def test_cfg3_crop_gradient_finite_differences(cuda):
    """torch.autograd gradient of L(x) = 0.5 ||A x - y||^2 on a 64^3 crop of
    the benchmark grid (0.5 mm voxels, all 720 views), with the detector cut
    to the crop's footprint (the central 128 x 128 pixels of the 1024 x 768
    detector, same 0.75 mm pitch and pixel boundaries), against the FP64
    oracle: directional derivatives <grad L, e> = <A x - y, A e> and central
    differences of L.  x is half the phantom and y its noisy projections, an
    iterate partway to the solution (a residual that is mostly signal, as in
    a reconstruction, not noise that cancels)."""
    p = cfg3_params(NumberOfImage=[64, 64, 64], NumberOfDetectorPixels=[128, 128])
    P = Projector(p, device=cuda)
    g = OracleGeometry(p)
    rng = np.random.default_rng(1)
    ph = phantoms.random_ellipsoids((64, 64, 64), n=30, seed=1, device="cpu").numpy()
    x = (0.5 * ph).astype(np.float32)
    y = (g.forward(ph) + 0.01 * rng.standard_normal((720, 128, 128))).astype(np.float32)
    xt = torch.from_numpy(x).to(cuda).requires_grad_(True)
    loss = 0.5 * torch.sum((dd_project(xt, P) - torch.from_numpy(y).to(cuda)) ** 2)
    loss.backward()
    grad = xt.grad.double().cpu().numpy()
    r0 = g.forward(x) - y.astype(np.float64)

    def L(v):
        r = g.forward(v.astype(np.float32)) - y.astype(np.float64)
        return 0.5 * np.sum(r * r)

    dirs = {"gauss0": rng.standard_normal(x.shape), "gauss1": rng.standard_normal(x.shape),
            "ellipsoids": phantoms.random_ellipsoids((64, 64, 64), n=8, seed=7, device="cpu").numpy()}
    errs = {}
    for name, e in dirs.items():
        e = (e / np.linalg.norm(e)).astype(np.float32)
        fd = float(np.sum(r0 * g.forward(e)))                  # directional derivative, FP64
        an = float(np.sum(grad * e))
        errs[name] = abs(fd - an) / abs(fd)
        h = 1e-2
        errs["central_" + name] = abs((L(x + h * e) - L(x - h * e)) / (2 * h) - fd) / abs(fd)
    _report("crop64_gradient", errs)
    assert max(v for k, v in errs.items() if not k.startswith("central")) <= 1e-4, errs
    assert max(v for k, v in errs.items() if k.startswith("central")) <= 1e-3, errs
