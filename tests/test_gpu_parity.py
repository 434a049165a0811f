"""Parity of the CUDA path (through the C ABI, via Projector/Reconstruction)
with the reference's golden vectors and with the FP64 oracle.

Bar: max|gpu - ref| / max|ref| <= 1e-4 for every projection stack, volume and
filtered stack (float32 arithmetic on both sides)."""
import numpy as np
import pytest
import torch

from ctreconstruction_gb300 import Projector, Reconstruction
from oracle.oracle import OracleGeometry
from _util import RTOL, cone_params, golden_ids, load_golden, rel_err

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


@pytest.mark.parametrize("name", golden_ids())
def test_golden_forward_backward(cuda, name):
    p, flavour, d = load_golden(name)
    P = Projector(p, flavour=flavour)
    if "forward" in d.files:
        out = P.forward(_t(d["image"], cuda)).cpu().numpy()
        assert rel_err(out, d["forward"]) < RTOL
    if "backward" in d.files:
        out = P.backproject_fdk(_t(d["proj"], cuda)).cpu().numpy()
        assert rel_err(out, d["backward"]) < RTOL


@pytest.mark.parametrize("name", [n for n in golden_ids() if n in ("numba_basic", "numba_fan", "pycuda_basic",
                                                                     "pycuda_offset")])
def test_golden_filtering(cuda, name):
    p, flavour, d = load_golden(name)
    P = Projector(p, flavour=flavour)
    keys = [k for k in d.files if k.startswith("filter_")]
    assert keys
    for k in keys:
        _, ft, co = k.split("_")
        q = _t(d["proj"], cuda)
        P.filter(q, ft, float(co))
        assert rel_err(q.cpu().numpy(), d[k]) < RTOL, k


def test_reconstruction_class_roundtrip(cuda):
    p, flavour, d = load_golden("numba_basic")
    R = Reconstruction(p, flavour=flavour)
    R.image = d["image"].copy()
    R.forward()
    assert isinstance(R.proj, np.ndarray) and rel_err(R.proj, d["forward"]) < RTOL
    R.proj = d["proj"].copy()
    R.Filtering()
    assert rel_err(R.proj, d["filter_hann_1"]) < RTOL
    R.proj = _t(d["proj"], cuda)
    R.backward()
    assert isinstance(R.image, torch.Tensor) and rel_err(R.image.cpu().numpy(), d["backward"]) < RTOL


GEOMS = {
    "cone_y_and_x_views": cone_params(n=(20, 18, 16), nviews=24, nu=36, nv=28, dx=0.9),
    "offcentre_short_scan": cone_params(n=(17, 21, 13), nviews=13, nu=30, nv=26, start=0.4, span=np.pi + 0.6,
                                        PhantomCenter=[1.1, -0.7, 0.4], ReconCenter=[-0.6, 0.8, -0.3]),
    "fine_detector": cone_params(n=16, nviews=10, nu=64, nv=48, du=0.35, dv=0.4),
    "coarse_detector": cone_params(n=24, nviews=10, nu=16, nv=12, du=2.7, dv=2.9),
    "helical": cone_params(n=16, nviews=20, nu=32, nv=16, Pitch=0.7, start=0.0, span=4 * np.pi),
    "curved": cone_params(n=18, nviews=12, nu=36, nv=24, DetectorShape='Curved'),
    "pycuda_offset": dict(cone_params(n=(19, 15, 11), nviews=11, nu=33, nv=21, ReconCenter=[0.3, -0.2, 0.5]),
                          DetectorOffset=[0.6, -0.45]),
    # sizes with nx, ny multiples of 4 take the TMA forward path
    "tma_cone": cone_params(n=(32, 28, 20), nviews=20, nu=48, nv=40, dx=0.8),
    "tma_offcentre": cone_params(n=(36, 24, 22), nviews=17, nu=56, nv=36, start=0.3, span=2 * np.pi,
                                 PhantomCenter=[2.1, -1.3, 0.9], ReconCenter=[-0.6, 0.8, -0.3]),
    "tma_fine": cone_params(n=(24, 24, 16), nviews=12, nu=100, nv=70, du=0.3, dv=0.35),
    "tma_wide_footprint": cone_params(n=(28, 32, 24), nviews=12, nu=12, nv=10, du=5.0, dv=4.5),
    "tma_tall_rows": cone_params(n=(24, 24, 48), nviews=10, nu=40, nv=20, du=1.0, dv=3.2),
    "tma_curved": cone_params(n=(28, 24, 20), nviews=14, nu=44, nv=32, DetectorShape='Curved'),
    "tma_helical": cone_params(n=(24, 24, 20), nviews=18, nu=40, nv=20, Pitch=0.6, span=4 * np.pi),
    "tma_pycuda": dict(cone_params(n=(32, 20, 14), nviews=9, nu=36, nv=24, ReconCenter=[0.5, 0.2, -0.4]),
                       DetectorOffset=[-0.7, 0.35]),
    "tma_partial_tiles": cone_params(n=(20, 28, 18), nviews=11, nu=45, nv=27),
    # a detector row spans 0.89-1.25 voxel rows: 32-row tiles, rows over three cells
    "tma_32row_mid": cone_params(n=(24, 24, 24), nviews=12, nu=40, nv=40, dv=1.6),
    # 1.1-1.56 voxel rows per detector row: 16-row tiles, rows over three cells
    "tma_16row_mid": cone_params(n=(24, 24, 32), nviews=10, nu=40, nv=20, dv=2.0),
}


@pytest.mark.parametrize("gname", sorted(GEOMS))
def test_against_fp64_oracle(cuda, gname):
    p = GEOMS[gname]
    flavour = "pycuda" if "DetectorOffset" in p else "numba"
    g = OracleGeometry(p, flavour)
    P = Projector(p, flavour=flavour)
    rng = np.random.default_rng(abs(hash(gname)) % 2 ** 32)
    x = rng.random((g.nz, g.ny, g.nx), dtype=np.float32)
    y = rng.random((g.nviews, g.nv, g.nu), dtype=np.float32)
    assert rel_err(P.forward(_t(x, cuda)).cpu().numpy(), g.forward(x)) < RTOL
    assert rel_err(P.backproject_fdk(_t(y, cuda)).cpu().numpy(), g.backward_fdk(y)) < RTOL
    assert rel_err(P.backproject_matched(_t(y, cuda)).cpu().numpy(), g.backward_matched(y)) < RTOL


@pytest.mark.parametrize("gname", ["cone_y_and_x_views", "curved", "helical", "tma_cone", "tma_curved"])
def test_matched_backprojector_is_adjoint(cuda, gname):
    """Dot-product test <A x, y> = <x, A^T y> to 1e-5 relative, on
    non-negative random x and y (volumes and projections are non-negative).
    With zero-mean x and y the inner product is itself a cancelling sum whose
    size varies from seed to seed, so its relative error measures that
    cancellation as much as the adjoint: at these sizes Gaussian seeds give
    1e-7 to 1.5e-5 for the same kernels, uniform ones 1e-9 to 1e-8.  The
    full-size test also runs Gaussian data."""
    p = GEOMS[gname]
    P = Projector(p)
    gen = torch.Generator(device=cuda).manual_seed(3)
    x = torch.rand(P.volume_shape, device=cuda, generator=gen)
    y = torch.rand(P.proj_shape(), device=cuda, generator=gen)
    lhs = torch.sum(P.forward(x).double() * y.double()).item()
    rhs = torch.sum(x.double() * P.backproject_matched(y).double()).item()
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))


@pytest.mark.parametrize("gname", ["cone_y_and_x_views", "tma_cone"])
def test_forward_without_transposed_copy_matches(cuda, gname):
    p = GEOMS[gname]
    P = Projector(p)
    x = torch.rand(P.volume_shape, device=cuda)
    a = P.forward(x)
    b = torch.empty_like(a)
    from ctreconstruction_gb300 import _lib
    import ctypes
    _lib.call("ctgb_forward", ctypes.byref(P.c), ctypes.c_void_p(P.table.data_ptr()), ctypes.c_void_p(x.data_ptr()),
              None, ctypes.c_void_p(b.data_ptr()), 0, P.params.NumberOfViews,
              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert rel_err(b.cpu().numpy(), a.cpu().numpy()) < 1e-5


def test_view_ranges_and_accumulate(cuda):
    p = GEOMS["cone_y_and_x_views"]
    P = Projector(p)
    x = torch.rand(P.volume_shape, device=cuda)
    full = P.forward(x)
    part = torch.cat([P.forward(x, view0=0, nviews=7), P.forward(x, view0=7, nviews=17)])
    assert torch.equal(full, part)
    y = torch.rand(P.proj_shape(), device=cuda)
    whole = P.backproject_fdk(y)
    acc = P.backproject_fdk(y[:9].contiguous(), view0=0, nviews=9)
    P.backproject_fdk(y[9:].contiguous(), out=acc, view0=9, nviews=15, accumulate=True)
    assert rel_err(acc.cpu().numpy(), whole.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("gname", ["offcentre_short_scan", "tma_offcentre"])
def test_deterministic(cuda, gname):
    p = GEOMS[gname]
    P = Projector(p)
    x = torch.rand(P.volume_shape, device=cuda)
    y = torch.rand(P.proj_shape(), device=cuda)
    assert torch.equal(P.forward(x), P.forward(x))
    assert torch.equal(P.backproject_fdk(y), P.backproject_fdk(y))
    assert torch.equal(P.backproject_matched(y), P.backproject_matched(y))


def test_bad_inputs_raise(cuda):
    P = Projector(GEOMS["curved"])
    with pytest.raises(ValueError):
        P.forward(torch.rand(P.volume_shape))            # CPU tensor
    with pytest.raises(ValueError):
        P.forward(torch.rand(P.volume_shape, device=cuda, dtype=torch.float64))
    with pytest.raises(ValueError):
        P.forward(torch.rand((3, 3, 3), device=cuda))


def test_bounded_wait_runs_out_into_the_status_word(cuda):
    """A bounded device wait that nothing satisfies (the self-test kernel's
    mbarrier gets no arrival) gives up after its poll limit, sets
    CTGB_DEVERR_TIMEOUT in the device status word and returns; the context
    stays usable (a projection afterwards matches the oracle) and the status
    clears."""
    import ctypes
    from ctreconstruction_gb300 import _lib
    st = ctypes.c_int32(0)
    _lib.call("ctgb_device_status", ctypes.byref(st), 1)            # start clean
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("ctgb_selftest_bounded_wait", 1000, stream)
    _lib.call("ctgb_device_status", ctypes.byref(st), 1)
    assert st.value & 1, st.value                                    # CTGB_DEVERR_TIMEOUT
    _lib.call("ctgb_device_status", ctypes.byref(st), 0)
    assert st.value == 0
    p = GEOMS["tma_cone"]
    g = OracleGeometry(p)
    P = Projector(p)
    x = np.random.default_rng(3).random((g.nz, g.ny, g.nx), dtype=np.float32)
    assert rel_err(P.forward(_t(x, cuda)).cpu().numpy(), g.forward(x)) < RTOL
    _lib.call("ctgb_device_status", ctypes.byref(st), 0)
    assert st.value == 0


def test_device_status_clean_after_runs(cuda):
    """No kernel reported a wait timeout or bounds problem."""
    import ctypes
    from ctreconstruction_gb300 import _lib
    st = ctypes.c_int32(-1)
    _lib.call("ctgb_device_status", ctypes.byref(st), 1)
    assert st.value == 0


@pytest.mark.parametrize("gname", ["tma_cone", "curved", "coarse_detector", "helical", "pycuda_offset"])
def test_fdk_backprojector_entry_points_agree(cuda, gname):
    """ctgb_backproject_fdk (row tables) and ctgb_backproject_fdk_ws
    (integrated projections, small workspace to force view chunks) agree with
    the FP64 oracle."""
    import ctypes
    from ctreconstruction_gb300 import _lib
    p = GEOMS[gname]
    flavour = "pycuda" if "DetectorOffset" in p else "numba"
    g = OracleGeometry(p, flavour)
    P = Projector(p, flavour=flavour)
    rng = np.random.default_rng(21)
    y = rng.random((g.nviews, g.nv, g.nu), dtype=np.float32)
    want = g.backward_fdk(y)
    yt = _t(y, cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    a = torch.empty(P.volume_shape, device=cuda)
    _lib.call("ctgb_backproject_fdk", ctypes.byref(P.c), ctypes.c_void_p(P.table.data_ptr()),
              ctypes.c_void_p(yt.data_ptr()), ctypes.c_void_p(a.data_ptr()), 0, g.nviews, g.dtheta, 0, stream)
    n = ctypes.c_size_t(0)
    _lib.call("ctgb_backproject_fdk_workspace_bytes", ctypes.byref(P.c), 3, ctypes.byref(n))
    ws = torch.empty(n.value // 4, device=cuda)
    b = torch.empty(P.volume_shape, device=cuda)
    _lib.call("ctgb_backproject_fdk_ws", ctypes.byref(P.c), ctypes.c_void_p(P.table.data_ptr()),
              ctypes.c_void_p(yt.data_ptr()), ctypes.c_void_p(b.data_ptr()), 0, g.nviews, g.dtheta, 0,
              ctypes.c_void_p(ws.data_ptr()), n.value, stream)
    assert rel_err(a.cpu().numpy(), want) < RTOL
    assert rel_err(b.cpu().numpy(), want) < RTOL
    # the two stages as separate calls: same kernels, same bits as the chunked
    # path when one chunk holds every view (a full orbit with four-fold
    # symmetry takes the row walk instead)
    integ = P.integrate(yt)
    c = P.backproject_fdk_integrated(integ)
    d = P.backproject_fdk(yt)
    if P.orbit_size() == 4:
        assert torch.equal(a, d)
    else:
        assert torch.equal(c, d)
    assert rel_err(c.cpu().numpy(), want) < RTOL


ORBIT_GEOMS = {
    # square grid centred on the axis, full orbit: quarter-turn orbits
    "quarter": (cone_params(n=(28, 28, 20), nviews=16, nu=48, nv=36, dx=0.8), 4),
    "quarter_curved": (cone_params(n=(24, 24, 18), nviews=20, nu=40, nv=30, DetectorShape='Curved'), 4),
    # unit spacing: slice centres exactly antisymmetric, so the matched
    # backprojector also takes its quarter-turn orbit kernel
    "quarter_unit": (cone_params(n=(24, 24, 18), nviews=16, nu=40, nv=30), 4),
    # rectangular grid (even height): half-turn orbits
    "half": (cone_params(n=(30, 22, 20), nviews=18, nu=48, nv=36, dx=0.8), 2),
    # off-centre grid or a short scan: no symmetry
    "none_offcentre": (cone_params(n=(24, 24, 16), nviews=16, nu=40, nv=30, ReconCenter=[1.3, -0.7, 0.4]), 1),
    "none_short": (cone_params(n=(24, 24, 16), nviews=14, nu=40, nv=30, start=0.3, span=np.pi + 0.5), 1),
}


@pytest.mark.parametrize("gname", ["quarter", "quarter_curved", "quarter_unit", "half"])
def test_matched_orbit_matches_oracle_and_is_adjoint(cuda, gname):
    """A full-orbit matched backprojection (the quarter-turn orbit kernel where
    the scan allows it) against the FP64 oracle's literal transpose, and the
    dot-product test against the forward projector with uniform and with
    Gaussian vectors (terms of both signs: the sensitive case)."""
    p, nc = ORBIT_GEOMS[gname]
    g = OracleGeometry(p)
    P = Projector(p, device=cuda)
    rng = np.random.default_rng(7)
    y = rng.random((g.nviews, g.nv, g.nu), dtype=np.float32)
    x = rng.random((g.nz, g.ny, g.nx), dtype=np.float32)
    yt, xt = _t(y, cuda), _t(x, cuda)
    bt = P.backproject_matched(yt)
    e = rel_err(bt.cpu().numpy(), g.backward_matched(y))
    assert e < RTOL
    for kind in ("uniform", "gauss"):
        if kind == "gauss":
            yt = _t(rng.standard_normal(y.shape).astype(np.float32), cuda)
            xt = _t(rng.standard_normal(x.shape).astype(np.float32), cuda)
            bt = P.backproject_matched(yt)
        ax = P.forward(xt)
        lhs = float((ax.double() * yt.double()).sum())
        rhs = float((xt.double() * bt.double()).sum())
        print("matched orbit %s nc=%d err %.2e adjoint(%s) %.2e" % (gname, nc, e, kind, abs(lhs - rhs) / abs(lhs)))
        assert abs(lhs - rhs) <= 1e-5 * abs(lhs), kind


@pytest.mark.parametrize("gname", sorted(ORBIT_GEOMS))
def test_fdk_orbits_tile_the_full_call(cuda, gname):
    """The row-walk FDK backprojector over a whole orbit (one call), and over
    three ranges of base views (accumulated), match the FP64 oracle; the orbit
    size is the one the geometry's symmetry allows."""
    p, nc = ORBIT_GEOMS[gname]
    g = OracleGeometry(p)
    P = Projector(p, device=cuda)
    assert P.orbit_size() == nc
    rng = np.random.default_rng(5)
    y = rng.random((g.nviews, g.nv, g.nu), dtype=np.float32)
    want = g.backward_fdk(y)
    yt = _t(y, cuda)
    full = torch.empty(P.volume_shape, device=cuda)
    import ctypes
    from ctreconstruction_gb300 import _lib
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("ctgb_backproject_fdk", ctypes.byref(P.c), ctypes.c_void_p(P.table.data_ptr()),
              ctypes.c_void_p(yt.data_ptr()), ctypes.c_void_p(full.data_ptr()), 0, g.nviews, g.dtheta, 0, stream)
    period = g.nviews // nc
    cuts = [0, period // 3, (2 * period) // 3, period]
    part = torch.full(P.volume_shape, float("nan"), device=cuda)
    for i in range(3):
        P.backproject_fdk_orbits(yt, part, cuts[i], cuts[i + 1] - cuts[i], accumulate=i > 0)
    e_full, e_part = rel_err(full.cpu().numpy(), want), rel_err(part.cpu().numpy(), want)
    print("orbits %s nc=%d full %.2e parts %.2e" % (gname, nc, e_full, e_part))
    assert e_full < RTOL and e_part < RTOL



@pytest.mark.parametrize("gname", ["cone_y_and_x_views", "tma_cone", "curved", "helical", "pycuda_offset",
                                   "tma_offcentre"])
def test_matched_backprojector_entry_points_agree(cuda, gname):
    """ctgb_backproject_matched (row sweep, no workspace) and
    ctgb_backproject_matched_ws (integrated projections, small workspace to
    force view chunks) agree with the FP64 oracle's transpose of the forward,
    and each is the adjoint of the forward (uniform data, 1e-5)."""
    import ctypes
    from ctreconstruction_gb300 import _lib
    p = GEOMS[gname]
    flavour = "pycuda" if "DetectorOffset" in p else "numba"
    g = OracleGeometry(p, flavour)
    P = Projector(p, flavour=flavour)
    rng = np.random.default_rng(23)
    y = rng.random((g.nviews, g.nv, g.nu), dtype=np.float32)
    want = g.backward_matched(y)
    yt = _t(y, cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    a = torch.empty(P.volume_shape, device=cuda)
    _lib.call("ctgb_backproject_matched", ctypes.byref(P.c), ctypes.c_void_p(P.table.data_ptr()),
              ctypes.c_void_p(yt.data_ptr()), ctypes.c_void_p(a.data_ptr()), 0, g.nviews, 1.0, 0, stream)
    n = ctypes.c_size_t(0)
    _lib.call("ctgb_backproject_fdk_workspace_bytes", ctypes.byref(P.c), 3, ctypes.byref(n))
    ws = torch.empty(n.value // 4, device=cuda)
    b = torch.empty(P.volume_shape, device=cuda)
    _lib.call("ctgb_backproject_matched_ws", ctypes.byref(P.c), ctypes.c_void_p(P.table.data_ptr()),
              ctypes.c_void_p(yt.data_ptr()), ctypes.c_void_p(b.data_ptr()), 0, g.nviews, 1.0, 0,
              ctypes.c_void_p(ws.data_ptr()), n.value, stream)
    assert rel_err(a.cpu().numpy(), want) < RTOL
    assert rel_err(b.cpu().numpy(), want) < RTOL
    x = torch.rand(P.volume_shape, device=cuda, generator=torch.Generator(device=cuda).manual_seed(5))
    lhs = torch.sum(P.forward(x).double() * yt.double()).item()
    for v in (a, b):
        rhs = torch.sum(x.double() * v.double()).item()
        assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))


@pytest.mark.parametrize("gname", ["cone_y_and_x_views", "offcentre_short_scan", "curved", "helical", "tma_cone",
                                   "pycuda_offset"])
def test_ray_projector_matches_oracle(cuda, gname):
    """Siddon ray sums and their transpose against the FP64 restatement of
    matlab/RayDrivenProjection3DSiddon.m on the same geometry."""
    p = GEOMS[gname]
    flavour = "pycuda" if "DetectorOffset" in p else "numba"
    g = OracleGeometry(p, flavour)
    P = Projector(p, flavour=flavour)
    rng = np.random.default_rng(11)
    x = rng.random((g.nz, g.ny, g.nx), dtype=np.float32)
    y = rng.random((g.nviews, g.nv, g.nu), dtype=np.float32)
    assert rel_err(P.ray_forward(_t(x, cuda)).cpu().numpy(), g.ray_forward(x)) < RTOL
    assert rel_err(P.ray_backproject(_t(y, cuda)).cpu().numpy(), g.ray_backward(y)) < RTOL


def test_ray_method_through_reconstruction(cuda):
    p = dict(GEOMS["cone_y_and_x_views"], Method='Ray')
    g = OracleGeometry(p)
    R = Reconstruction(p)
    rng = np.random.default_rng(12)
    R.image = rng.random((g.nz, g.ny, g.nx), dtype=np.float32)
    R.forward()
    assert rel_err(R.proj, g.ray_forward(R.image)) < RTOL
    gen = torch.Generator(device=cuda).manual_seed(5)
    P = Projector(p)
    a = torch.randn(P.volume_shape, device=cuda, generator=gen)
    b = torch.randn(P.proj_shape(), device=cuda, generator=gen)
    lhs = torch.sum(P.ray_forward(a).double() * b.double()).item()
    rhs = torch.sum(a.double() * P.ray_backproject(b).double()).item()
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))


def test_reconstruction_pinned_host_tensors(cuda):
    """CPU (pinned) tensors in -> pinned CPU tensors out, same values as the
    NumPy round trip."""
    p, flavour, d = load_golden("numba_basic")
    R = Reconstruction(p, flavour=flavour)
    R.image = torch.from_numpy(d["image"].copy()).pin_memory()
    R.forward()
    assert isinstance(R.proj, torch.Tensor) and not R.proj.is_cuda and R.proj.is_pinned()
    assert rel_err(R.proj.numpy(), d["forward"]) < RTOL
    R.proj = torch.from_numpy(d["proj"].copy()).pin_memory()
    R.backward()
    assert not R.image.is_cuda and rel_err(R.image.numpy(), d["backward"]) < RTOL


def test_reconstruction_pinned_chunks_match_device(cuda):
    """The pinned host path runs views in chunks with the copies on a second
    stream: forward identical to the one-launch device path, backward equal
    to float rounding (the chunks accumulate in a different order), and a
    second call on the same object gives the same values."""
    p = cone_params(n=48, nviews=90, nu=64, nv=56, du=1.2, dv=1.2)
    R = Reconstruction(p)
    P = R.projector
    gen = torch.Generator(device=cuda).manual_seed(11)
    vol = torch.rand(P.volume_shape, device=cuda, generator=gen)
    want_proj = P.forward(vol)
    want_vol = P.backproject_fdk(want_proj)
    torch.cuda.synchronize()
    for _ in range(2):
        R.image = vol.cpu().pin_memory()
        R.forward()
        assert R.proj.is_pinned()
        assert torch.equal(R.proj, want_proj.cpu())
        R.backward()
        assert not R.image.is_cuda
        assert rel_err(R.image.numpy(), want_vol.cpu().numpy()) < 1e-5
