"""libctgb.so on the CPU: it loads, exports every entry point include/ctgb.h
declares, and its host-side geometry/filter tables agree with the oracle.
No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

from ctreconstruction_gb300 import _lib
from ctreconstruction_gb300.geometry import ReconstructionParams
from oracle.oracle import OracleGeometry, ramp_filter
from _util import cone_params, load_golden

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ctgb.h")


def declared_symbols():
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(ctgb_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    assert lib.ctgb_version().decode().startswith("ctgb")


def _table(params, flavour=None):
    c = ReconstructionParams.from_dict(params, flavour).to_ctgb()
    n = ctypes.c_size_t(0)
    _lib.call("ctgb_table_bytes", ctypes.byref(c), ctypes.byref(n))
    buf = np.zeros(n.value // 4, dtype=np.float32)
    _lib.call("ctgb_table_build", ctypes.byref(c), buf.ctypes.data_as(ctypes.c_void_p), n.value)
    return buf


def _header(buf):
    i = buf.view(np.int32)
    f = buf
    h = dict(nx=i[0], ny=i[1], nz=i[2], nu=i[3], nv=i[4], nviews=i[5], curved=i[6], flavour=i[7])
    names = ["eps_fwd", "eps_bp", "dx", "dy", "dz", "du_bp", "dv_bp", "sad", "sdd", "src0x", "src0y", "src0z",
             "det0y", "dtheta", "du_fwd", "dv_fwd", "u0_fwd"]
    for k, nm in enumerate(names):
        h[nm] = float(f[8 + k])
    off = buf.view(np.int64)
    base = (8 + len(names) + 1) // 2   # int64 index after the float block (+pad0)
    keys = ["off_xplane", "off_yplane", "off_zplane", "off_xpix", "off_ypix", "off_zpix", "off_ki", "off_pp",
            "off_views", "view_stride"]
    for k, nm in enumerate(keys):
        h[nm] = int(off[base + k])
    return h


@pytest.mark.parametrize("name,flavour", [("numba_offcentre", "numba"), ("pycuda_offset", "pycuda"),
                                          ("numba_helical", "numba"), ("numba_curved", "numba")])
def test_geometry_table_matches_oracle_geometry(name, flavour):
    p, fl, _ = load_golden(name)
    buf = _table(p, fl)
    h = _header(buf)
    g = OracleGeometry(p, fl)
    assert (h["nx"], h["ny"], h["nz"], h["nu"], h["nv"], h["nviews"]) == (g.nx, g.ny, g.nz, g.nu, g.nv, g.nviews)
    assert h["sad"] == pytest.approx(g.sad, rel=1e-6) and h["sdd"] == pytest.approx(g.sdd, rel=1e-6)
    assert h["dtheta"] == pytest.approx(g.dtheta, rel=1e-6)
    C = p['ReconCenter'] if fl == 'pycuda' else p['PhantomCenter']
    xplane = C[0] + (np.arange(g.nx + 1) - (g.nx - 1) / 2.0) * g.dx - g.dx / 2
    yplane = C[1] + (np.arange(g.ny + 1) - (g.ny - 1) / 2.0) * -g.dy + g.dy / 2
    np.testing.assert_allclose(buf[h["off_xplane"]:h["off_xplane"] + g.nx + 1], xplane, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(buf[h["off_yplane"]:h["off_yplane"] + g.ny + 1], yplane, rtol=1e-6, atol=1e-6)
    # dominant axis per view, restating distance_forward's test (Reconstruction_numba.py:896,966)
    for v, th in enumerate(g.angles):
        S = np.array([-g.sad * np.sin(th), g.sad * np.cos(th)])
        D = np.array([(g.sdd - g.sad) * np.sin(th), -(g.sdd - g.sad) * np.cos(th)])
        ax, ay = abs(S[0] - D[0]), abs(S[1] - D[1])
        want = 0 if ax >= ay else 1
        rec = buf[h["off_views"] + v * h["view_stride"]:]
        assert int(rec[0]) == want


def test_dominant_axis_ties_break_like_the_reference():
    """At 720 views over 2 pi, views 90, 270, 450 and 630 sit at 45 degrees,
    where |S_x - D_x| and |S_y - D_y| agree to the last bit or two.  The
    table's axis must follow distance_forward's test
    (Reconstruction_numba.py:896,966) evaluated as the reference evaluates it:
    math.sin/cos, NumPy float64 products and differences, no fused
    multiply-adds."""
    import math
    from _util import cfg3_params
    p = cfg3_params(NumberOfImage=[8, 8, 8], NumberOfDetectorPixels=[8, 8])
    buf = _table(p)
    h = _header(buf)
    SAD, SDD = 1000.0, 1500.0
    angles = np.linspace(0.0, 2 * np.pi, 721)[:-1]
    ties = 0
    for v, th in enumerate(angles):
        S = np.array([-SAD * math.sin(th), SAD * math.cos(th)])
        D = np.array([(SDD - SAD) * math.sin(th), -(SDD - SAD) * math.cos(th)])
        ax, ay = abs(S[0] - D[0]), abs(S[1] - D[1])
        ties += ax == ay
        assert int(buf[h["off_views"] + v * h["view_stride"]]) == (0 if ax >= ay else 1), v
    assert ties >= 1


def test_quarter_turn_views_are_exact_rotations():
    """On a full circular orbit with a view count divisible by 4 the table
    stores view v + n/4 as the exact rotation (x, y) -> (-y, x) of view v's
    float values, except in groups whose dominant axis does not alternate (the
    45-degree views, where the reference's tie-break slices along x twice):
    the symmetric backprojectors share set-ups across those groups."""
    from _util import cfg3_params
    p = cfg3_params(NumberOfImage=[8, 8, 8], NumberOfDetectorPixels=[16, 8])
    buf = _table(p)
    h = _header(buf)
    nu, n, q = 16, 720, 180
    rec = lambda v: buf[h["off_views"] + v * h["view_stride"]:h["off_views"] + (v + 1) * h["view_stride"]]
    bx, by = 16, 16 + nu + 1                  # Bx[nu+1], By[nu+1] after the 16 scalars
    axes = [int(rec(v)[0]) for v in range(n)]
    broken = {g for g in range(q) if any(axes[(g + (k + 1) * q) % n] != 1 - axes[g + k * q] for k in range(3))}
    assert broken == {90}                     # the 45-degree group: views 90, 270, 450, 630
    for v in range(q, n):
        if v % q in broken:
            continue
        a, b = rec(v - q), rec(v)
        assert b[1] == -a[2] and b[2] == a[1], v                        # source x, y
        assert np.array_equal(b[bx:bx + nu + 1], -a[by:by + nu + 1]), v  # column boundaries
        assert np.array_equal(b[by:by + nu + 1], a[bx:bx + nu + 1]), v


@pytest.mark.parametrize("over,nc", [({}, 4), ({'NumberOfImage': [12, 10, 8]}, 2), ({'NumberOfViews': 18}, 2),
                                     ({'ReconCenter': [0.5, 0.0, 0.0]}, 1), ({'Pitch': 0.5}, 1),
                                     ({'EndAngle': np.pi + 0.4}, 1), ({'NumberOfImage': [11, 12, 8]}, 2),
                                     ({'NumberOfImage': [11, 11, 8]}, 1)])
def test_fdk_orbit_size(over, nc):
    """The rotation-orbit size the FDK backprojector can share set-ups over:
    4 for a square grid of even side centred on the axis on a full orbit of
    4k views, 2 for an even-height grid (or 4k + 2 views), 1 otherwise."""
    p = cone_params(n=12, nviews=16, nu=20, nv=16, **over)
    c = ReconstructionParams.from_dict(p, None).to_ctgb()
    got = ctypes.c_int32(0)
    _lib.call("ctgb_backproject_fdk_orbit_size", ctypes.byref(c), ctypes.byref(got))
    assert got.value == nc


def test_backprojection_entry_points_reject_bad_arguments_on_the_host():
    """The backprojection entry points check their arguments on the host and
    return before any launch: NULL pointers, base or view ranges outside the
    scan, a missing or too small workspace, and the bounded-wait self-test's
    poll count.  The device pointers are placeholders that no failing call
    reaches."""
    c = ReconstructionParams.from_dict(cone_params(n=12, nviews=16, nu=20, nv=16), None).to_ctgb()
    dev = ctypes.c_void_p(256)
    nc = ctypes.c_int32(0)
    _lib.call("ctgb_backproject_fdk_orbit_size", ctypes.byref(c), ctypes.byref(nc))
    assert nc.value == 4
    period = c.nviews // nc.value
    with pytest.raises(ValueError, match="NULL argument"):
        _lib.call("ctgb_backproject_fdk_orbits", ctypes.byref(c), None, dev, dev, 0, 1, 1.0, 0, None)
    with pytest.raises(ValueError, match="base views"):
        _lib.call("ctgb_backproject_fdk_orbits", ctypes.byref(c), dev, dev, dev, period - 1, 2, 1.0, 0, None)
    with pytest.raises(ValueError, match="NULL workspace"):
        _lib.call("ctgb_backproject_matched_ws", ctypes.byref(c), dev, dev, dev, 0, 1, 1.0, 0, None, 0, None)
    with pytest.raises(ValueError, match="workspace below one view"):
        _lib.call("ctgb_backproject_matched_ws", ctypes.byref(c), dev, dev, dev, 0, 1, 1.0, 0, dev, 16, None)
    with pytest.raises(ValueError, match="view range"):
        _lib.call("ctgb_backproject_matched_ws", ctypes.byref(c), dev, dev, dev, 0, c.nviews + 1, 1.0, 0, dev,
                  1 << 30, None)
    for polls in (0, (1 << 20) + 1):
        with pytest.raises(ValueError, match="polls"):
            _lib.call("ctgb_selftest_bounded_wait", polls, None)


def test_table_rejects_bad_geometry():
    p = ReconstructionParams.from_dict(cone_params()).to_ctgb()
    p.nu = 0
    n = ctypes.c_size_t(0)
    with pytest.raises(ValueError, match="sizes must be positive"):
        _lib.call("ctgb_table_bytes", ctypes.byref(p), ctypes.byref(n))
    p = ReconstructionParams.from_dict(cone_params()).to_ctgb()
    _lib.call("ctgb_table_bytes", ctypes.byref(p), ctypes.byref(n))
    small = np.zeros(8, dtype=np.float32)
    with pytest.raises(ValueError, match="too small"):
        _lib.call("ctgb_table_build", ctypes.byref(p), small.ctypes.data_as(ctypes.c_void_p), small.nbytes)


def test_empty_view_ranges_need_no_buffers():
    """An empty view range is a no-op that needs no device buffers (an empty
    tensor's data pointer is NULL); a range outside the scan is still an
    error (host-only: nothing is launched)."""
    p = ReconstructionParams.from_dict(cone_params(nviews=16)).to_ctgb()
    for view0 in (0, 7, 16):
        _lib.call("ctgb_forward", ctypes.byref(p), None, None, None, None, view0, 0, None)
        _lib.call("ctgb_forward_static", ctypes.byref(p), None, None, None, view0, 0, None)
    with pytest.raises(ValueError, match="view range"):
        _lib.call("ctgb_forward", ctypes.byref(p), None, None, None, None, 17, 0, None)
    with pytest.raises(ValueError, match="view range"):
        _lib.call("ctgb_forward_static", ctypes.byref(p), None, None, None, -1, 0, None)
    with pytest.raises(ValueError, match="NULL"):
        _lib.call("ctgb_forward_static", ctypes.byref(p), None, None, None, 0, 1, None)
    with pytest.raises(ValueError, match="NULL"):   # projections read: they must be there
        _lib.call("ctgb_backproject_fdk", ctypes.byref(p), ctypes.c_void_p(16), None, ctypes.c_void_p(16), 0, 1,
                  1.0, 1, None)


def test_null_device_pointers_are_rejected_without_a_launch():
    p = ReconstructionParams.from_dict(cone_params()).to_ctgb()
    with pytest.raises(ValueError, match="NULL"):
        _lib.call("ctgb_forward", ctypes.byref(p), None, None, None, None, 0, 1, None)
    with pytest.raises(ValueError, match="view range"):
        _lib.call("ctgb_backproject_fdk", ctypes.byref(p), ctypes.c_void_p(16), ctypes.c_void_p(16),
                  ctypes.c_void_p(16), 10, 100, 1.0, 0, None)


def test_batch_plans_validate_jobs_on_the_host():
    """The batched plans check their jobs before anything touches a device:
    no jobs, a view range outside the scan, a missing epilogue operand."""
    p = ReconstructionParams.from_dict(cone_params(nviews=8)).to_ctgb()
    n = ctypes.c_size_t(0)
    fake = ctypes.c_void_p(256)
    with pytest.raises(ValueError, match="no jobs"):
        _lib.call("ctgb_batch_forward_plan_bytes", None, 0, ctypes.byref(n))
    job = _lib.CtgbFwdJob(ctypes.pointer(p), fake, fake, fake, fake, 4, 8, _lib.FWD_STORE, 0.0, None, None)
    with pytest.raises(ValueError, match="view range"):
        _lib.call("ctgb_batch_forward_plan_bytes", ctypes.byref(job), 1, ctypes.byref(n))
    job = _lib.CtgbFwdJob(ctypes.pointer(p), fake, fake, fake, fake, 0, 8, _lib.FWD_POCS_RESIDUAL, 1e-5, None, None)
    with pytest.raises(ValueError, match="needs p0"):
        _lib.call("ctgb_batch_forward_plan_bytes", ctypes.byref(job), 1, ctypes.byref(n))
    job = _lib.CtgbFwdJob(ctypes.pointer(p), fake, fake, fake, fake, 0, 8, _lib.FWD_STORE, 0.0, None, None)
    _lib.call("ctgb_batch_forward_plan_bytes", ctypes.byref(job), 1, ctypes.byref(n))
    assert n.value > 0
    ws = ctypes.c_size_t(0)
    _lib.call("ctgb_backproject_fdk_workspace_bytes", ctypes.byref(p), 8, ctypes.byref(ws))
    bj = _lib.CtgbBpJob(ctypes.pointer(p), fake, fake, fake, fake, ws.value - 4, 0, 8, 1.0, 0, _lib.BP_STORE,
                        0.0, 0.0, None, None)
    with pytest.raises(ValueError, match="workspace"):
        _lib.call("ctgb_batch_backproject_plan_bytes", ctypes.byref(bj), 1, ctypes.byref(n))
    bj = _lib.CtgbBpJob(ctypes.pointer(p), fake, fake, fake, fake, ws.value, 0, 8, 1.0, 0, _lib.BP_EM_UPDATE,
                        0.0, 0.0, None, None)
    with pytest.raises(ValueError, match="epilogue output"):
        _lib.call("ctgb_batch_backproject_plan_bytes", ctypes.byref(bj), 1, ctypes.byref(n))


def test_filter_apply_rejects_bad_row_lengths_without_a_launch():
    """ctgb_filter_apply sizes its shared memory from zpl: a length that is not
    a power of two in [2, 8192] is refused on the host (nothing launched)."""
    fake = ctypes.c_void_p(256)
    for zpl in (0, 1, 3, 96, 16384):
        with pytest.raises(ValueError, match="bad arguments"):
            _lib.call("ctgb_filter_apply", fake, zpl, fake, 4, None)
    _lib.call("ctgb_filter_apply", fake, 64, fake, 0, None)   # no rows: no launch


@pytest.mark.parametrize("ft,cut", [("ram-lak", 1.0), ("shepp-logan", 0.3), ("cosine", 1.0), ("hamming", 1.0),
                                    ("hann", 0.5)])
def test_filter_table_matches_oracle_spectrum(ft, cut):
    params = cone_params(nu=40, nv=8, du=0.7)
    c = ReconstructionParams.from_dict(params).to_ctgb()
    n = ctypes.c_size_t(0)
    _lib.call("ctgb_filter_bytes", ctypes.byref(c), ctypes.byref(n))
    buf = np.zeros(n.value // 4, dtype=np.float32)
    _lib.call("ctgb_filter_build", ctypes.byref(c), _lib.FILTER_TYPES[ft], cut, buf.ctypes.data_as(ctypes.c_void_p),
              n.value)
    i = buf.view(np.int32)
    zpl = int(i[0])
    assert zpl == int(2 ** np.ceil(np.log2(2.0 * (40 - 1))))
    off_h = int(buf.view(np.int64)[4])
    R, D = 100.0, 50.0
    tau = 0.7 * R / (R + D)
    want = np.fft.ifftshift(ramp_filter(zpl + 1, tau, ft, cut)) * tau / zpl
    np.testing.assert_allclose(buf[off_h:off_h + zpl], want, rtol=2e-6, atol=1e-7 * np.abs(want).max())


def test_integration_table_names_every_declared_symbol():
    with open(os.path.join(os.path.dirname(HEADER), "..", "INTEGRATION.md")) as f:
        text = f.read()
    missing = [s for s in declared_symbols() if not re.search(r"`%s[`(]" % s, text)]
    assert not missing, missing


def test_product_never_imports_the_oracle():
    pkg = os.path.join(os.path.dirname(HEADER), "..", "ctreconstruction_gb300")
    for root, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cpp", ".h", ".cuh")):
                with open(os.path.join(root, f)) as fh:
                    text = fh.read()
                assert "import oracle" not in text and "from oracle" not in text, f


def test_forward_tile_rows():
    """ctgb_forward_tile_rows: 32-row tiles while a detector row spans at
    most 1.3 voxel rows where rays meet the volume, else 16 (host-only)."""
    def rows(p):
        c = ReconstructionParams.from_dict(p).to_ctgb()
        n = ctypes.c_int32(0)
        _lib.call("ctgb_forward_tile_rows", ctypes.byref(c), ctypes.byref(n))
        return n.value
    # (dv / dz) * (SAD + half-diagonal) / SDD: 1.5 * (100 + 17) / 150 = 1.17
    assert rows(cone_params(n=24, dv=1.5)) == 32
    assert rows(cone_params(n=24, dv=1.75)) == 16                      # 1.37
    assert rows(cone_params(n=24, dv=1.5, PhantomCenter=[20.0, 0.0, 0.0])) == 16   # 1.37 off centre
    assert rows(cone_params(n=(24, 24, 32), dv=2.0)) == 16
    assert rows(cone_params(n=(24, 24, 24), dv=1.6)) == 32             # 1.25
    # 512^3 at 0.5 mm, 0.75 mm rows, SAD 1000, SDD 1500: 1.18
    big = dict(cone_params(n=512, dx=0.5, dv=0.75, nu=1024, nv=768, nviews=720),
               SourceInit=[0.0, 1000.0, 0.0], DetectorInit=[0.0, -500.0, 0.0])
    assert rows(big) == 32


@pytest.mark.parametrize("flavour", ["numba", "pycuda"])
def test_forward_tile_rows_follows_its_bound(flavour):
    """The tile-height choice over seeded random geometries equals
    (dv / dz) * (SAD + |centre - origin| + in-plane half-diagonal) / SDD <= 1.3,
    with the centre the flavour's volume centre (host-only)."""
    rng = np.random.default_rng(7)
    for _ in range(40):
        sad = rng.uniform(50.0, 1200.0)
        sdd = sad * rng.uniform(1.1, 2.5)
        n = [int(v) for v in rng.integers(8, 600, size=3)]
        dx = float(rng.uniform(0.2, 2.0))
        dv = float(rng.uniform(0.2, 3.0))
        pc = [float(v) for v in rng.uniform(-20.0, 20.0, size=3)]
        rc = [float(v) for v in rng.uniform(-20.0, 20.0, size=3)]
        org = [float(v) for v in rng.uniform(-5.0, 5.0, size=2)] + [0.0]
        p = dict(cone_params(n=tuple(n), dx=dx, dv=dv), SourceInit=[org[0], org[1] + sad, 0.0],
                 DetectorInit=[org[0], org[1] - (sdd - sad), 0.0], RotationOrigin=org, PhantomCenter=pc,
                 ReconCenter=rc)
        centre = rc if flavour == "pycuda" else pc
        reach = sad + np.hypot(centre[0] - org[0], centre[1] - org[1]) + 0.5 * np.hypot(n[0] * dx, n[1] * dx)
        ratio = dv / dx * reach / sdd
        if abs(ratio - 1.3) < 1e-6:
            continue
        c = ReconstructionParams.from_dict(p, flavour).to_ctgb()
        rows = ctypes.c_int32(0)
        _lib.call("ctgb_forward_tile_rows", ctypes.byref(c), ctypes.byref(rows))
        assert rows.value == (32 if ratio <= 1.3 else 16), (ratio, rows.value)


def test_forward_launch_count():
    """ctgb_forward_launches: a full circle from theta 0 alternates y, x, y,
    x, y dominant views, which take one launch per axis; more than 2048
    views of one axis take another launch (host-only call)."""
    p = cone_params(n=16, nviews=360, nu=32, nv=24, start=0.0, span=2 * np.pi)
    c = ReconstructionParams.from_dict(p).to_ctgb()
    n = ctypes.c_int32(0)
    _lib.call("ctgb_forward_launches", ctypes.byref(c), 0, 360, ctypes.byref(n))
    assert n.value == 2
    _lib.call("ctgb_forward_launches", ctypes.byref(c), 0, 10, ctypes.byref(n))
    assert n.value == 1
    c6 = ReconstructionParams.from_dict(cone_params(n=16, nviews=6000, nu=32, nv=24)).to_ctgb()
    _lib.call("ctgb_forward_launches", ctypes.byref(c6), 0, 6000, ctypes.byref(n))
    assert n.value == 4     # 3000 views per axis: two launches each
    with pytest.raises(ValueError):
        _lib.call("ctgb_forward_launches", ctypes.byref(c), 350, 20, ctypes.byref(n))
