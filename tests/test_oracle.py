"""The CPU oracle against the reference's own outputs (golden vectors from
python/Reconstruction_numba.py and python/Reconstruction_pycuda.py, see
tests/golden/make_golden.py) and against its own adjoint identity."""
import numpy as np
import pytest

from oracle.oracle import OracleGeometry
from _util import golden_cases, golden_ids, load_golden, rel_err, cone_params

ORACLE_TOL = 1e-5   # FP64 restatement vs the reference's float32 arithmetic


@pytest.mark.parametrize("name", golden_ids())
def test_oracle_matches_reference_golden(name):
    p, flavour, d = load_golden(name)
    g = OracleGeometry(p, flavour)
    if "forward" in d.files:
        assert rel_err(g.forward(d["image"]), d["forward"]) < ORACLE_TOL
    if "backward" in d.files:
        assert rel_err(g.backward_fdk(d["proj"]), d["backward"]) < ORACLE_TOL
    for k in d.files:
        if k.startswith("filter_"):
            _, ft, co = k.split("_")
            assert rel_err(g.filtering(d["proj"], ft, float(co)), d[k]) < ORACLE_TOL, k


def test_golden_set_covers_the_path():
    names = golden_ids()
    assert any(n.startswith("numba_") for n in names) and any(n.startswith("pycuda_") for n in names)
    kinds = set()
    for _, p, fl, d in golden_cases():
        kinds.update(d.files)
        kinds.add(p.get("DetectorShape", "Flat"))
        if p.get("Pitch", 0):
            kinds.add("helical")
    for need in ("forward", "backward", "Curved", "helical", "filter_ram-lak_1", "filter_hann_1",
                 "filter_shepp-logan_1", "filter_cosine_1", "filter_hamming_1"):
        assert need in kinds, need


def test_oracle_matched_is_adjoint():
    p = cone_params(n=(9, 8, 7), nviews=6, nu=14, nv=11)
    g = OracleGeometry(p)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(g.nz * g.ny * g.nx).astype(np.float32).reshape(g.nz, g.ny, g.nx)
    y = rng.standard_normal(g.nviews * g.nv * g.nu).astype(np.float32).reshape(g.nviews, g.nv, g.nu)
    lhs = float(np.sum(g.forward(x) * y.astype(np.float64)))
    rhs = float(np.sum(x.astype(np.float64) * g.backward_matched(y)))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))


def test_oracle_fdk_backprojector_is_not_the_adjoint():
    """The reference's backward() carries dtheta and R^2/(R-y)^2: it is not A^T."""
    p = cone_params(n=8, nviews=6, nu=12, nv=10)
    g = OracleGeometry(p)
    rng = np.random.default_rng(1)
    x = rng.random((8, 8, 8), dtype=np.float32)
    y = rng.random((6, 10, 12), dtype=np.float32)
    lhs = float(np.sum(g.forward(x) * y))
    rhs = float(np.sum(x * g.backward_fdk(y)))
    assert abs(lhs / rhs - 1.0) > 1e-3


def test_oracle_view_ranges_compose():
    p = cone_params(n=10, nviews=8, nu=16, nv=12)
    g = OracleGeometry(p)
    rng = np.random.default_rng(2)
    x = rng.random((10, 10, 10), dtype=np.float32)
    full = g.forward(x)
    part = np.concatenate([g.forward(x, 0, 3), g.forward(x, 3, 5)])
    assert np.array_equal(full, part)
    y = rng.random((8, 12, 16), dtype=np.float32)
    whole = g.backward_fdk(y)
    split = g.backward_fdk(y[:5], 0, 5) + g.backward_fdk(y[5:], 5, 3)
    assert np.allclose(whole, split, rtol=1e-12, atol=1e-12)


def test_os_sart_oracle_one_subset_is_the_pocs_formula():
    """oracle.os_sart with one subset and one pass from zero is one POCS step
    with the matched pair; two subsets of 3 views cover the 6-view scan."""
    from oracle import oracle as ora
    from _util import cone_params
    p = cone_params(n=(10, 9, 8), nviews=6, nu=20, nv=16)
    g = ora.OracleGeometry(p)
    rng = np.random.default_rng(2)
    proj0 = rng.random((6, 16, 20)).astype(np.float32)
    got = ora.os_sart(p, proj0, 1, 1, lam=0.8)
    a1 = g.forward(np.ones((8, 9, 10), np.float32))
    b1 = g.backward_matched(np.ones((6, 16, 20), np.float32))
    r = np.where(a1 == 0, 0, proj0 / (a1 + 1e-5))
    b = g.backward_matched(r.astype(np.float32))
    want = np.maximum(0.8 * np.where(b1 == 0, 0, b) / (b1 + 1e-5), 0)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()
    subs = [ora.OracleGeometry(dict(p, StartAngle=s * 2 * np.pi / 6, EndAngle=s * 2 * np.pi / 6 + 2 * np.pi,
                                    NumberOfViews=3)) for s in range(2)]
    ang = np.sort(np.concatenate([q.angles for q in subs]))
    assert np.allclose(ang, g.angles)
