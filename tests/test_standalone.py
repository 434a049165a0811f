"""CPU checks of the standalone reconstructors' oracle and host logic:
the FP64 restatement against the reference's own Filter functions and its
compiled interpolation kernels (tests/golden/conebeam_ref.npz), against
python/FanBeam.py's own Reconstruction() (tests/golden/fanbeam_*.npz), and
the "key: value" parameter-file parser."""
import json
import os

import numpy as np
import pytest

from oracle import standalone as sa
from _util import GOLDEN, rel_err

REF = np.load(os.path.join(GOLDEN, "conebeam_ref.npz"))
P = json.loads(str(REF["params"]))


def test_cone_spectrum_matches_reference_filter():
    nx = P['DetectorWidth']
    zpl = sa._zpl(nx)
    R, D = P['SourceToAxis'], P['SourceToDetector'] - P['SourceToAxis']
    got = sa.standalone_filter(zpl + 1, P['DetectorPixelWidth'] * R / (D + R), 'ram-lak', 0.3)
    assert rel_err(got, REF["spectrum"]) < 1e-12


@pytest.mark.parametrize("key", [k for k in REF.files if k.startswith("fan_filter_")])
def test_fan_spectrum_matches_reference_filter(key):
    _, _, ft, co = key.split("_")
    got = sa.standalone_filter(2049, 0.37, ft, float(co))
    assert rel_err(got, REF[key]) < 1e-12


FAN_GOLDENS = ["fanbeam_square", "fanbeam_short"]


def fan_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return json.loads(str(d["params"])), d["sino"], d["recon"]


def fan_oracle_slice(p, sino_slice):
    """FanBeam.Reconstruction (FanBeam.py:82-138) of one slice through the
    FP64 restatement: image [ReconY][ReconX] on linspace(-fov/2, fov/2)."""
    R, sdd, pw, nx = p['SourceToAxis'], p['SourceToDetector'], p['DetectorPixelWidth'], p['DetectorWidth']
    fov = 2 * R * np.sin(np.arctan(nx * pw / 2 / sdd))
    x = np.linspace(-fov / 2, fov / 2, p['ReconX'])
    ns = p['NumberOfViews']
    ang = np.linspace(0, p['AngleCoverage'] * np.pi / 180.0, ns + 1)[:-1]
    Q, gam = sa.fan_filter(sino_slice, R, sdd, pw, False, 'hann', 0.3)
    return sa.fan_backproject(Q, gam, x, x, R, sdd, ang, False)


@pytest.mark.parametrize("name", FAN_GOLDENS)
def test_fan_oracle_matches_reference_fanbeam(name):
    """The FP64 fan-beam restatement reproduces python/FanBeam.py's own
    Reconstruction() (run unmodified by tests/golden/make_golden.py)."""
    p, sino, recon = fan_golden(name)
    for j in range(sino.shape[2]):
        got = fan_oracle_slice(p, sino[:, :, j].astype(np.float64))
        assert rel_err(got, recon[:, :, j]) < 1e-6, j


def test_cone_filtering_and_backprojection_match_reference():
    proj = np.moveaxis(REF["proj"], 2, 0)           # [views][rows][cols]
    q = sa.conebeam_filter(P, proj)
    assert rel_err(q, REF["filtered"]) < 1e-5
    recon = sa.conebeam_backproject(P, REF["filtered"].astype(np.float64))
    assert rel_err(recon, REF["recon"]) < 1e-5


def test_params_txt_parser(tmp_path):
    from ctreconstruction_gb300.standalone import read_params_txt
    f = tmp_path / "p.txt"
    f.write_text("DataPath: ./CBCTData/LogData/\nSourceToAxis: 1000\nSourceToDetector: 1500\n"
                 "DetectorPixelWidth: 0.390625\nDetectorPixelHeight: 0.390625\nDetectorWidth: 1024\n"
                 "DetectorHeight: 768\nNumberOfViews: 680\nAngleCoverage: 360\nprecision: float32\n"
                 "ReconVolume: 512*512*256\n")
    p = read_params_txt(str(f))
    assert p['SourceToAxis'] == 1000.0 and p['DetectorWidth'] == 1024.0
    assert p['ReconX'] == 512 and p['ReconZ'] == 256 and p['precision'] == 'float32'
    assert abs(p['AngleCoverage'] - 2 * np.pi) < 1e-12
    g = tmp_path / "bad.txt"
    g.write_text("SourceToAxis: 10\nBogus: 3\nSourceToDetector: 20\n")
    q = read_params_txt(str(g))
    assert q['SourceToAxis'] == 10.0 and q['SourceToDetector'] == 0   # parse stops at the unknown key


def test_balanced_arc_kernel_reconstructs_analytic_phantom():
    """The oracle's balanced equiangular kernel (Kak & Slaney eq. 3.124) on
    exact line integrals: amplitude 1 and only window smoothing left."""
    import torch
    from ctreconstruction_gb300 import phantoms
    R, sdd, nch, nv, n, px = 570.0, 1040.0, 984, 180, 64, 4.8
    half = (n - 1) / 2 * px
    ell = [(v, cx * half, cy * half, a * half, b * half, ph)
           for v, cx, cy, a, b, ph in phantoms.random_ellipses(12, seed=4)]
    dg = 1.0 / sdd
    gam = (np.arange(nch) - (nch - 1) / 2) * dg
    dth = 2 * np.pi / nv
    sino = phantoms.ellipse_fan_sinogram(ell, R, nv, gam, dth, arc=True, device="cpu").numpy()
    Q, g = sa.fan_filter(sino, R, sdd, 1.0, arc=True, filter_type='hann', cutoff=1.0, balanced=True)
    x = np.linspace(-half, half, n)
    img = sa.fan_backproject(Q, g, x, x, R, sdd, np.arange(nv) * dth, arc=True)
    truth = phantoms.ellipse_image(ell, torch.linspace(-half, half, n), torch.linspace(-half, half, n)).numpy()
    k = (img * truth).sum() / (truth * truth).sum()
    assert abs(k - 1) < 0.05
    assert np.linalg.norm(img - k * truth) / np.linalg.norm(k * truth) < 0.2
