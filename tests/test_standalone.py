"""CPU checks of the standalone reconstructors' oracle and host logic:
the FP64 restatement against the reference's own Filter functions and its
compiled interpolation kernels (tests/golden/conebeam_ref.npz), and the
"key: value" parameter-file parser."""
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
