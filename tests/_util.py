"""Shared helpers for the tests: golden fixtures and error measures."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Parity bar: float32 results within 1e-4 of the reference / FP64 oracle,
# measured as max|a-b| / max|b| over the whole projection stack or volume.
RTOL = 1e-4


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def _dd_golden_files():
    """Golden vectors of the DD path (Reconstruction_numba / _pycuda)."""
    return [f for f in sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))
            if os.path.basename(f).startswith(("numba_", "pycuda_"))]


def golden_cases():
    out = []
    for f in _dd_golden_files():
        d = np.load(f)
        out.append((os.path.basename(f)[:-4], json.loads(str(d["params"])), str(d["flavour"]), d))
    return out


def golden_ids():
    return [os.path.basename(f)[:-4] for f in _dd_golden_files()]


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return json.loads(str(d["params"])), str(d["flavour"]), d


def cone_params(n=24, nviews=16, nu=40, nv=32, du=1.0, dv=1.0, dx=1.0, start=0.0, span=2 * np.pi, **kw):
    p = {'SourceInit': [0.0, 100.0, 0.0], 'DetectorInit': [0.0, -50.0, 0.0], 'StartAngle': start,
         'EndAngle': start + span, 'NumberOfDetectorPixels': [nu, nv], 'DetectorPixelSize': [du, dv],
         'NumberOfViews': nviews, 'ImagePixelSpacing': [dx, dx, dx],
         'NumberOfImage': [n, n, n] if isinstance(n, int) else list(n),
         'PhantomCenter': [0.0, 0.0, 0.0], 'RotationOrigin': [0.0, 0.0, 0.0], 'ReconCenter': [0.0, 0.0, 0.0],
         'Method': 'Distance', 'FilterType': 'hann', 'cutoff': 1.0, 'GPU': 1, 'DetectorShape': 'Flat',
         'Pitch': 0.0}
    p.update(kw)
    return p


def cfg3_params(**kw):
    """The DD-pair benchmark scan: 512^3 at 0.5 mm, 720 views over 2 pi,
    1024x768 detector at 0.75 mm, SAD 1000 mm, SDD 1500 mm."""
    p = {'SourceInit': [0.0, 1000.0, 0.0], 'DetectorInit': [0.0, -500.0, 0.0], 'StartAngle': 0.0,
         'EndAngle': 2 * np.pi, 'NumberOfDetectorPixels': [1024, 768], 'DetectorPixelSize': [0.75, 0.75],
         'NumberOfViews': 720, 'ImagePixelSpacing': [0.5, 0.5, 0.5], 'NumberOfImage': [512, 512, 512],
         'PhantomCenter': [0.0, 0.0, 0.0], 'RotationOrigin': [0.0, 0.0, 0.0], 'ReconCenter': [0.0, 0.0, 0.0],
         'Method': 'Distance', 'FilterType': 'hann', 'cutoff': 1.0, 'GPU': 1, 'DetectorShape': 'Flat',
         'Pitch': 0.0}
    p.update(kw)
    return p


def cfg1_params(**kw):
    """The FDK benchmark scan: 128^3 at 1 mm, 360 views over 2 pi, 256x192
    detector at 1.5 mm, SAD 1000 mm, SDD 1500 mm, Hann ramp."""
    p = cfg3_params(NumberOfDetectorPixels=[256, 192], DetectorPixelSize=[1.5, 1.5], NumberOfViews=360,
                    ImagePixelSpacing=[1.0, 1.0, 1.0], NumberOfImage=[128, 128, 128])
    p.update(kw)
    return p
