"""Generate the golden vectors in tests/golden/*.npz from the reference itself.

Give the reference checkout as the first argument or in the
``CTGB_REFERENCE_ROOT`` environment variable; the fixtures it writes are
committed, so the tests never need the reference at run time.

* numba flavour (``python/Reconstruction_numba.py`` + ``GPUFuncs_numba.py``):
  run unmodified with ``GPU: 1`` on the serial CPU stand-in for numba in
  ``_numba_stub.py``.  Gives ``forward()``, ``backward()`` (flat and curved
  detectors) and ``Filtering()`` for every filter type.
* pycuda flavour (``python/Reconstruction_pycuda.py``): run unmodified with the
  reference's CUDA-C kernels compiled for the host (``oracle/build_ref.py``)
  behind the pycuda stand-in in ``_pycuda_stub.py``.  Gives ``forward()`` and
  ``backward()`` with ``ReconCenter`` and ``DetectorOffset`` in play.

Inputs are seeded, so rerunning reproduces the files.

    python tests/golden/make_golden.py /path/to/reference [--only-fanbeam]
    CTGB_REFERENCE_ROOT=/path/to/reference python tests/golden/make_golden.py
"""
import copy
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)

PI = np.pi


def base_params(**kw):
    p = {'SourceInit': [0.0, 100.0, 0.0], 'DetectorInit': [0.0, -50.0, 0.0], 'StartAngle': 0.0,
         'EndAngle': 2 * PI, 'NumberOfDetectorPixels': [16, 12], 'DetectorPixelSize': [1.0, 1.0],
         'NumberOfViews': 12, 'ImagePixelSpacing': [0.8, 0.7, 0.9], 'NumberOfImage': [10, 12, 8],
         'PhantomCenter': [0.0, 0.0, 0.0], 'RotationOrigin': [0.0, 0.0, 0.0], 'ReconCenter': [0.0, 0.0, 0.0],
         'Method': 'Distance', 'FilterType': 'hann', 'cutoff': 1.0, 'GPU': 1, 'DetectorShape': 'Flat',
         'Pitch': 0.0}
    p.update(kw)
    return p


# (name, params, what): what is a subset of {"forward", "backward", "filter"}
NUMBA_CASES = [
    ("numba_basic", base_params(), {"forward", "backward", "filter"}),
    ("numba_offcentre", base_params(PhantomCenter=[0.6, -0.4, 0.3], ReconCenter=[-0.5, 0.35, -0.2],
                                    StartAngle=0.3, EndAngle=0.3 + PI, NumberOfViews=7,
                                    NumberOfImage=[9, 11, 6], ImagePixelSpacing=[1.0, 0.9, 1.1]),
     {"forward", "backward"}),
    ("numba_helical", base_params(Pitch=0.5, NumberOfViews=10, SourceInit=[0.0, 100.0, 0.5],
                                  DetectorInit=[0.0, -50.0, 0.5]), {"forward", "backward"}),
    ("numba_curved", base_params(DetectorShape='Curved', NumberOfViews=9), {"forward", "backward"}),
    ("numba_fan", base_params(NumberOfDetectorPixels=[24, 1], NumberOfImage=[12, 12, 1],
                              ImagePixelSpacing=[0.9, 0.9, 1.0], DetectorPixelSize=[1.0, 1.5],
                              NumberOfViews=16), {"forward", "backward", "filter"}),
    ("numba_wide", base_params(NumberOfDetectorPixels=[20, 14], DetectorPixelSize=[0.6, 0.7],
                               NumberOfImage=[12, 10, 9], ImagePixelSpacing=[0.5, 0.55, 0.6],
                               NumberOfViews=8, StartAngle=0.1, EndAngle=0.1 + 2 * PI), {"forward", "backward"}),
]

FILTER_TYPES = [('ram-lak', 1.0), ('shepp-logan', 1.0), ('cosine', 1.0), ('hamming', 1.0), ('hann', 1.0),
                ('hann', 0.5), ('shepp-logan', 0.3)]

PYCUDA_CASES = [
    ("pycuda_basic", dict(base_params(), DetectorOffset=[0.0, 0.0])),
    ("pycuda_offset", dict(base_params(ReconCenter=[0.4, -0.3, 0.25], PhantomCenter=[9.0, 9.0, 9.0],
                                       StartAngle=-0.2, EndAngle=-0.2 + 2 * PI, NumberOfViews=9,
                                       NumberOfImage=[11, 9, 7]), DetectorOffset=[0.45, -0.3])),
]


def inputs_for(p, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = p['NumberOfImage']
    nu, nv = p['NumberOfDetectorPixels']
    image = rng.random((nz, ny, nx), dtype=np.float32)
    proj = rng.random((p['NumberOfViews'], nv, nu), dtype=np.float32)
    return image, proj


def run_case(Recon, p, image, proj, what):
    out = {}
    if "forward" in what:
        R = Recon(copy.deepcopy(p))
        R.image = image.copy()
        R.forward()
        out["forward"] = np.asarray(R.proj, dtype=np.float32)
    if "backward" in what:
        R = Recon(copy.deepcopy(p))
        R.proj = proj.copy()
        R.backward()
        out["backward"] = np.asarray(R.image, dtype=np.float32)
    return out


def conebeam_golden(ref_root, lib_path):
    """python/ConeBeamGPU.py's reconstruction on a small case: the filter
    spectrum from the reference's ConeBeam.Filter (ConeBeam.py parses; the
    GPU file does not under Python 3), its filtering loop (ConeBeamGPU.py:
    296-302) and, for the backprojection, the reference's own kernels
    CalculateInterpolGrid + Interpol2dLineargpu run through oracle/_ref."""
    import ctypes
    import ConeBeam as CB
    import FanBeam as FB
    p = {'SourceToAxis': 100.0, 'SourceToDetector': 150.0, 'DetectorPixelWidth': 1.1, 'DetectorPixelHeight': 1.2,
         'DetectorWidth': 24, 'DetectorHeight': 16, 'NumberOfViews': 12, 'AngleCoverage': 2 * PI,
         'ReconX': 16, 'ReconY': 16, 'ReconZ': 8}
    R, D = p['SourceToAxis'], p['SourceToDetector'] - p['SourceToAxis']
    nx, ny, ns = p['DetectorWidth'], p['DetectorHeight'], p['NumberOfViews']
    X, Y, Z = p['ReconX'], p['ReconY'], p['ReconZ']
    rng = np.random.default_rng(300)
    proj = rng.random((ny, nx, ns)).astype(np.float32)             # reference layout: views last
    zpl = int(2 ** np.ceil(np.log2(2 * (nx - 1))))
    filt = CB.ConeBeam.Filter(zpl + 1, p['DetectorPixelWidth'] * R / (D + R), 'ram-lak', 0.3)
    fov = 2 * R * np.sin(np.arctan(nx * p['DetectorPixelWidth'] / 2 / (D + R)))
    fovz = 2 * R * np.sin(np.arctan(ny * p['DetectorPixelHeight'] / 2 / (D + R)))
    x = np.linspace(-fov / 2, fov / 2, X); y = np.linspace(-fov / 2, fov / 2, Y); z = np.linspace(-fovz / 2, fovz / 2, Z)
    xx, yy = np.meshgrid(x, y)
    ang = np.linspace(0, p['AngleCoverage'], ns + 1)[:-1]
    dtheta = ang[1] - ang[0]
    ki = (np.arange(0, nx) - (nx - 1) / 2) * p['DetectorPixelWidth'] * R / (R + D)
    pp = (np.arange(0, ny) - (ny - 1) / 2) * p['DetectorPixelHeight'] * R / (R + D)
    kk, ppm = np.meshgrid(ki, pp)
    weight = R / np.sqrt(R ** 2 + kk ** 2 + ppm ** 2)
    lib = ctypes.CDLL(lib_path)
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    pad = 64
    ki_pad = np.zeros(nx + 2 * pad, np.float32); ki_pad[pad:pad + nx] = ki
    pp_pad = np.zeros(ny + 2 * pad, np.float32); pp_pad[pad:pad + ny] = pp
    dest = np.zeros(X * Y * Z, np.float32)
    IX, IY, IW = (np.zeros(X * Y * Z, np.float32) for _ in range(3))
    zz = z.astype(np.float32)
    interp = np.array([ki.min(), ki[1] - ki[0], pp.min(), pp[1] - pp[0], nx, ny, X, Y, Z, 0, dtheta], np.float32)
    gridp = np.array([R, X, Y, Z], np.float32)
    Qs = np.zeros((ns, ny, nx), np.float32)
    for i in range(ns):
        wproj = weight * np.fliplr(proj[:, :, i])
        Q = np.zeros(wproj.shape)
        for k in range(ny):
            tmp = np.real(np.fft.ifft(np.fft.ifftshift(filt * np.fft.fftshift(np.fft.fft(wproj[k, :], zpl)))))
            Q[k, :] = tmp[0:nx]
        Qs[i] = Q
        t = (xx * np.cos(ang[i]) + yy * np.sin(ang[i])).flatten().astype(np.float32)
        s_ = (-xx * np.sin(ang[i]) + yy * np.cos(ang[i])).flatten().astype(np.float32)
        Qf = np.ascontiguousarray(Q.flatten().astype(np.float32))
        lib.ref_fdk_interp_view(fp(dest), fp(Qf), ctypes.cast(ctypes.addressof(ki_pad.ctypes.data_as(
            ctypes.POINTER(ctypes.c_float)).contents) + 4 * pad, ctypes.POINTER(ctypes.c_float)),
            ctypes.cast(ctypes.addressof(pp_pad.ctypes.data_as(ctypes.POINTER(ctypes.c_float)).contents) + 4 * pad,
                        ctypes.POINTER(ctypes.c_float)),
            fp(IX), fp(IY), fp(IW), fp(t), fp(s_), fp(zz), fp(gridp), fp(interp), 4)
    fan = {}
    for ft, co in (('hann', 0.3), ('ram-lak', 0.3), ('hamming', 0.5)):
        fan['fan_filter_%s_%g' % (ft, co)] = FB.FanBeam.Filter(2049, 0.37, ft, co)
    np.savez_compressed(os.path.join(HERE, "conebeam_ref.npz"), params=json.dumps(p), proj=proj,
                        spectrum=filt, filtered=Qs, recon=dest.reshape(Z, Y, X), **fan)
    print("conebeam_ref: recon range", float(dest.min()), float(dest.max()))


FAN_CASES = [
    # name, params, ReconVolume (x*y), slices (DetectorHeight), seed
    ("fanbeam_square", {'SourceToAxis': 57.0, 'SourceToDetector': 104.0, 'DetectorPixelWidth': 0.9,
                        'DetectorWidth': 61, 'NumberOfViews': 48, 'AngleCoverage': 360.0}, (24, 24), 2, 400),
    ("fanbeam_short", {'SourceToAxis': 80.0, 'SourceToDetector': 150.0, 'DetectorPixelWidth': 1.1,
                       'DetectorWidth': 45, 'NumberOfViews': 36, 'AngleCoverage': 240.0}, (32, 32), 1, 401),
]
# (Reconstruction() supports square images only: it adds a [ReconX, ReconY]
# reshape of the [ReconY, ReconX] interpolation grid to a [ReconY, ReconX]
# weight, FanBeam.py:133-134, which does not broadcast otherwise.)


def fanbeam_golden(ref_root):
    """python/FanBeam.py's Reconstruction(), unmodified, on synthetic
    sinograms.  Two defects stop it from running as written, and both are
    bridged from outside the module, the way _numba_stub supplies numba:
    * it calls ceil and log2 without importing them (FanBeam.py:89): they are
      supplied as module attributes (math.ceil, math.log2);
    * it hands interp1d the whole zero-padded filtered row Q (FanBeam.py:
      119-128: length ZeroPaddedLength) against the nx detector positions
      gamma, which scipy rejects: the module's interp1d is wrapped to take the
      first nx samples, the truncation the reference's cone-beam scripts
      make (ConeBeamGPU.py:300, Q[k, :] = tmp[0:nx]) and the only reading
      under which the call is defined.
    LoadData() is bypassed (it reads .dat files and keeps only one of them,
    FanBeam.py:160-167): the sinogram [NumberOfViews][DetectorWidth]
    [DetectorHeight] is set on the object directly.  Reconstruction() fixes
    the filter at Hann, cutoff 0.3.  Writes tests/golden/<name>.npz with the
    parameters, sinogram and reconstruction [ReconX][ReconY][DetectorHeight]."""
    import math
    import tempfile
    import _numba_stub
    _numba_stub.install()                    # also registers a matplotlib stand-in
    sys.path.insert(0, os.path.join(ref_root, "python"))
    import FanBeam as FB
    FB.ceil, FB.log2 = math.ceil, math.log2
    scipy_interp1d = FB.interp1d

    def interp1d_first_n(x, y, **kw):
        return scipy_interp1d(x, np.asarray(y)[..., :len(x)], **kw)

    FB.interp1d = interp1d_first_n
    for name, p, (rx, ry), nslices, seed in FAN_CASES:
        with tempfile.TemporaryDirectory() as tmp:
            pf = os.path.join(tmp, "ReconstructionParamsFan.txt")
            with open(pf, "w") as f:
                for k in ('SourceToAxis', 'SourceToDetector', 'DetectorPixelWidth', 'DetectorWidth',
                          'NumberOfViews', 'AngleCoverage'):
                    f.write("%s: %r\n" % (k, p[k]))
                f.write("DetectorHeight: %d\n" % nslices)
                f.write("ReconVolume: %d*%d\n" % (rx, ry))
                f.write("DataPath: %s/\nprecision: float32\n" % tmp)
            R = FB.FanBeam(pf)
            rng = np.random.default_rng(seed)
            sino = rng.random((int(p['NumberOfViews']), int(p['DetectorWidth']), nslices)).astype(np.float32)
            R.sino = sino.astype(np.float64)
            R.Reconstruction(os.path.join(tmp, "recon.dat"))
            recon = np.asarray(R.recon, dtype=np.float32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), params=json.dumps(dict(p, DetectorHeight=nslices,
                                                                                         ReconX=rx, ReconY=ry)),
                            sino=sino, recon=recon)
        print("%s: recon %s range %.4g .. %.4g" % (name, recon.shape, recon.min(), recon.max()))


def main(ref_root):
    sys.path.insert(0, os.path.join(ref_root, "python"))
    import _numba_stub
    _numba_stub.install()
    import Reconstruction_numba as RN

    from oracle import build_ref
    lib = build_ref.build(ref_root)
    import _pycuda_stub
    _pycuda_stub.install(lib)
    import Reconstruction_pycuda as RP

    for i, (name, p, what) in enumerate(NUMBA_CASES):
        t0 = time.time()
        image, proj = inputs_for(p, 100 + i)
        out = run_case(RN.Reconstruction, p, image, proj, what)
        extra = {}
        if "filter" in what:
            for ft, cut in FILTER_TYPES:
                q = dict(p, FilterType=ft, cutoff=cut)
                R = RN.Reconstruction(copy.deepcopy(q))
                R.proj = proj.copy()
                R.Filtering()
                extra["filter_%s_%g" % (ft, cut)] = np.asarray(R.proj, dtype=np.float32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), params=json.dumps(p), flavour="numba",
                            image=image, proj=proj, **out, **extra)
        print("%s: %.1fs %s" % (name, time.time() - t0, sorted(list(out) + list(extra))))

    conebeam_golden(ref_root, lib)

    for i, (name, p) in enumerate(PYCUDA_CASES):
        t0 = time.time()
        image, proj = inputs_for(p, 200 + i)
        out = run_case(RP.Reconstruction, p, image, proj, {"forward", "backward"})
        R = RP.Reconstruction(copy.deepcopy(p))
        R.proj = proj.copy()
        R.Filtering()
        out["filter_%s_%g" % (p['FilterType'], p['cutoff'])] = np.asarray(R.proj, dtype=np.float32)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), params=json.dumps(p), flavour="pycuda",
                            image=image, proj=proj, **out)
        print("%s: %.1fs %s" % (name, time.time() - t0, sorted(out)))


if __name__ == "__main__":
    pos = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = pos[0] if pos else os.environ.get("CTGB_REFERENCE_ROOT")
    if not root or not os.path.isdir(os.path.join(root, "python")):
        sys.exit("make_golden.py: give the reference checkout as the first argument or in CTGB_REFERENCE_ROOT")
    if "--only-fanbeam" in sys.argv:
        fanbeam_golden(root)
    else:
        main(root)
        fanbeam_golden(root)
