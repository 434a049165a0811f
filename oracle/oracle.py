"""Python side of the CPU oracle.  TEST INFRASTRUCTURE: imported only by
tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg, as the
checker.  Nothing in ``ctreconstruction_gb300`` imports it.

* ``OracleGeometry`` restates the reference's host-side geometry
  (python/Reconstruction_numba.py:57-90, python/Reconstruction_pycuda.py:64-99)
  in float64 and packs it for ``ctoracle.c``.
* ``forward`` / ``backward_fdk`` / ``backward_matched`` call the FP64 C
  restatement of the DD kernels.
* ``filtering`` restates ``Filter``/``filter_proj``/``Filtering``
  (Reconstruction_numba.py:190-259) in float64 numpy.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
_LIB = None


class CtGeom(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("nu", ctypes.c_int),
                ("nv", ctypes.c_int), ("nviews", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("du", ctypes.c_double), ("dv", ctypes.c_double), ("sad", ctypes.c_double),
                ("sdd", ctypes.c_double), ("src", ctypes.c_double * 3), ("det", ctypes.c_double * 3),
                ("center_fwd", ctypes.c_double * 3), ("center_bp", ctypes.c_double * 3),
                ("det_offset", ctypes.c_double * 2), ("helical", ctypes.c_double), ("curved", ctypes.c_int),
                ("pycuda", ctypes.c_int), ("eps_fwd", ctypes.c_double), ("eps_bp", ctypes.c_double)]


def build(force=False):
    """Compile ctoracle.c into oracle/_build/libctoracle.so (gcc, OpenMP)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "ctoracle.c")
    lib = os.path.join(BUILD, "libctoracle.so")
    newest = max(os.path.getmtime(src), os.path.getmtime(os.path.abspath(__file__)))
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        # -ffp-contract=off: the same rounding as NumPy (no fused multiply-adds)
        # on every host, so exact ties (a 45-degree view's dominant axis) break
        # the way the reference's NumPy breaks them.
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC", "-std=c11",
                        "-D_DEFAULT_SOURCE", "-o", lib, src, "-lm"], check=True)
    return lib


def lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build())
        P = ctypes.POINTER
        _LIB.ct_forward.argtypes = [P(CtGeom), P(ctypes.c_double), ctypes.c_int, ctypes.c_int,
                                    P(ctypes.c_float), P(ctypes.c_double), ctypes.c_int]
        _LIB.ct_backproject_matched.argtypes = [P(CtGeom), P(ctypes.c_double), ctypes.c_int, ctypes.c_int,
                                                P(ctypes.c_float), P(ctypes.c_double), ctypes.c_int]
        _LIB.ct_backproject_fdk.argtypes = [P(CtGeom), P(ctypes.c_double), ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, P(ctypes.c_float), P(ctypes.c_double), ctypes.c_int]
        _LIB.ct_ray_forward.argtypes = [P(CtGeom), P(ctypes.c_double), ctypes.c_int, ctypes.c_int,
                                        P(ctypes.c_float), P(ctypes.c_double), ctypes.c_int]
        _LIB.ct_ray_backproject.argtypes = [P(CtGeom), P(ctypes.c_double), ctypes.c_int, ctypes.c_int,
                                            P(ctypes.c_float), P(ctypes.c_double)]
    return _LIB


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OracleGeometry:
    """Float64 restatement of the reference's geometry for one params dict.

    flavour 'numba' (Reconstruction_numba.py) or 'pycuda'
    (Reconstruction_pycuda.py): the latter puts the forward planes at
    ReconCenter, adds DetectorOffset and clamps weights at 1e-6 (forward) /
    not at all (backward) instead of 1e-5.
    """

    def __init__(self, params, flavour="numba"):
        p = params
        self.p = p
        self.flavour = flavour
        self.nu, self.nv = (int(v) for v in p['NumberOfDetectorPixels'])
        self.du, self.dv = (float(v) for v in p['DetectorPixelSize'])
        self.nx, self.ny, self.nz = (int(v) for v in p['NumberOfImage'])
        self.dx, self.dy, self.dz = (float(v) for v in p['ImagePixelSpacing'])
        origin = np.array(p.get('RotationOrigin', p.get('Origin', [0, 0, 0])), dtype=np.float64)
        self.src = np.array(p['SourceInit'], dtype=np.float64)
        self.det = np.array(p['DetectorInit'], dtype=np.float64)
        self.sad = float(np.sqrt(np.sum((self.src - origin) ** 2.0)))
        self.sdd = float(np.sqrt(np.sum((self.src - self.det) ** 2.0)))
        self.helical = float(p.get('Pitch', 0)) * (self.nv * self.dv) * self.sad / self.sdd
        self.nviews = int(p['NumberOfViews'])
        a = np.linspace(float(p['StartAngle']), float(p['EndAngle']), self.nviews + 1)
        self.angles = np.ascontiguousarray(a[:-1], dtype=np.float64)
        self.dtheta = float(self.angles[1] - self.angles[0]) if self.nviews > 1 else 0.0
        self.curved = p.get('DetectorShape', 'Flat') == 'Curved'
        rc = p.get('ReconCenter', [0, 0, 0])
        pc = p.get('PhantomCenter', [0, 0, 0])
        g = CtGeom()
        g.nx, g.ny, g.nz, g.nu, g.nv, g.nviews = self.nx, self.ny, self.nz, self.nu, self.nv, self.nviews
        g.dx, g.dy, g.dz, g.du, g.dv = self.dx, self.dy, self.dz, self.du, self.dv
        g.sad, g.sdd = self.sad, self.sdd
        g.src[:] = list(self.src)
        g.det[:] = list(self.det)
        g.center_fwd[:] = [float(v) for v in (rc if flavour == "pycuda" else pc)]
        g.center_bp[:] = [float(v) for v in rc]
        off = p.get('DetectorOffset', [0, 0]) if flavour == "pycuda" else [0, 0]
        g.det_offset[:] = [float(v) for v in off]
        g.helical = self.helical
        g.curved = int(self.curved)
        g.pycuda = int(flavour == "pycuda")
        g.eps_fwd = 1e-6 if flavour == "pycuda" else 1e-5
        g.eps_bp = 0.0 if flavour == "pycuda" else 1e-5
        self.g = g

    # -- projectors ---------------------------------------------------------
    def forward(self, image, view0=0, nview=None, nthreads=0):
        nview = self.nviews - view0 if nview is None else nview
        vol = np.ascontiguousarray(image, dtype=np.float32).reshape(self.nz, self.ny, self.nx)
        out = np.zeros((nview, self.nv, self.nu), dtype=np.float64)
        lib().ct_forward(ctypes.byref(self.g), _dp(self.angles), view0, nview, _fp(vol), _dp(out),
                         nthreads or os.cpu_count())
        return out

    def backward_fdk(self, proj, view0=0, nview=None, nthreads=0, dtheta=None):
        nview = self.nviews - view0 if nview is None else nview
        q = np.ascontiguousarray(proj, dtype=np.float32).reshape(nview, self.nv, self.nu)
        out = np.zeros((self.nz, self.ny, self.nx), dtype=np.float64)
        dt = self.dtheta if dtheta is None else dtheta
        lib().ct_backproject_fdk(ctypes.byref(self.g), _dp(self.angles), view0, nview, dt, _fp(q), _dp(out),
                                 nthreads or os.cpu_count())
        return out

    def backward_matched(self, proj, view0=0, nview=None, nthreads=0):
        nview = self.nviews - view0 if nview is None else nview
        q = np.ascontiguousarray(proj, dtype=np.float32).reshape(nview, self.nv, self.nu)
        out = np.zeros((self.nz, self.ny, self.nx), dtype=np.float64)
        lib().ct_backproject_matched(ctypes.byref(self.g), _dp(self.angles), view0, nview, _fp(q), _dp(out),
                                     nthreads or os.cpu_count())
        return out

    def ray_forward(self, image, view0=0, nview=None, nthreads=0):
        """Siddon ray sums (matlab/RayDrivenProjection3DSiddon.m) to every pixel centre."""
        nview = self.nviews - view0 if nview is None else nview
        vol = np.ascontiguousarray(image, dtype=np.float32).reshape(self.nz, self.ny, self.nx)
        out = np.zeros((nview, self.nv, self.nu), dtype=np.float64)
        lib().ct_ray_forward(ctypes.byref(self.g), _dp(self.angles), view0, nview, _fp(vol), _dp(out),
                             nthreads or os.cpu_count())
        return out

    def ray_backward(self, proj, view0=0, nview=None):
        """Transpose of ray_forward."""
        nview = self.nviews - view0 if nview is None else nview
        q = np.ascontiguousarray(proj, dtype=np.float32).reshape(nview, self.nv, self.nu)
        out = np.zeros((self.nz, self.ny, self.nx), dtype=np.float64)
        lib().ct_ray_backproject(ctypes.byref(self.g), _dp(self.angles), view0, nview, _fp(q), _dp(out))
        return out

    # -- FDK filtering (Reconstruction_numba.py:190-259) ----------------------
    def filtering(self, proj, filter_type=None, cutoff=None):
        ft = self.p.get('FilterType', 'ram-lak') if filter_type is None else filter_type
        co = float(self.p.get('cutoff', 1) if cutoff is None else cutoff)
        return fdk_filter(np.asarray(proj, dtype=np.float64), self.nu, self.nv, self.du, self.dv, self.sad,
                          self.sdd, ft, co,
                          self.p.get('DetectorOffset', [0, 0]) if self.flavour == "pycuda" else [0, 0],
                          pycuda=self.flavour == "pycuda")


def ramp_filter(N, pixel_size, filter_type, cutoff):
    """Reconstruction.Filter (Reconstruction_numba.py:190-225) in float64."""
    x = np.arange(0, N) - (N - 1) / 2.0
    h = np.zeros(len(x))
    h[x == 0] = 1.0 / (8.0 * pixel_size ** 2)
    odd = np.mod(x, 2.0) == 1
    h[odd] = -0.5 / (np.pi * pixel_size * x[odd]) ** 2
    h = h[:-1]
    filt = np.abs(np.fft.fftshift(np.fft.fft(h)))
    w = 2 * np.pi * x[:-1] / (N - 1)
    with np.errstate(divide="ignore", invalid="ignore"):
        if filter_type == 'shepp-logan':
            zero = w == 0
            tmp = filt[zero]
            filt = filt * np.sin(w / (2.0 * cutoff)) / (w / (2.0 * cutoff))
            filt[zero] = tmp * np.sin(w[zero] / (2.0 * cutoff))
        elif filter_type == 'cosine':
            filt = filt * np.cos(w / (2.0 * cutoff))
        elif filter_type == 'hamming':
            filt = filt * (0.54 + 0.46 * np.cos(w / cutoff))
        elif filter_type == 'hann':
            filt = filt * (0.5 + 0.5 * np.cos(w / cutoff))
    filt[np.abs(w) > np.pi * cutoff / (2.0 * pixel_size)] = 0
    return filt


def fdk_filter(proj, nu, nv, du, dv, sad, sdd, filter_type, cutoff, offset=(0, 0), pycuda=False):
    """Filtering + filter_proj (Reconstruction_numba.py:227-259): cosine
    pre-weight at isocentre-scaled detector coordinates, zero-padded ramp
    filter per detector row, times deltaS."""
    R, D = sad, sdd - sad
    zpl = int(2 ** np.ceil(np.log2(2.0 * (nu - 1))))
    ki = (np.arange(0, nu + 1) - nu / 2.0) * du + offset[0]
    p = (np.arange(0, nv + 1) - nv / 2.0) * (-dv if pycuda else dv) + offset[1]
    kk, pp = np.meshgrid(ki[:-1] * R / (R + D), p[:-1] * R / (R + D))
    weight = R / np.sqrt(R ** 2 + kk ** 2 + pp ** 2)
    delta_s = du * R / (R + D)
    filt = ramp_filter(zpl + 1, du * R / (D + R), filter_type, cutoff)
    wp = proj.reshape(-1, nv, nu) * weight[None]
    spec = np.fft.fftshift(np.fft.fft(wp, zpl, axis=-1), axes=-1)
    q = np.real(np.fft.ifft(np.fft.ifftshift(filt * spec, axes=-1), axis=-1))[..., :nu]
    return q * delta_s


# -- iterative drivers (python/SART.py, python/EM.py, python/ASD_POCS.py) -------
def sart(g, proj0, niter, alpha=1.0, eps=1e-5, x0=None):
    """SART.py:27-59 in float32 NumPy over the oracle projectors."""
    f32 = np.float32
    norm1 = g.backward_fdk(np.ones((g.nviews, g.nv, g.nu), np.float32)).astype(f32)
    norm2 = g.forward(np.ones((g.nz, g.ny, g.nx), np.float32)).astype(f32)
    x = np.zeros((g.nz, g.ny, g.nx), f32) if x0 is None else x0.astype(f32).copy()
    for _ in range(niter):
        p = g.forward(x).astype(f32)
        r = (p - proj0) / (norm2 + f32(eps))
        b = g.backward_fdk(r.astype(f32)).astype(f32)
        x = x - f32(alpha) * (b / norm1 + f32(eps))
    return x


def mlem(g, proj0, niter, eps=1e-5, x0=None):
    """EM.py:20-44 (proj0 is modified where the forward projection is zero)."""
    f32 = np.float32
    norm = g.backward_fdk(np.ones((g.nviews, g.nv, g.nu), np.float32)).astype(f32)
    x = np.ones((g.nz, g.ny, g.nx), f32) if x0 is None else x0.astype(f32).copy()
    for _ in range(niter):
        p = g.forward(x).astype(f32)
        proj0[p == 0] = 0
        p[p == 0] = f32(eps)
        r = proj0 / p
        b = g.backward_fdk(r.astype(f32)).astype(f32)
        x = x * (b / norm)
    return x


def os_sart(params, proj0, nsubsets, niter, lam=0.8, eps=1e-5, x0=None, flavour="numba"):
    """Ordered-subsets SART as ctreconstruction_gb300.iterative.OSSART states
    it (no reference counterpart; its update is ASD_POCS.py:171-179's POCS
    step on one subset at a time), in float32 NumPy over the FP64 oracle
    projectors with the matched (transposed) backprojection.  Subset s holds
    views s, s + nsubsets, ...: the scan with StartAngle + s * dtheta and
    NumberOfViews / nsubsets views.  Per subset:
        r = (p0_s - A_s x) / (A_s 1 + eps), 0 where A_s 1 == 0
        x = max(0, x + lam * B_s r / (B_s 1 + eps)), B_s r taken as 0 where B_s 1 == 0."""
    f32 = np.float32
    nv = int(params['NumberOfViews'])
    span = float(params['EndAngle']) - float(params['StartAngle'])
    dth = span / nv
    subsets = []
    for s in range(nsubsets):
        d = dict(params)
        d['StartAngle'] = float(params['StartAngle']) + s * dth
        d['EndAngle'] = d['StartAngle'] + span
        d['NumberOfViews'] = nv // nsubsets
        g = OracleGeometry(d, flavour)
        a1 = g.forward(np.ones((g.nz, g.ny, g.nx), np.float32)).astype(f32)
        b1 = g.backward_matched(np.ones((g.nviews, g.nv, g.nu), np.float32)).astype(f32)
        subsets.append((g, np.ascontiguousarray(proj0[s::nsubsets], dtype=f32), a1, b1))
    g0 = subsets[0][0]
    x = np.zeros((g0.nz, g0.ny, g0.nx), f32) if x0 is None else x0.astype(f32).copy()
    for _ in range(niter):
        for g, ps0, a1, b1 in subsets:
            p = g.forward(x).astype(f32)
            r = np.where(a1 == 0, f32(0), (ps0 - p) / (a1 + f32(eps))).astype(f32)
            b = g.backward_matched(r).astype(f32)
            b = np.where(b1 == 0, f32(0), b)
            x = np.maximum(x + f32(lam) * b / (b1 + f32(eps)), f32(0)).astype(f32)
    return x


def tv_grad(image, eps=1e-7):
    """ASD_POCS.py:55-77 (np.lib.pad replaced by np.pad)."""
    f32 = np.float32
    e = f32(eps)
    x = image
    c = x[1:-1, 1:-1, 1:-1]
    w1 = c - x[0:-2, 1:-1, 1:-1]; w2 = c - x[1:-1, 0:-2, 1:-1]; w3 = c - x[1:-1, 1:-1, 0:-2]
    t1 = (w1 + w2 + w3) / np.sqrt(e + w1 ** 2 + w2 ** 2 + w3 ** 2)
    w4 = x[2:, 1:-1, 1:-1] - c; w5 = x[2:, 1:-1, 1:-1] - x[2:, 0:-2, 1:-1]; w6 = x[2:, 1:-1, 1:-1] - x[2:, 1:-1, 0:-2]
    t2 = (-w4) / np.sqrt(e + w4 ** 2 + w5 ** 2 + w6 ** 2)
    w7 = x[1:-1, 2:, 1:-1] - x[0:-2, 2:, 1:-1]; w8 = x[1:-1, 2:, 1:-1] - c; w9 = x[1:-1, 2:, 1:-1] - x[1:-1, 2:, 0:-2]
    t3 = (-w8) / np.sqrt(e + w7 ** 2 + w8 ** 2 + w9 ** 2)
    w10 = x[1:-1, 1:-1, 2:] - x[0:-2, 1:-1, 2:]; w11 = x[1:-1, 1:-1, 2:] - x[1:-1, 0:-2, 2:]; w12 = x[1:-1, 1:-1, 2:] - c
    t4 = (-w12) / np.sqrt(e + w10 ** 2 + w11 ** 2 + w12 ** 2)
    dtv = t1 + t2 + t3 + t4
    tv_norm = np.sqrt(np.sum(dtv.astype(np.float64) ** 2))
    if abs(tv_norm) < eps:
        tv_norm = 1.0
    dtv = (dtv / f32(tv_norm)).astype(f32)
    return np.pad(dtv, ((1, 1), (1, 1), (1, 1)), 'constant')


def asd_pocs(g, proj0, niter, beta=1.0, beta_red=0.999, na=5, ng=20, alpha=0.007, r_max=0.99, alpha_red=0.95,
             eps=1e-7, x0=None):
    """ASD_POCS.py:137-201; x0 defaults to Filtering() + backward() of proj0."""
    f32 = np.float32
    norm1 = g.backward_fdk(np.ones((g.nviews, g.nv, g.nu), np.float32)).astype(f32)
    norm2 = g.forward(np.ones((g.nz, g.ny, g.nx), np.float32)).astype(f32)
    if x0 is None:
        x = g.backward_fdk(g.filtering(proj0).astype(f32)).astype(f32)
    else:
        x = x0.astype(f32).copy()
    log = []
    for _ in range(niter):
        f0 = x.copy()
        for _a in range(na):
            tmp = x.copy()
            p = g.forward(x).astype(f32)
            r = (proj0 - p) / (norm2 + f32(eps))
            r[norm2 == 0] = 0
            b = g.backward_fdk(r.astype(f32)).astype(f32)
            b[norm1 == 0] = 0
            x = tmp + f32(beta) * b / (norm1 + f32(eps))
            x[x < 0] = 0
        dp = float(np.sqrt(np.sum((x.astype(np.float64) - f0) ** 2)))
        dtvg = alpha * dp
        f0 = x.copy()
        for _g in range(ng):
            x = (x - f32(dtvg) * tv_grad(x, eps)).astype(f32)
        dg = float(np.sqrt(np.sum((x.astype(np.float64) - f0) ** 2)))
        if dg > r_max * dp:
            alpha *= alpha_red
        beta *= beta_red
        log.append({"dtvg": dtvg, "beta": beta, "dp": dp, "dg": dg, "alpha": alpha})
    return x, log
