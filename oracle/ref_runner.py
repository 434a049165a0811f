"""Drive the reference's own kernels compiled for the host
(oracle/_ref/libctref.so, built by oracle/build_ref.py) the way
python/Reconstruction_pycuda.py drives them on a GPU.

TEST INFRASTRUCTURE / CPU BASELINE ONLY.  The host-side per-view set-up is a
float64 NumPy restatement of Reconstruction_pycuda.distance_forward
(:762-1060) and distance_backproj (:320-442); the kernels are the reference's
distance_project_on_{x,y,z}3 and flat_distance_backproj_arb2.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libctref.so")
_lib = None


def available():
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(LIB)
        _lib.ref_dd_forward3.restype = None
        _lib.ref_backproj_arb2.restype = None
        _lib.ref_max_threads.restype = ctypes.c_int
    return _lib


def _fp(a):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class RefScan:
    """Reference (pycuda-flavour) host geometry for one params dict."""

    def __init__(self, p):
        self.p = p
        self.nu, self.nv = (int(v) for v in p['NumberOfDetectorPixels'])
        self.du, self.dv = (float(v) for v in p['DetectorPixelSize'])
        self.nx, self.ny, self.nz = (int(v) for v in p['NumberOfImage'])
        self.dx, self.dy, self.dz = (float(v) for v in p['ImagePixelSpacing'])
        src = np.array(p['SourceInit'], dtype=np.float64)
        det = np.array(p['DetectorInit'], dtype=np.float64)
        org = np.array(p.get('RotationOrigin', [0, 0, 0]), dtype=np.float64)
        self.src, self.det = src, det
        self.sad = float(np.sqrt(np.sum((src - org) ** 2)))
        self.sdd = float(np.sqrt(np.sum((src - det) ** 2)))
        self.H = float(p.get('Pitch', 0)) * (self.nv * self.dv) * self.sad / self.sdd
        n = int(p['NumberOfViews'])
        self.angles = np.linspace(float(p['StartAngle']), float(p['EndAngle']), n + 1)[:-1]
        self.off = [float(v) for v in p.get('DetectorOffset', [0, 0])]
        rc = np.array(p.get('ReconCenter', [0, 0, 0]), dtype=np.float64)
        self.rc = rc
        dx, dy, dz = self.dx, -self.dy, -self.dz
        self.Xplane = (rc[0] + (np.arange(self.nx + 1) - (self.nx - 1) / 2.0) * dx - dx / 2).astype(np.float32)
        self.Yplane = (rc[1] + (np.arange(self.ny + 1) - (self.ny - 1) / 2.0) * dy - dy / 2).astype(np.float32)
        self.Zplane = (rc[2] + (np.arange(self.nz + 1) - (self.nz - 1) / 2.0) * dz - dz / 2).astype(np.float32)

    def _detector(self, S, th):
        nu, nv, du, dv = self.nu, self.nv, self.du, self.dv
        eu = [np.cos(th), np.sin(th), 0]
        ew = [np.sin(th), -np.cos(th), 0]
        u = (np.arange(nu) - (nu - 1.0) / 2.0) * du + self.off[0]
        v = (np.arange(nv) - (nv - 1.0) / 2.0) * -1.0 * dv + self.off[1]
        U, V = np.meshgrid(u, v)
        I = np.zeros([3, nv, nu], dtype=np.float32)
        for k, evk in enumerate((0.0, 0.0, 1.0)):
            I[k] = S[k] + U * eu[k] + self.sdd * ew[k] + V * evk
        u2 = (np.arange(nu + 1) - (nu - 1) / 2.0) * du - du / 2.0 + self.off[0]
        v2 = (np.arange(nv + 1) - (nv - 1) / 2.0) * -1.0 * dv + dv / 2.0 + self.off[1]
        U2, V2 = np.meshgrid(u2, v2)
        B = np.zeros([3, nv + 1, nu + 1], dtype=np.float32)
        for k, evk in enumerate((0.0, 0.0, 1.0)):
            B[k] = S[k] + U2 * eu[k] + self.sdd * ew[k] + V2 * evk
        return I, B

    def forward_view(self, image, i, nthreads=0):
        """One view of Reconstruction_pycuda.distance_forward, float32 [nv, nu]."""
        th = self.angles[i]
        sad, sdd, H = self.sad, self.sdd, self.H
        S = np.array([-sad * np.sin(th), sad * np.cos(th), self.src[2] + H * th / (2 * np.pi)])
        D = np.array([(sdd - sad) * np.sin(th), -(sdd - sad) * np.cos(th), self.det[2] + H * th / (2 * np.pi)])
        I, B = self._detector(S, th)
        U1 = np.array([B[0, :-1, :-1], B[1, :-1, :-1], I[2]])
        U2 = np.array([B[0, 1:, 1:], B[1, 1:, 1:], I[2]])
        V1 = np.array([I[0], I[1], B[2, 1:, 1:]])
        V2 = np.array([I[0], I[1], B[2, :-1, :-1]])
        d = np.abs(S - D)
        if d[0] >= d[1] and d[0] >= d[2]:
            a, b1, b2, axis, da = 0, 1, 2, 0, self.dx
        elif d[1] >= d[0] and d[1] >= d[2]:
            a, b1, b2, axis, da = 1, 0, 2, 1, -self.dy
        else:
            a, b1, b2, axis, da = 2, 0, 1, 2, -self.dz
        sU1 = (S[b1] - U1[b1]) / (S[a] - U1[a]); iU1 = -sU1 * S[a] + S[b1]
        sU2 = (S[b1] - U2[b1]) / (S[a] - U2[a]); iU2 = -sU2 * S[a] + S[b1]
        sV1 = (S[b2] - V1[b2]) / (S[a] - V1[a]); iV1 = -sV1 * S[a] + S[b2]
        sV2 = (S[b2] - V2[b2]) / (S[a] - V2[a]); iV2 = -sV2 * S[a] + S[b2]
        t1 = (S[b1] - I[b1]) / (S[a] - I[a])
        t2 = (S[b2] - I[b2]) / (S[a] - I[a])
        inter = np.abs(da) / (np.cos(np.arctan(t1)) * np.cos(np.arctan(t2)))
        f = [np.ascontiguousarray(x, dtype=np.float32).ravel() for x in
             (sU1, sU2, sV1, sV2, iU1, iU2, iV1, iV2)]
        inter = np.ascontiguousarray(inter, dtype=np.float32).ravel()
        param = np.array([self.dx, -self.dy, -self.dz, self.nx, self.ny, self.nz, self.nu, self.nv, 0],
                         dtype=np.float32)
        dest = np.zeros(self.nu * self.nv, dtype=np.float32)
        src = np.ascontiguousarray(image, dtype=np.float32).ravel()
        n_slices = (self.nx, self.ny, self.nz)[axis]
        lib().ref_dd_forward3(axis, _fp(dest), _fp(src), *[_fp(x) for x in f], _fp(self.Xplane), _fp(self.Yplane),
                              _fp(self.Zplane), _fp(inter), _fp(param), n_slices,
                              nthreads or lib().ref_max_threads())
        return dest.reshape(self.nv, self.nu)

    def backward_view(self, proj_view, i, dtheta, out=None, voxel0=0, nvox=None, nthreads=0):
        """One view of Reconstruction_pycuda.distance_backproj (adds into out)."""
        nu, nv = self.nu, self.nv
        dx, dy, dz, dv = self.dx, -self.dy, -self.dz, -self.dv
        rc = self.rc
        xp = (rc[0] + (np.arange(self.nx) - (self.nx - 1) / 2.0) * dx).astype(np.float32)
        yp = (rc[1] + (np.arange(self.ny) - (self.ny - 1) / 2.0) * dy).astype(np.float32)
        zp = (rc[2] + (np.arange(self.nz) - (self.nz - 1) / 2.0) * dz).astype(np.float32)
        ki = ((np.arange(nu + 1) - (nu - 1) / 2.0) * self.du + self.off[0]).astype(np.float32)
        pp = ((np.arange(nv + 1) - (nv - 1) / 2.0) * dv + self.off[1]).astype(np.float32)
        th = self.angles[i]
        sz = self.src[2] + self.H * th / (2 * np.pi)
        dzz = self.det[2] + self.H * th / (2 * np.pi)
        params = np.array([dx, dy, dz, self.nx, self.ny, self.nz, nu, nv, self.du, dv, self.src[0], self.src[1], sz,
                           self.det[0], self.det[1], dzz, th, 0.0, self.sad, 0], dtype=np.float32)
        q = np.ascontiguousarray(proj_view * dtheta, dtype=np.float32).ravel()
        if out is None:
            out = np.zeros(self.nx * self.ny * self.nz, dtype=np.float32)
        total = self.nx * self.ny * self.nz
        nvox = total - voxel0 if nvox is None else nvox
        lib().ref_backproj_arb2(_fp(out), _fp(q), _fp(xp), _fp(yp), _fp(zp), _fp(ki), _fp(pp), _fp(params),
                                ctypes.c_long(voxel0), ctypes.c_long(nvox), nthreads or lib().ref_max_threads())
        return out
