"""FP64 NumPy restatement of the standalone reconstructors.  TEST
INFRASTRUCTURE (the checker for ctreconstruction_gb300.standalone/fanbeam).

* cone beam: python/ConeBeamGPU.py:203-321 with its kernels
  CalculateInterpolGrid / Interpol2dLineargpu (python/GPUFuncs_pycuda.py:40-102)
* fan beam, line detector: python/FanBeam.py:82-138 (Q truncated to the
  detector width, which the script's interp1d call needs)
* fan beam, arc detector: matlab/FanBeamReconArc.m:20-47, matlab/FilterArc.m
"""
import math

import numpy as np

FILTERS = ('ram-lak', 'shepp-logan', 'cosine', 'hamming', 'hann')


def standalone_filter(N, tau, filter_type, cutoff, arc=False, balanced=False):
    """ConeBeam.Filter / FanBeam.Filter (ConeBeamGPU.py:353-379, FanBeam.py:175-209):
    spectrum doubled, cutoff |w| > pi*cutoff.  arc: matlab/FilterArc.m kernel
    (odd taps -1/(2 pi^2 tau^2 sin^2(n tau))), not doubled, cutoff |w| > pi*cutoff/(2 tau).
    arc and balanced: Kak & Slaney eq. (3.124) kernel (odd taps
    -1/(2 pi^2 sin^2(n tau))), not doubled, cutoff |w| > pi*cutoff."""
    x = np.arange(0, N) - (N - 1) / 2
    h = np.zeros(len(x))
    h[x == 0] = 1 / (8 * tau ** 2)
    odd = np.mod(x, 2) == 1
    if arc:
        h[odd] = -1.0 / (2 * np.pi ** 2 * (1.0 if balanced else tau ** 2) * np.sin(x[odd] * tau) ** 2)
    else:
        h[odd] = -0.5 / (np.pi * tau * x[odd]) ** 2
    h = h[:-1]
    filt = np.abs(np.fft.fftshift(np.fft.fft(h))) * (1.0 if arc else 2.0)
    w = 2 * np.pi * x[:-1] / (N - 1)
    with np.errstate(divide="ignore", invalid="ignore"):
        if filter_type == 'shepp-logan':
            zero = w == 0
            tmp = filt[zero]
            filt = filt * np.sin(w / (2 * cutoff)) / (w / (2 * cutoff))
            filt[zero] = tmp * np.sin(w[zero] / (2 * cutoff))
        elif filter_type == 'cosine':
            filt = filt * np.cos(w / (2 * cutoff))
        elif filter_type == 'hamming':
            filt = filt * (0.54 + 0.46 * np.cos(w / cutoff))
        elif filter_type == 'hann':
            filt = filt * (0.5 + 0.5 * np.cos(w / cutoff))
    lim = np.pi * cutoff / (2 * tau) if (arc and not balanced) else np.pi * cutoff
    filt[np.abs(w) > lim] = 0
    return filt


def _zpl(n):
    return int(2 ** math.ceil(math.log2(2 * (n - 1))))


def _apply(rows, filt, zpl):
    spec = np.fft.fftshift(np.fft.fft(rows, zpl, axis=-1), axes=-1)
    return np.real(np.fft.ifft(np.fft.ifftshift(filt * spec, axes=-1), axis=-1))[..., :rows.shape[-1]]


def conebeam_grids(p):
    R = p['SourceToAxis']
    D = p['SourceToDetector'] - R
    nx, ny = int(p['DetectorWidth']), int(p['DetectorHeight'])
    fov = 2 * R * math.sin(math.atan(nx * p['DetectorPixelWidth'] / 2 / (D + R)))
    fovz = 2 * R * math.sin(math.atan(ny * p['DetectorPixelHeight'] / 2 / (D + R)))
    x = np.linspace(-fov / 2, fov / 2, int(p['ReconX']))
    y = np.linspace(-fov / 2, fov / 2, int(p['ReconY']))
    z = np.linspace(-fovz / 2, fovz / 2, int(p['ReconZ']))
    ki = (np.arange(nx) - (nx - 1) / 2) * p['DetectorPixelWidth'] * R / (R + D)
    pp = (np.arange(ny) - (ny - 1) / 2) * p['DetectorPixelHeight'] * R / (R + D)
    ns = int(p['NumberOfViews'])
    ang = np.linspace(0, p['AngleCoverage'], ns + 1)[:-1]
    return R, D, x, y, z, ki, pp, ang


def conebeam_filter(p, proj, filter_type='ram-lak', cutoff=0.3):
    """proj [ns][ny][nx] -> Q: weight * fliplr(proj), ramp (ConeBeamGPU.py:229-302)."""
    R, D, x, y, z, ki, pp, ang = conebeam_grids(p)
    nx = int(p['DetectorWidth'])
    zpl = _zpl(nx)
    filt = standalone_filter(zpl + 1, p['DetectorPixelWidth'] * R / (D + R), filter_type, cutoff)
    kk, ppm = np.meshgrid(ki, pp)
    weight = R / np.sqrt(R ** 2 + kk ** 2 + ppm ** 2)
    wp = weight[None] * np.asarray(proj, np.float64)[:, :, ::-1]
    return _apply(wp, filt, zpl)


def _lin(v, grid):
    """Interpol2dLineargpu's 1-D weights on an ascending uniform grid."""
    g0, dg, n = grid[0], grid[1] - grid[0], len(grid)
    f = (v - g0) / dg
    lo, hi = np.floor(f).astype(np.int64), np.ceil(f).astype(np.int64)
    ok = (hi < n) & (lo >= 0)
    lc, hc = np.clip(lo, 0, n - 1), np.clip(hi, 0, n - 1)
    w1, w2 = v - grid[lc], grid[hc] - v
    both = (np.abs(w1) < 1e-4) & (np.abs(w2) < 1e-4)
    w1 = np.where(both, 1.0, w1)
    den = np.where(ok, w1 + w2, 1.0)    # samples off the grid are discarded; keep them finite
    return lc, hc, w2 / den, w1 / den, ok


def conebeam_backproject(p, Q):
    """Q [ns][ny][nx] filtered -> recon [Z][Y][X] (the GPU kernels' grid order)."""
    R, D, x, y, z, ki, pp, ang = conebeam_grids(p)
    xx, yy = np.meshgrid(x, y)
    dth = ang[1] - ang[0]
    recon = np.zeros((len(z), len(y), len(x)))
    for i, a in enumerate(ang):
        t = xx * np.cos(a) + yy * np.sin(a)
        s = -xx * np.sin(a) + yy * np.cos(a)
        U = R * t / (R - s)
        W = R ** 2 / (R - s) ** 2
        ul, uh, ua, ub, uok = _lin(U, ki)
        for k, zk in enumerate(z):
            V = R * zk / (R - s)
            vl, vh, va, vb, vok = _lin(V, pp)
            q = Q[i]
            M = ua * q[vl, ul] + ub * q[vl, uh]
            N = ua * q[vh, ul] + ub * q[vh, uh]
            S = va * M + vb * N
            recon[k] += np.where(uok & vok, S * dth * W, 0.0)
    return recon


def fan_filter(sino, R, sdd, pw, arc=False, filter_type='hann', cutoff=0.3, balanced=False):
    """One slice's sinogram [ns][nch] -> Q (FanBeam.py:106-122 / FanBeamReconArc.m:20-27)."""
    nch = sino.shape[-1]
    zpl = _zpl(nch)
    if arc:
        dg = pw / sdd
        gam = (np.arange(nch) - (nch - 1) / 2) * dg
        filt = standalone_filter(zpl + 1, dg, filter_type, cutoff, arc=True, balanced=balanced)
        wp = np.asarray(sino, np.float64) * (R * dg * np.cos(gam))[None]
    else:
        tau = pw * R / sdd
        gam = (np.arange(nch) - (nch - 1) / 2) * tau
        filt = standalone_filter(zpl + 1, tau, filter_type, cutoff)
        wp = np.asarray(sino, np.float64) * (R / np.sqrt(R ** 2 + gam ** 2))[None]
    return _apply(wp, filt, zpl), gam


def fan_backproject(Q, gam, x, y, R, sdd, angles, arc=False):
    """Voxel-driven fan backprojection; image [len(y)][len(x)]."""
    D = sdd - R
    xx, yy = np.meshgrid(x, y)
    dth = angles[1] - angles[0]
    img = np.zeros(xx.shape)
    for i, a in enumerate(angles):
        t = xx * np.cos(a) + yy * np.sin(a)
        s = -xx * np.sin(a) + yy * np.cos(a)
        if arc:
            u = np.arctan2(t, R - s)
            w = 1.0 / ((R - s) ** 2 + t ** 2)
        else:
            u = R * t / (R - s)
            w = 1.0 / ((D - s) / D) ** 2
        vq = np.interp(u, gam, Q[i], left=0.0, right=0.0)
        img += dth * w * vq
    return img
