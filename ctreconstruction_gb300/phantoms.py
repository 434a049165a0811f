"""Synthetic phantoms (seeded), generated on the device.

* ``shepp_logan_3d``: the modified 3-D Shepp-Logan phantom (10 ellipsoids,
  Kak & Slaney's axes with Toft's modified intensities, the usual published
  table) on a [-1, 1]^3 grid.
* ``random_ellipsoids``: n ellipsoids with centres uniform in the ball of
  radius 0.8, semi-axes U(a0, a1), uniformly random rotations and additive
  values U(v0, v1) — the synthetic stand-in for the scans the benchmarks name.
"""
import math

import numpy as np
import torch

# (value, a, b, c, x0, y0, z0, phi_deg) — modified Shepp-Logan, 3-D.
_SHEPP_LOGAN_3D = [
    (1.0, 0.6900, 0.920, 0.810, 0.000, 0.0000, 0.00, 0.0),
    (-0.8, 0.6624, 0.874, 0.780, 0.000, -0.0184, 0.00, 0.0),
    (-0.2, 0.1100, 0.310, 0.220, 0.220, 0.0000, 0.00, -18.0),
    (-0.2, 0.1600, 0.410, 0.280, -0.220, 0.0000, 0.00, 18.0),
    (0.1, 0.2100, 0.250, 0.410, 0.000, 0.3500, -0.15, 0.0),
    (0.1, 0.0460, 0.046, 0.050, 0.000, 0.1000, 0.25, 0.0),
    (0.1, 0.0460, 0.046, 0.050, 0.000, -0.1000, 0.25, 0.0),
    (0.1, 0.0460, 0.023, 0.050, -0.080, -0.6050, 0.00, 0.0),
    (0.1, 0.0230, 0.023, 0.020, 0.000, -0.6060, 0.00, 0.0),
    (0.1, 0.0230, 0.046, 0.020, 0.060, -0.6050, 0.00, 0.0),
]


def _grid(shape, device):
    nz, ny, nx = shape
    z = torch.linspace(1.0, -1.0, nz, device=device)    # index 0 is +z (reference axis order)
    y = torch.linspace(1.0, -1.0, ny, device=device)
    x = torch.linspace(-1.0, 1.0, nx, device=device)
    return z, y, x


def _add_ellipsoid(vol, z, y, x, val, axes, centre, rot, chunk=16):
    """vol += val inside {p : |R^T (p - c) / axes| <= 1}, processed in z chunks."""
    a, b, c = axes
    R = torch.as_tensor(rot, dtype=torch.float32, device=vol.device)
    cx, cy, cz = centre
    Y, X = torch.meshgrid(y - cy, x - cx, indexing="ij")
    for z0 in range(0, vol.shape[0], chunk):
        Z = (z[z0:z0 + chunk] - cz)[:, None, None]
        px = X[None] * R[0, 0] + Y[None] * R[1, 0] + Z * R[2, 0]
        py = X[None] * R[0, 1] + Y[None] * R[1, 1] + Z * R[2, 1]
        pz = X[None] * R[0, 2] + Y[None] * R[1, 2] + Z * R[2, 2]
        inside = (px / a) ** 2 + (py / b) ** 2 + (pz / c) ** 2 <= 1.0
        vol[z0:z0 + chunk] += val * inside.to(vol.dtype)


def shepp_logan_3d(shape, device="cuda"):
    vol = torch.zeros(shape, dtype=torch.float32, device=device)
    z, y, x = _grid(shape, device)
    for val, a, b, c, x0, y0, z0, phi in _SHEPP_LOGAN_3D:
        t = math.radians(phi)
        rot = [[math.cos(t), math.sin(t), 0.0], [-math.sin(t), math.cos(t), 0.0], [0.0, 0.0, 1.0]]
        _add_ellipsoid(vol, z, y, x, val, (a, b, c), (x0, y0, z0), rot)
    return vol


def _random_rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
            [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
            [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]


def random_ellipsoids(shape, n=30, seed=1, axes=(0.05, 0.3), values=(-0.2, 0.5), radius=0.8, device="cuda"):
    rng = np.random.default_rng(seed)
    vol = torch.zeros(shape, dtype=torch.float32, device=device)
    z, y, x = _grid(shape, device)
    for _ in range(n):
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        centre = d * radius * rng.random() ** (1.0 / 3.0)
        ax = rng.uniform(axes[0], axes[1], 3)
        val = rng.uniform(values[0], values[1])
        _add_ellipsoid(vol, z, y, x, float(val), tuple(ax), tuple(centre), _random_rotation(rng))
    return vol


def random_ellipses(count=20, seed=0, axes=(0.03, 0.3), values=(-0.1, 0.4), radius=0.8):
    """`count` ellipses (value, cx, cy, a, b, phi) in units of the image
    half-width: centres uniform in the disk of the given radius, semi-axes
    U(axes), angles U(0, pi), additive values U(values)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        r = radius * math.sqrt(rng.random())
        t = 2 * math.pi * rng.random()
        a, b = rng.uniform(axes[0], axes[1], 2)
        out.append((float(rng.uniform(values[0], values[1])), r * math.cos(t), r * math.sin(t), float(a), float(b),
                    float(rng.uniform(0, math.pi))))
    return out


def ellipse_image(ellipses, x, y):
    """Image [len(y)][len(x)] of the ellipses sampled at the pixel centres
    x (ascending) and y; ellipse coordinates are physical (same units)."""
    Y, X = torch.meshgrid(y, x, indexing="ij")
    img = torch.zeros(Y.shape, dtype=torch.float32, device=Y.device)
    for val, cx, cy, a, b, phi in ellipses:
        xr = (X - cx) * math.cos(phi) + (Y - cy) * math.sin(phi)
        yr = -(X - cx) * math.sin(phi) + (Y - cy) * math.cos(phi)
        img += val * (((xr / a) ** 2 + (yr / b) ** 2) <= 1.0).float()
    return img


def ellipse_fan_sinogram(ellipses, R, nviews, gammas, dtheta, arc=False, theta0=0.0, device="cuda"):
    """Exact line integrals of the ellipses along fan rays, [nviews][nch].

    View i has its source at angle theta = theta0 + i*dtheta on the circle of
    radius R: in the rotated frame t = x cos + y sin, s = -x sin + y cos the
    source sits at (t, s) = (0, R).  Channel j's ray passes through the
    point (t, s) = (u_j, 0) with u_j = gammas[j] (line detector, channel
    positions scaled to the axis) or u_j = R tan(gammas[j]) (arc detector,
    channel angles) — the geometry the fan backprojector inverts."""
    th = theta0 + dtheta * torch.arange(nviews, dtype=torch.float64, device=device)
    g = torch.as_tensor(gammas, dtype=torch.float64, device=device)
    u = R * torch.tan(g) if arc else g
    c, s = torch.cos(th)[:, None], torch.sin(th)[:, None]
    sx, sy = -R * s, R * c                                  # source (x, y)
    px, py = u[None] * c, u[None] * s                       # point on the central line
    dx, dy = px - sx, py - sy
    nrm = torch.sqrt(dx * dx + dy * dy)
    dx, dy = dx / nrm, dy / nrm
    sino = torch.zeros((nviews, g.numel()), dtype=torch.float64, device=device)
    for val, cx, cy, a, b, phi in ellipses:
        cp, sp = math.cos(phi), math.sin(phi)
        ox, oy = sx - cx, sy - cy
        p1 = (ox * cp + oy * sp) / a
        p2 = (-ox * sp + oy * cp) / b
        d1 = (dx * cp + dy * sp) / a
        d2 = (-dx * sp + dy * cp) / b
        dd = d1 * d1 + d2 * d2
        pd = p1 * d1 + p2 * d2
        disc = pd * pd - dd * (p1 * p1 + p2 * p2 - 1.0)
        sino += val * 2.0 * torch.sqrt(torch.clamp(disc, min=0.0)) / dd
    return sino.float()
