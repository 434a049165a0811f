"""CPU checks of the U-Net oracle (oracle/unet.py): its hand-written backward
against central finite differences in plain FP64, and its building blocks
against direct definitions."""
import numpy as np
import pytest

from oracle import unet as U


def _params(rng):
    p = {}
    for name, segs, cout in U.LAYERS:
        cin = sum(segs)
        p[name + ".w"] = rng.standard_normal((27, cout, cin)) * np.sqrt(2.0 / (27 * cin))
        p[name + ".b"] = rng.standard_normal(cout) * 0.05
    p["head"] = rng.standard_normal(17) * 0.1
    return p


def test_conv_matches_direct_sum():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1, 3, 4, 5, 2))
    w = rng.standard_normal((27, 3, 2))
    out = U.conv(x, w)
    z, y, xx, co = 1, 2, 0, 1
    want = 0.0
    for t, (dz, dy, dx) in enumerate(U.TAPS):
        zz, yy, x2 = z + dz, y + dy, xx + dx
        if 0 <= zz < 3 and 0 <= yy < 4 and 0 <= x2 < 5:
            want += x[0, zz, yy, x2] @ w[t, co]
    assert abs(out[0, z, y, xx, co] - want) < 1e-12


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.14159], np.float32)
    r = U.to_bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-12


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = _params(rng)
    x = np.abs(rng.standard_normal((1, 4, 8, 8))) + 0.1
    s = np.array([0.7])
    gy = rng.standard_normal(x.shape)
    f = lambda q: float((U.forward(q, x, s, bf16=False)[0] * gy).sum())
    y, A = U.forward(p, x, s, bf16=False)
    G = U.backward(p, A, s, gy, bf16=False)
    h = 1e-6
    for key in ("e1a.w", "e2b.w", "b2.w", "d2a.w", "d1a.w", "d1b.w", "d1b.b", "b1.b", "head"):
        flat = p[key].reshape(-1)
        for idx in rng.choice(flat.size, 3, replace=False):
            q = {k: v.copy() for k, v in p.items()}
            q[key].reshape(-1)[idx] += h
            fp = f(q)
            q[key].reshape(-1)[idx] -= 2 * h
            fm = f(q)
            num = (fp - fm) / (2 * h)
            ana = G[key].reshape(-1)[idx]
            assert abs(num - ana) <= 1e-5 * max(1.0, abs(num)), (key, idx, num, ana)
