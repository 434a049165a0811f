"""FP64 NumPy restatement of the learned proximal step's 3-D U-Net
(ctreconstruction_gb300/learned.py) — forward and backward.  TEST
INFRASTRUCTURE: the checker for the library's U-Net kernels, never part of
the product.

`bf16=True` rounds to bfloat16 (round to nearest even) at the points where
the GPU path stores bf16 — the packed input, every post-ReLU activation,
pooled values and the masked gradients fed to convolutions — and uses
bf16-rounded weights, so GPU and oracle differ only by fp32 accumulation
order.  `bf16=False` is plain FP64 (for finite-difference checks of the
oracle itself).

Layout: activations [N, D, H, W, C]; conv weights [27, Cout, Cin] with tap
(dz+1)*9 + (dy+1)*3 + (dx+1); zero padding.
"""
import numpy as np

LAYERS = (
    ("e1a", (16,), 16), ("e1b", (16,), 16),
    ("e2a", (16,), 32), ("e2b", (32,), 32),
    ("b1", (32,), 64), ("b2", (64,), 64),
    ("d2a", (64, 32), 32), ("d2b", (32,), 32),
    ("d1a", (32, 16), 16), ("d1b", (16,), 16),
)
TAPS = [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def to_bf16(a):
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _shift(x, dz, dy, dx):
    """y[v] = x[v + (dz, dy, dx)] with zeros outside (x: [N, D, H, W, C])."""
    y = np.zeros_like(x)
    n, d, h, w, c = x.shape
    zs, ys, xs = slice(max(0, -dz), min(d, d - dz)), slice(max(0, -dy), min(h, h - dy)), slice(max(0, -dx), min(w, w - dx))
    zt, yt, xt = slice(max(0, dz), min(d, d + dz)), slice(max(0, dy), min(h, h + dy)), slice(max(0, dx), min(w, w + dx))
    y[:, zs, ys, xs] = x[:, zt, yt, xt]
    return y


def conv(x, wt):
    """out[v, co] = sum_tap sum_ci x[v + tap, ci] * wt[tap, co, ci]."""
    out = np.zeros(x.shape[:4] + (wt.shape[1],))
    for t, (dz, dy, dx) in enumerate(TAPS):
        out += _shift(x, dz, dy, dx) @ wt[t].T
    return out


def conv_wgrad(x, g):
    """dW[tap, co, ci] = sum_v g[v, co] * x[v + tap, ci]."""
    c = x.shape[-1]
    gw = np.zeros((27, g.shape[-1], c))
    g2 = g.reshape(-1, g.shape[-1])
    for t, (dz, dy, dx) in enumerate(TAPS):
        gw[t] = g2.T @ _shift(x, dz, dy, dx).reshape(-1, c)
    return gw


def conv_dgrad(g, wt):
    """dx[v, ci] = sum_tap sum_co g[v - tap, co] * wt[tap, co, ci]."""
    out = np.zeros(g.shape[:4] + (wt.shape[2],))
    for t, (dz, dy, dx) in enumerate(TAPS):
        out += _shift(g, -dz, -dy, -dx) @ wt[t]
    return out


def pool(x):
    n, d, h, w, c = x.shape
    return x.reshape(n, d // 2, 2, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4, 6))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def up_grad(g):
    n, d, h, w, c = g.shape
    return g.reshape(n, d // 2, 2, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4, 6))


def forward(params, x, scale, bf16=True):
    """params: dict of fp32/fp64 arrays keyed like UNet3D.params; x [N, D, H, W];
    scale [N].  Returns (y, activations)."""
    R = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    x = np.asarray(x, np.float64)
    s = np.asarray(scale, np.float64).reshape(-1, 1, 1, 1)
    W = {k: R(params[k + ".w"]) for k, _, _ in LAYERS}
    B = {k: np.asarray(params[k + ".b"], np.float64) for k, _, _ in LAYERS}
    a0 = np.zeros(x.shape + (16,))
    a0[..., 0] = R((x / s).astype(np.float32)) if bf16 else x / s
    A = {"a0": a0}

    def layer(name, inputs):
        xin = np.concatenate(inputs, axis=-1) if len(inputs) > 1 else inputs[0]
        return R(np.maximum(conv(xin, W[name]) + B[name], 0.0))

    A["e1a"] = layer("e1a", [a0])
    A["e1b"] = layer("e1b", [A["e1a"]])
    A["p1"] = R(pool(A["e1b"]))
    A["e2a"] = layer("e2a", [A["p1"]])
    A["e2b"] = layer("e2b", [A["e2a"]])
    A["p2"] = R(pool(A["e2b"]))
    A["b1"] = layer("b1", [A["p2"]])
    A["b2"] = layer("b2", [A["b1"]])
    A["u2"] = up(A["b2"])
    A["d2a"] = layer("d2a", [A["u2"], A["e2b"]])
    A["d2b"] = layer("d2b", [A["d2a"]])
    A["u1"] = up(A["d2b"])
    A["d1a"] = layer("d1a", [A["u1"], A["e1b"]])
    A["d1b"] = layer("d1b", [A["d1a"]])
    hw = np.asarray(params["head"], np.float64)
    y = x + s[..., 0] * (A["d1b"] @ hw[:16] + hw[16])
    return y, A


def backward(params, A, scale, gy, bf16=True):
    """Gradients of sum(gy * y) w.r.t. every parameter."""
    R = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    s = np.asarray(scale, np.float64).reshape(-1, 1, 1, 1)
    W = {k: R(params[k + ".w"]) for k, _, _ in LAYERS}
    hw = np.asarray(params["head"], np.float64)
    gin = np.asarray(gy, np.float64) * s
    G = {"head": np.concatenate([np.einsum("ndhw,ndhwc->c", gin, A["d1b"]), [gin.sum()]])}
    mask = lambda a: (a > 0).astype(np.float64)

    def grads(name, xs, g):
        G[name + ".w"] = np.concatenate([conv_wgrad(x, g) for x in xs], axis=-1)
        G[name + ".b"] = g.reshape(-1, g.shape[-1]).sum(0)

    g = R(mask(A["d1b"]) * gin[..., None] * hw[:16])
    grads("d1b", [A["d1a"]], g)
    g = R(mask(A["d1a"]) * conv_dgrad(g, W["d1b"]))
    grads("d1a", [A["u1"], A["e1b"]], g)
    gcat1 = conv_dgrad(g, W["d1a"])
    g = R(mask(A["d2b"]) * up_grad(gcat1[..., :32]))
    grads("d2b", [A["d2a"]], g)
    g = R(mask(A["d2a"]) * conv_dgrad(g, W["d2b"]))
    grads("d2a", [A["u2"], A["e2b"]], g)
    gcat2 = conv_dgrad(g, W["d2a"])
    g = R(mask(A["b2"]) * up_grad(gcat2[..., :64]))
    grads("b2", [A["b1"]], g)
    g = R(mask(A["b1"]) * conv_dgrad(g, W["b2"]))
    grads("b1", [A["p2"]], g)
    gp2 = conv_dgrad(g, W["b1"])
    g = R(mask(A["e2b"]) * (up(gp2) / 8.0 + gcat2[..., 64:]))
    grads("e2b", [A["e2a"]], g)
    g = R(mask(A["e2a"]) * conv_dgrad(g, W["e2b"]))
    grads("e2a", [A["p1"]], g)
    gp1 = conv_dgrad(g, W["e2a"])
    g = R(mask(A["e1b"]) * (up(gp1) / 8.0 + gcat1[..., 32:]))
    grads("e1b", [A["e1a"]], g)
    g = R(mask(A["e1a"]) * conv_dgrad(g, W["e1b"]))
    grads("e1a", [A["a0"]], g)
    return G
