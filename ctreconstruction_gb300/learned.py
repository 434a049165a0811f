"""Learned proximal step for ASD-POCS: a small 3-D U-Net on the tcgen05
convolution kernels (no reference counterpart; it replaces the TV-descent
step of python/ASD_POCS.py:186-190).

Network (3 levels, 16/32/64 channels, 3x3x3 convolutions with ReLU):

    e1 = conv(conv(x))          1 -> 16 -> 16           full resolution
    e2 = conv(conv(pool(e1)))   16 -> 32 -> 32          1/2
    b  = conv(conv(pool(e2)))   32 -> 64 -> 64          1/4
    d2 = conv(conv([up(b), e2]))   96 -> 32 -> 32       1/2
    d1 = conv(conv([up(d2), e1]))  48 -> 16 -> 16       full
    y  = x + s * (w . d1 + b0)     1x1x1 head, residual

x is divided by a per-sample scale s on the way in, so the network sees
unit-range volumes and its output is a correction in the caller's units.
Activations and weights run in bf16 with fp32 accumulation; master weights
are fp32.  Forward and backward are the library's kernels
(ctgb_unet_*); only parameter bookkeeping (slicing weight blocks, summing
per-block partial gradients, Adam) uses torch.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from .projector import _ptr, _stream

# name, input segments (channels of each concatenated input), output channels
# FLOPs of one forward per full-resolution voxel (2 x 27 x Cin x Cout per
# level, with the first layer's single real input channel).
FLOPS_PER_VOXEL = 2 * 27 * (1 * 16 + 16 * 16 + (16 * 32 + 32 * 32) / 8 + (32 * 64 + 64 * 64) / 64
                            + (96 * 32 + 32 * 32) / 8 + 48 * 16 + 16 * 16) + 2 * 16
LAYERS = (
    ("e1a", (16,), 16), ("e1b", (16,), 16),
    ("e2a", (16,), 32), ("e2b", (32,), 32),
    ("b1", (32,), 64), ("b2", (64,), 64),
    ("d2a", (64, 32), 32), ("d2b", (32,), 32),
    ("d1a", (32, 16), 16), ("d1b", (16,), 16),
)


def check_shape(d, h, w):
    """The volume sizes the kernels accept: D, H, W multiples of 4; the
    coarsest level's W (= W/4) 16, 32, 64 or a multiple of 128, and each
    level's H a multiple of 128 / min(W_level, 128)."""
    if d % 4 or h % 4 or w % 4:
        raise ValueError("U-Net volume dims must be multiples of 4, got %s" % ((d, h, w),))
    for k in range(3):
        wl, hl = w >> k, h >> k
        if not (wl in (16, 32, 64) or wl % 128 == 0):
            raise ValueError("U-Net level %d width %d: must be 16, 32, 64 or a multiple of 128" % (k, wl))
        r = 128 // min(wl, 128)
        if hl % r:
            raise ValueError("U-Net level %d height %d: must be a multiple of %d" % (k, hl, r))


def _bf(shape, dev):
    return torch.empty(shape, dtype=torch.bfloat16, device=dev)


class UNet3D:
    def __init__(self, device=None, seed=0):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        g = torch.Generator().manual_seed(seed)
        self.params = {}
        for name, segs, cout in LAYERS:
            cin = sum(segs)
            fan_in = 27 * (1 if name == "e1a" else cin)     # e1a: only channel 0 of its input is non-zero
            w = torch.randn((27, cout, cin), generator=g) * math.sqrt(2.0 / fan_in)
            self.params[name + ".w"] = w.to(self.device)
            self.params[name + ".b"] = torch.zeros(cout, device=self.device)
        # zero head: the untrained network is the identity map
        self.params["head"] = torch.zeros(17, device=self.device)
        for p in self.params.values():
            p.requires_grad_(True)
        self._cache = None

    # -- parameters -------------------------------------------------------------
    def state_dict(self):
        return {k: v.detach().cpu().clone() for k, v in self.params.items()}

    def load_state_dict(self, sd):
        for k, v in sd.items():
            self.params[k].data.copy_(torch.as_tensor(v).to(self.device))

    def save(self, path):
        np.savez(path, **{k: v.numpy() for k, v in self.state_dict().items()})

    def load(self, path):
        d = np.load(path)
        self.load_state_dict({k: torch.from_numpy(d[k]) for k in d.files})

    def _weights(self, need_bw=True):
        """bf16 forward blocks per segment and (need_bw) bf16
        flipped/transposed blocks for the data gradient, rebuilt from the fp32
        masters."""
        fw, bw = {}, {}
        for name, segs, cout in LAYERS:
            w = self.params[name + ".w"].detach()
            blocks, a = [], 0
            for c in segs:
                blocks.append(w[:, :, a:a + c].contiguous().to(torch.bfloat16).reshape(27 * cout, c))
                a += c
            fw[name] = blocks
            # dX = conv(dY, W') with W'[tap][ci][co] = W[26 - tap][co][ci]
            if need_bw:
                bw[name] = w.flip(0).permute(0, 2, 1).contiguous().to(torch.bfloat16).reshape(27 * sum(segs), cout)
        return fw, bw

    # -- kernels -----------------------------------------------------------------
    def _conv(self, xs, blocks, bias, cout, dims, mode):
        n, d, h, w = dims
        x0, c0 = xs[0]
        x1, c1 = xs[1] if len(xs) > 1 else (None, 0)
        if mode == 0:
            out = _bf((n, d, h, w, cout), self.device)
        else:
            out = torch.empty((n, d, h, w, cout), dtype=torch.float32, device=self.device)
        _lib.call("ctgb_unet_conv3d", _ptr(x0), c0, _ptr(x1) if x1 is not None else None, c1, _ptr(blocks[0]),
                  _ptr(blocks[1]) if len(blocks) > 1 else None, _ptr(bias) if bias is not None else None,
                  _ptr(out), cout, n, d, h, w, mode, _stream())
        return out

    def _pool(self, x, dims):
        n, d, h, w = dims
        c = x.shape[-1]
        out = _bf((n, d // 2, h // 2, w // 2, c), self.device)
        _lib.call("ctgb_unet_pool2", _ptr(x), _ptr(out), n, d, h, w, c, _stream())
        return out

    def _up(self, x, dims):
        n, d, h, w = dims                      # output (fine) dims
        c = x.shape[-1]
        out = _bf((n, d, h, w, c), self.device)
        _lib.call("ctgb_unet_up2", _ptr(x), _ptr(out), n, d, h, w, c, _stream())
        return out

    # -- forward -----------------------------------------------------------------
    def forward(self, x, scale, keep=False):
        """x: fp32 [N, D, H, W] (or [D, H, W]); scale: fp32 [N] (or a float).
        Returns y = x + scale * net(x / scale), fp32, same shape as x."""
        squeeze = x.dim() == 3
        if squeeze:
            x = x.unsqueeze(0)
        if not (x.is_cuda and x.dtype == torch.float32):
            raise ValueError("x must be a CUDA float32 tensor")
        x = x.contiguous()
        n, d, h, w = x.shape
        check_shape(d, h, w)
        scale = torch.as_tensor(scale, dtype=torch.float32, device=self.device).reshape(-1).expand(n).contiguous()
        fw, bw = self._weights(need_bw=keep)
        P = self.params
        L1, L2, L3 = (n, d, h, w), (n, d // 2, h // 2, w // 2), (n, d // 4, h // 4, w // 4)
        bias = {k: P[k + ".b"].detach() for k, _, _ in LAYERS}
        act = {}
        if keep:
            # the packed input is kept for e1a's weight gradient
            act["a0"] = _bf((n, d, h, w, 16), self.device)
            _lib.call("ctgb_unet_input", _ptr(x), _ptr(scale), _ptr(act["a0"]), n, d * h * w, _stream())
        # e1a has one real input channel: a CUDA-core pass from x itself
        # instead of 16-channel tensor-core work on mostly zeros.
        act["e1a"] = _bf((n, d, h, w, 16), self.device)
        _lib.call("ctgb_unet_first", _ptr(x), _ptr(scale), _ptr(fw["e1a"][0]), 16, _ptr(bias["e1a"]),
                  _ptr(act["e1a"]), n, d, h, w, _stream())
        act["e1b"] = self._conv([(act["e1a"], 16)], fw["e1b"], bias["e1b"], 16, L1, 0)
        act["p1"] = self._pool(act["e1b"], L1)
        act["e2a"] = self._conv([(act["p1"], 16)], fw["e2a"], bias["e2a"], 32, L2, 0)
        act["e2b"] = self._conv([(act["e2a"], 32)], fw["e2b"], bias["e2b"], 32, L2, 0)
        act["p2"] = self._pool(act["e2b"], L2)
        act["b1"] = self._conv([(act["p2"], 32)], fw["b1"], bias["b1"], 64, L3, 0)
        act["b2"] = self._conv([(act["b1"], 64)], fw["b2"], bias["b2"], 64, L3, 0)
        act["u2"] = self._up(act["b2"], L2)
        act["d2a"] = self._conv([(act["u2"], 64), (act["e2b"], 32)], fw["d2a"], bias["d2a"], 32, L2, 0)
        act["d2b"] = self._conv([(act["d2a"], 32)], fw["d2b"], bias["d2b"], 32, L2, 0)
        act["u1"] = self._up(act["d2b"], L1)
        act["d1a"] = self._conv([(act["u1"], 32), (act["e1b"], 16)], fw["d1a"], bias["d1a"], 16, L1, 0)
        act["d1b"] = self._conv([(act["d1a"], 16)], fw["d1b"], bias["d1b"], 16, L1, 0)
        y = torch.empty_like(x)
        _lib.call("ctgb_unet_head", _ptr(act["d1b"]), _ptr(P["head"].detach()), _ptr(x), _ptr(scale), _ptr(y), n,
                  d * h * w, _stream())
        self._cache = (act, scale, (L1, L2, L3), bw) if keep else None
        return y[0] if squeeze else y

    __call__ = forward

    # -- backward ----------------------------------------------------------------
    def _wgrad(self, x, cin, g, cout, dims):
        n, d, h, w = dims
        ch = ctypes.c_int32(0)
        _lib.call("ctgb_unet_wgrad_chunks", n, d, h, w, ctypes.byref(ch))
        part = torch.empty((ch.value, 27, cout, cin), dtype=torch.float32, device=self.device)
        _lib.call("ctgb_unet_wgrad", _ptr(x), cin, _ptr(g), cout, _ptr(part), n, d, h, w, _stream())
        return part.sum(0)

    def _bgrad(self, g, c):
        nvox = g.numel() // c
        blocks = int(max(1, min(1024, (nvox + 127) // 128)))
        part = torch.empty((blocks, c), dtype=torch.float32, device=self.device)
        _lib.call("ctgb_unet_colsum", _ptr(g), c, nvox, _ptr(part), blocks, _stream())
        return part.sum(0)

    def _layer_grads(self, grads, name, xs, g, dims):
        """Weight/bias gradients of one conv from its inputs xs [(act, c)] and
        output gradient g (bf16, after the ReLU mask)."""
        cout = g.shape[-1]
        parts = [self._wgrad(x, c, g, cout, dims) for x, c in xs]
        grads[name + ".w"] = torch.cat(parts, dim=2) if len(parts) > 1 else parts[0]
        grads[name + ".b"] = self._bgrad(g, cout)

    def _dgrad(self, g, wt, cin_total, dims):
        return self._conv([(g, g.shape[-1])], [wt], None, cin_total, dims, 1)

    def backward(self, gy):
        """Gradients of sum(gy * y) for the last forward(keep=True): a dict of
        fp32 tensors keyed like the parameters."""
        if self._cache is None:
            raise RuntimeError("backward() needs a forward(..., keep=True) first")
        act, scale, (L1, L2, L3), bw = self._cache
        squeeze = gy.dim() == 3
        gy = (gy.unsqueeze(0) if squeeze else gy).contiguous().float()
        n = L1[0]
        vps = L1[1] * L1[2] * L1[3]
        V1 = n * vps
        V2, V3 = V1 // 8, V1 // 64
        dev = self.device
        P = self.params
        grads = {}
        # head
        gd1b = _bf(L1 + (16,), dev)
        nb = ctypes.c_int32(0)
        _lib.call("ctgb_unet_head_grad_blocks", V1, ctypes.byref(nb))
        part = torch.empty((nb.value, 17), dtype=torch.float32, device=dev)
        _lib.call("ctgb_unet_head_grad", _ptr(gy), _ptr(act["d1b"]), _ptr(P["head"].detach()), _ptr(scale),
                  _ptr(gd1b), _ptr(part), n, vps, _stream())
        grads["head"] = part.sum(0)

        def relu_grad(gx, gs, go, a, c, nvox):
            out = _bf(a.shape, dev)
            _lib.call("ctgb_unet_relu_grad", _ptr(gx), gs, go, _ptr(a), _ptr(out), nvox, c, _stream())
            return out

        # d1b: d1a -> d1b
        self._layer_grads(grads, "d1b", [(act["d1a"], 16)], gd1b, L1)
        gx = self._dgrad(gd1b, bw["d1b"], 16, L1)
        gd1a = relu_grad(gx, 16, 0, act["d1a"], 16, V1)
        # d1a: [u1, e1b] -> d1a
        self._layer_grads(grads, "d1a", [(act["u1"], 32), (act["e1b"], 16)], gd1a, L1)
        gcat1 = self._dgrad(gd1a, bw["d1a"], 48, L1)          # [.., 48]: u1 part 0..31, skip part 32..47
        gd2b = _bf(L2 + (32,), dev)
        _lib.call("ctgb_unet_up2_grad", _ptr(gcat1), 48, 0, _ptr(act["d2b"]), _ptr(gd2b), *L2, 32, _stream())
        # d2b: d2a -> d2b
        self._layer_grads(grads, "d2b", [(act["d2a"], 32)], gd2b, L2)
        gx = self._dgrad(gd2b, bw["d2b"], 32, L2)
        gd2a = relu_grad(gx, 32, 0, act["d2a"], 32, V2)
        # d2a: [u2, e2b] -> d2a
        self._layer_grads(grads, "d2a", [(act["u2"], 64), (act["e2b"], 32)], gd2a, L2)
        gcat2 = self._dgrad(gd2a, bw["d2a"], 96, L2)          # u2 part 0..63, skip part 64..95
        gb2 = _bf(L3 + (64,), dev)
        _lib.call("ctgb_unet_up2_grad", _ptr(gcat2), 96, 0, _ptr(act["b2"]), _ptr(gb2), *L3, 64, _stream())
        # b2: b1 -> b2
        self._layer_grads(grads, "b2", [(act["b1"], 64)], gb2, L3)
        gx = self._dgrad(gb2, bw["b2"], 64, L3)
        gb1 = relu_grad(gx, 64, 0, act["b1"], 64, V3)
        # b1: p2 -> b1
        self._layer_grads(grads, "b1", [(act["p2"], 32)], gb1, L3)
        gp2 = self._dgrad(gb1, bw["b1"], 32, L3)
        ge2b = _bf(L2 + (32,), dev)
        _lib.call("ctgb_unet_pool2_grad", _ptr(gp2), _ptr(gcat2), 96, 64, _ptr(act["e2b"]), _ptr(ge2b), *L2, 32,
                  _stream())
        # e2b: e2a -> e2b
        self._layer_grads(grads, "e2b", [(act["e2a"], 32)], ge2b, L2)
        gx = self._dgrad(ge2b, bw["e2b"], 32, L2)
        ge2a = relu_grad(gx, 32, 0, act["e2a"], 32, V2)
        # e2a: p1 -> e2a
        self._layer_grads(grads, "e2a", [(act["p1"], 16)], ge2a, L2)
        gp1 = self._dgrad(ge2a, bw["e2a"], 16, L2)
        ge1b = _bf(L1 + (16,), dev)
        _lib.call("ctgb_unet_pool2_grad", _ptr(gp1), _ptr(gcat1), 48, 32, _ptr(act["e1b"]), _ptr(ge1b), *L1, 16,
                  _stream())
        # e1b: e1a -> e1b
        self._layer_grads(grads, "e1b", [(act["e1a"], 16)], ge1b, L1)
        gx = self._dgrad(ge1b, bw["e1b"], 16, L1)
        ge1a = relu_grad(gx, 16, 0, act["e1a"], 16, V1)
        # e1a: a0 -> e1a (no gradient needed for the input)
        self._layer_grads(grads, "e1a", [(act["a0"], 16)], ge1a, L1)
        return grads


# ---- training ----------------------------------------------------------------

def random_patches(pairs, size, count, generator):
    """count random (pre, post) crops of `size` (d, h, w) from a list of
    (pre, post) volume pairs; returns two [count, d, h, w] tensors."""
    d, h, w = size
    pre, post = [], []
    for _ in range(count):
        i = int(torch.randint(len(pairs), (1,), generator=generator))
        a, b = pairs[i]
        z = int(torch.randint(a.shape[0] - d + 1, (1,), generator=generator))
        y = int(torch.randint(a.shape[1] - h + 1, (1,), generator=generator))
        x = int(torch.randint(a.shape[2] - w + 1, (1,), generator=generator))
        pre.append(a[z:z + d, y:y + h, x:x + w])
        post.append(b[z:z + d, y:y + h, x:x + w])
    return torch.stack(pre).contiguous(), torch.stack(post).contiguous()


def train(net, pairs, steps=200, batch=4, size=(32, 32, 64), lr=1e-3, seed=0, scale=None, log_every=0,
          graph=True):
    """Fit net(pre) ~ post by MSE with Adam (fp32 master weights).  scale:
    the per-sample input scale (default: the pairs' mean absolute pre value).
    Returns the loss history.

    graph: after one eager step, the whole step — the bf16 weight blocks,
    forward, loss, backward and the Adam update — is captured in a CUDA graph
    and replayed, the batch being copied into the graph's static input
    buffers; the results are the eager steps' bit for bit (the same kernels
    in the same order), without the host launching some 200 small kernels
    and torch ops per step.  Losses stay on the device until the end."""
    gen = torch.Generator().manual_seed(seed)
    params = list(net.params.values())
    dev = net.device
    # the device-side (capturable) Adam in both modes, so eager and graph
    # steps do the same arithmetic
    opt = torch.optim.Adam(params, lr=lr, capturable=True)
    if scale is None:
        scale = float(torch.stack([p[0].abs().mean() for p in pairs]).mean().clamp(min=1e-12))
    pre_s = torch.empty((batch,) + tuple(size), dtype=torch.float32, device=dev)
    post_s = torch.empty_like(pre_s)
    scale_t = torch.full((batch,), scale, dtype=torch.float32, device=dev)
    loss_s = torch.zeros((), dtype=torch.float32, device=dev)
    inv_s2 = 1.0 / scale ** 2

    def step():
        y = net.forward(pre_s, scale_t, keep=True)
        diff = y - post_s
        loss_s.copy_((diff * diff).mean() * inv_s2)
        gy = diff * (2.0 * inv_s2 / diff.numel())
        grads = net.backward(gy)
        for k, p in net.params.items():
            p.grad = grads[k]
        opt.step()

    g = None
    losses = []
    for it in range(steps):
        pre, post = random_patches(pairs, size, batch, gen)
        pre_s.copy_(pre)
        post_s.copy_(post)
        if graph and it > 0:
            if g is None:
                torch.cuda.synchronize(dev)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    step()
            g.replay()
        else:
            step()
        losses.append(loss_s.clone())
        if log_every and it % log_every == 0:
            print("step %d loss %.4e" % (it, float(losses[-1])))
    losses = [float(v) for v in torch.stack(losses).cpu()] if losses else []
    net.scale = scale
    return losses


# ---- the learned step inside ASD-POCS -------------------------------------------

class LearnedProx:
    """A `prox` for iterative.asd_pocs: the U-Net's output replaces the TV
    descent, with the plain TV step kept as judge and fallback.

    Every `judge_every`-th call also runs the plain step and projects both
    results: the network's volume is accepted only while its data residual
    ||A x - p|| stays within `tol` (1 %) of the plain step's; otherwise (or
    if the output is not finite) the plain result is used.  Between judged
    calls the network's output is used as is.  `scale` is the network's
    input scale (default: the training scale stored on the net)."""

    def __init__(self, net, projector, proj0, scale=None, tol=0.01, judge_every=1):
        self.net, self.P, self.proj0 = net, projector, proj0
        self.scale = float(scale if scale is not None else getattr(net, "scale", 1.0))
        self.tol, self.judge_every = float(tol), int(judge_every)
        self.calls = self.accepted = self.rejected = 0
        self._proj = None

    def residual(self, x):
        if self._proj is None:
            self._proj = torch.empty(self.P.proj_shape(), dtype=torch.float32, device=x.device)
        self.P.forward(x, out=self._proj)
        return float(torch.linalg.vector_norm(self._proj - self.proj0))

    def __call__(self, x, plain):
        cand = self.net.forward(x, self.scale)
        self.calls += 1
        if self.judge_every > 0 and (self.calls - 1) % self.judge_every == 0:
            ref = plain()
            ok = bool(torch.isfinite(cand).all()) and self.residual(cand) <= (1.0 + self.tol) * self.residual(ref)
            if not ok:
                self.rejected += 1
                return ref
        self.accepted += 1
        return cand


def tv_pairs(projector, phantom_list, niter, crops, size, seed=0, ahead=0, **asd_kwargs):
    """(pre-TV, post-TV) training pairs from ASD-POCS itself: for each
    phantom, project it, run `niter` ASD-POCS iterations and keep `crops`
    random crops of `size` from the volume before and after every TV step.

    ahead = K > 0 pairs the volume before the TV step of iteration k with
    the volume after the TV step of iteration k + K (same crop), for
    k = 0 .. niter - 1 - K: a network fitted to these pairs steps K
    iterations along the plain run's trajectory per call.  Returns a list of
    (pre, post) device tensors."""
    from . import iterative
    gen = torch.Generator().manual_seed(seed)
    d, h, w = size
    ahead = int(ahead)
    if ahead < 0 or ahead >= niter:
        raise ValueError("ahead must be in [0, niter)")
    pairs = []

    def crop_pairs(pre, post):
        nz, ny, nx = pre.shape
        for _ in range(crops):
            z = int(torch.randint(nz - d + 1, (1,), generator=gen))
            y = int(torch.randint(ny - h + 1, (1,), generator=gen))
            x = int(torch.randint(nx - w + 1, (1,), generator=gen))
            pairs.append((pre[z:z + d, y:y + h, x:x + w].clone(), post[z:z + d, y:y + h, x:x + w].clone()))

    norms = iterative.normalisers(projector)
    for ph in phantom_list:
        proj0 = projector.forward(ph)
        if ahead == 0:
            iterative.asd_pocs(projector, proj0, niter=niter, norms=norms, on_tv=crop_pairs, **asd_kwargs)
            continue
        pres, posts = [], []
        iterative.asd_pocs(projector, proj0, niter=niter, norms=norms,
                           on_tv=lambda pre, post: (pres.append(pre.clone()), posts.append(post.clone())),
                           **asd_kwargs)
        for k in range(niter - ahead):
            crop_pairs(pres[k], posts[k + ahead])
        del pres, posts
    return pairs
