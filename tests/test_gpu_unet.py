"""The learned proximal step's kernels on the GPU: the tcgen05 convolution
against torch's fp32 conv3d on the same bf16 values, the CUDA-core passes
against torch, and the whole network's parameter gradients against the FP64
oracle (oracle/unet.py, bf16 rounding emulated at the same points)."""
import ctypes

import numpy as np
import pytest
import torch
import torch.nn.functional as F

from ctreconstruction_gb300 import _lib
from ctreconstruction_gb300.learned import UNet3D, train
from ctreconstruction_gb300.projector import _ptr, _stream
from oracle import unet as U

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def _torch_conv(x, w):
    """x [N,D,H,W,C] bf16 (values), w [27, Cout, Cin] -> fp32 [N,D,H,W,Cout]."""
    cout, cin = w.shape[1], w.shape[2]
    wt = w.float().reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2).contiguous()
    out = F.conv3d(x.float().permute(0, 4, 1, 2, 3), wt, padding=1)
    return out.permute(0, 2, 3, 4, 1).contiguous()


CONFIGS = [
    # (c0, c1, cout, (n, d, h, w))
    (16, 0, 16, (1, 4, 32, 64)),
    (16, 0, 32, (2, 3, 16, 32)),
    (32, 0, 32, (1, 4, 16, 32)),
    (32, 0, 64, (1, 2, 8, 16)),
    (64, 0, 64, (1, 3, 8, 16)),
    (64, 32, 32, (1, 4, 16, 32)),
    (32, 16, 16, (1, 4, 32, 64)),
    (16, 0, 48, (1, 4, 32, 64)),
    (64, 0, 96, (1, 2, 8, 16)),
    # rows of 128 voxels: the x-tap reuse kernel
    (16, 0, 16, (1, 2, 3, 256)),
    (32, 0, 32, (1, 2, 2, 128)),
    (64, 32, 32, (1, 2, 2, 128)),
    (32, 16, 48, (1, 2, 2, 256)),
    (64, 0, 96, (1, 1, 2, 128)),
    (16, 0, 64, (2, 2, 2, 128)),
]


@pytest.mark.parametrize("c0,c1,cout,dims", CONFIGS)
def test_conv3d_matches_torch(cuda, c0, c1, cout, dims):
    gen = torch.Generator(device=cuda).manual_seed(c0 * 7 + c1 + cout)
    n, d, h, w = dims
    x0 = torch.randn((n, d, h, w, c0), device=cuda, generator=gen).to(torch.bfloat16)
    x1 = torch.randn((n, d, h, w, c1), device=cuda, generator=gen).to(torch.bfloat16) if c1 else None
    wt = (torch.randn((27, cout, c0 + c1), device=cuda, generator=gen) * 0.1).to(torch.bfloat16)
    bias = torch.randn(cout, device=cuda, generator=gen) * 0.1
    blocks = [wt[:, :, :c0].contiguous().reshape(27 * cout, c0)]
    if c1:
        blocks.append(wt[:, :, c0:].contiguous().reshape(27 * cout, c1))
    xin = torch.cat([x0, x1], dim=-1) if c1 else x0
    want = _torch_conv(xin, wt)
    raw = torch.empty((n, d, h, w, cout), device=cuda)
    act = torch.empty((n, d, h, w, cout), device=cuda, dtype=torch.bfloat16)
    for mode, out in ((1, raw), (0, act)):
        _lib.call("ctgb_unet_conv3d", _ptr(x0), c0, _ptr(x1) if c1 else None, c1, _ptr(blocks[0]),
                  _ptr(blocks[1]) if c1 else None, _ptr(bias), _ptr(out), cout, n, d, h, w, mode, _stream())
    torch.cuda.synchronize()
    assert _rel(raw.cpu(), want.cpu()) < 1e-4
    ref_act = torch.relu(want + bias).to(torch.bfloat16).float()
    assert _rel(act.float().cpu(), ref_act.cpu()) < 1e-2           # one bf16 rounding apart at most


@pytest.mark.parametrize("dims", [(1, 4, 32, 64), (2, 3, 5, 128), (1, 2, 3, 200)])
def test_first_layer_matches_input_and_conv(cuda, dims):
    """ctgb_unet_first (CUDA cores, from x) against ctgb_unet_input followed by
    the tensor-core conv on the packed 16-channel input: the same bf16
    products, fp32 sums in another order, so outputs agree to one bf16
    rounding and almost all are identical."""
    n, d, h, w = dims
    gen = torch.Generator(device=cuda).manual_seed(d * h + w)
    x = torch.randn((n, d, h, w), device=cuda, generator=gen) * 0.02
    scale = torch.rand(n, device=cuda, generator=gen) * 0.02 + 0.01
    wt = (torch.randn((27, 16, 16), device=cuda, generator=gen) * 0.3).to(torch.bfloat16).reshape(27 * 16, 16)
    bias = torch.randn(16, device=cuda, generator=gen) * 0.1
    got = torch.empty((n, d, h, w, 16), device=cuda, dtype=torch.bfloat16)
    _lib.call("ctgb_unet_first", _ptr(x), _ptr(scale), _ptr(wt), 16, _ptr(bias), _ptr(got), n, d, h, w, _stream())
    a0 = torch.empty((n, d, h, w, 16), device=cuda, dtype=torch.bfloat16)
    _lib.call("ctgb_unet_input", _ptr(x), _ptr(scale), _ptr(a0), n, d * h * w, _stream())
    torch.cuda.synchronize()
    want = _torch_conv(a0, wt.reshape(27, 16, 16))
    want = torch.relu(want + bias).to(torch.bfloat16)
    assert _rel(got.float().cpu(), want.float().cpu()) < 1e-2
    assert (got == want).float().mean().item() > 0.98
    if w % 128 == 0 or w in (16, 32, 64):
        ref = torch.empty_like(got)
        _lib.call("ctgb_unet_conv3d", _ptr(a0), 16, None, 0, _ptr(wt), None, _ptr(bias), _ptr(ref), 16, n, d, h, w, 0,
                  _stream())
        torch.cuda.synchronize()
        assert _rel(got.float().cpu(), ref.float().cpu()) < 1e-2


def test_conv3d_rejects_bad_shapes(cuda):
    x = torch.zeros((1, 2, 3, 48, 16), device=cuda, dtype=torch.bfloat16)
    wt = torch.zeros((27 * 16, 16), device=cuda, dtype=torch.bfloat16)
    out = torch.zeros((1, 2, 3, 48, 16), device=cuda)
    with pytest.raises(ValueError):
        _lib.call("ctgb_unet_conv3d", _ptr(x), 16, None, 0, _ptr(wt), None, None, _ptr(out), 16, 1, 2, 3, 48, 1,
                  _stream())
    with pytest.raises(ValueError):
        _lib.call("ctgb_unet_conv3d", _ptr(x), 24, None, 0, _ptr(wt), None, None, _ptr(out), 16, 1, 2, 4, 64, 1,
                  _stream())


def test_pool_up_and_wgrad_match_torch(cuda):
    gen = torch.Generator(device=cuda).manual_seed(5)
    n, d, h, w, c = 2, 4, 8, 16, 32
    x = torch.randn((n, d, h, w, c), device=cuda, generator=gen).to(torch.bfloat16)
    p = torch.empty((n, d // 2, h // 2, w // 2, c), device=cuda, dtype=torch.bfloat16)
    _lib.call("ctgb_unet_pool2", _ptr(x), _ptr(p), n, d, h, w, c, _stream())
    want = F.avg_pool3d(x.float().permute(0, 4, 1, 2, 3), 2).permute(0, 2, 3, 4, 1)
    assert _rel(p.float().cpu(), want.cpu()) < 1e-2
    u = torch.empty_like(x)
    _lib.call("ctgb_unet_up2", _ptr(p), _ptr(u), n, d, h, w, c, _stream())
    assert torch.equal(u, p.repeat_interleave(2, 1).repeat_interleave(2, 2).repeat_interleave(2, 3))
    # weight gradient of a 32 -> 16 conv against torch autograd
    g = torch.randn((n, d, h, w, 16), device=cuda, generator=gen).to(torch.bfloat16)
    ch = ctypes.c_int32(0)
    _lib.call("ctgb_unet_wgrad_chunks", n, d, h, w, ctypes.byref(ch))
    part = torch.empty((ch.value, 27, 16, c), device=cuda)
    _lib.call("ctgb_unet_wgrad", _ptr(x), c, _ptr(g), 16, _ptr(part), n, d, h, w, _stream())
    dw = part.sum(0)
    wt = torch.zeros((16, c, 3, 3, 3), device=cuda, requires_grad=True)
    out = F.conv3d(x.float().permute(0, 4, 1, 2, 3), wt, padding=1)
    out.backward(g.float().permute(0, 4, 1, 2, 3))
    want = wt.grad.permute(2, 3, 4, 0, 1).reshape(27, 16, c)
    assert _rel(dw.cpu(), want.cpu()) < 1e-4


def test_network_gradients_match_oracle(cuda):
    net = UNet3D(device=cuda, seed=3)
    rng = np.random.default_rng(4)
    for k, v in net.params.items():       # non-zero head and biases so every path carries gradient
        if k == "head" or k.endswith(".b"):
            v.data.copy_(torch.from_numpy(rng.standard_normal(v.shape) * 0.1).float())
    n, d, h, w = 1, 4, 32, 64
    x = torch.from_numpy(np.abs(rng.standard_normal((n, d, h, w))).astype(np.float32) * 0.02 + 0.01).to(cuda)
    scale = torch.tensor([0.02], device=cuda)
    gy = torch.from_numpy(rng.standard_normal((n, d, h, w)).astype(np.float32)).to(cuda)
    y = net.forward(x, scale, keep=True)
    G = net.backward(gy)
    act = {k: v.float().cpu().numpy().astype(np.float64) for k, v in net._cache[0].items()}
    p = {k: v.detach().cpu().numpy() for k, v in net.params.items()}
    s, g = scale.cpu().numpy(), gy.cpu().numpy()
    y_o, A = U.forward(p, x.cpu().numpy(), s, bf16=True)
    assert _rel(y.cpu().numpy(), y_o) < 1e-3
    # Backward from the GPU's own activations: differences are fp32 vs fp64
    # accumulation plus the bf16 rounding flips they cause in the gradients.
    G_t = U.backward(p, act, s, g, bf16=True)
    # Free-running oracle: a rounding flip in one activation spreads through
    # the following convolutions (9 % of d1b's elements differ by one bf16
    # ulp at this size) and moves ReLU masks, so only a loose agreement holds.
    G_o = U.backward(p, A, s, g, bf16=True)
    for k in G_o:
        a = G[k].cpu().numpy().astype(np.float64)
        err_t = np.linalg.norm(a - G_t[k]) / max(np.linalg.norm(G_t[k]), 1e-30)
        err_o = np.linalg.norm(a - G_o[k]) / max(np.linalg.norm(G_o[k]), 1e-30)
        assert err_t < 2e-2, (k, err_t)
        assert err_o < 1.5e-1, (k, err_o)


def test_training_reduces_loss(cuda):
    """Fit the network to a fixed smoothing operator on random volumes: the
    loss drops well below the identity map's."""
    gen = torch.Generator(device=cuda).manual_seed(0)
    pairs = []
    for _ in range(4):
        v = torch.rand((16, 64, 64), device=cuda, generator=gen) * 0.02
        s = F.avg_pool3d(v[None, None], 3, stride=1, padding=1, count_include_pad=False)[0, 0]
        pairs.append((v, s))
    net = UNet3D(device=cuda, seed=1)
    losses = train(net, pairs, steps=60, batch=2, size=(8, 32, 64), lr=2e-3, seed=0)
    assert np.mean(losses[-10:]) < 0.5 * np.mean(losses[:3])


def test_graph_training_matches_eager(cuda):
    """The graph-replayed training step gives the eager steps' losses and
    parameters bit for bit."""
    gen = torch.Generator(device=cuda).manual_seed(2)
    pairs = []
    for _ in range(3):
        v = torch.rand((16, 32, 64), device=cuda, generator=gen) * 0.02
        pairs.append((v, F.avg_pool3d(v[None, None], 3, stride=1, padding=1, count_include_pad=False)[0, 0]))
    runs = []
    for graph in (False, True):
        net = UNet3D(device=cuda, seed=4)
        losses = train(net, pairs, steps=6, batch=2, size=(8, 32, 64), lr=2e-3, seed=1, graph=graph)
        runs.append((losses, {k: v.detach().clone() for k, v in net.params.items()}))
    assert runs[0][0] == runs[1][0]
    for k in runs[0][1]:
        assert torch.equal(runs[0][1][k], runs[1][1][k]), k


def test_learned_asd_pocs_small(cuda):
    """The whole learned path at 64^3 / 30 views: pairs from ASD-POCS itself,
    a short training run, then ASD-POCS with the learned step (judged by the
    plain TV step) on a held-out phantom.

    Gain over the method without the network: on held-out (pre, post) pairs
    the trained network's output is closer to the TV result than its input
    is (the untrained network is the identity).  The judge keeps the learned
    run within 5 % of the plain run's RMSE whatever it accepts."""
    from ctreconstruction_gb300 import Projector, iterative, learned, phantoms
    p = {'SourceInit': [0.0, 1000.0, 0.0], 'DetectorInit': [0.0, -500.0, 0.0], 'StartAngle': 0.0,
         'EndAngle': 2 * np.pi, 'NumberOfDetectorPixels': [128, 96], 'DetectorPixelSize': [1.5, 1.5],
         'NumberOfViews': 30, 'ImagePixelSpacing': [1.0, 1.0, 1.0], 'NumberOfImage': [64, 64, 64]}
    P = Projector(p, device=cuda)
    asd = dict(alpha=0.05, ng=20, na=3)
    size = (16, 32, 64)
    train_ph = [phantoms.random_ellipsoids((64, 64, 64), n=12, seed=50 + i, device=cuda) * 0.02 for i in range(3)]
    pairs = learned.tv_pairs(P, train_ph, niter=6, crops=8, size=size, seed=0, **asd)
    assert len(pairs) == 3 * 6 * 8
    net = learned.UNet3D(device=cuda, seed=0)
    losses = learned.train(net, pairs, steps=150, batch=4, size=size, lr=1e-3, seed=0)
    assert np.mean(losses[-10:]) < np.mean(losses[:10])
    ph = phantoms.random_ellipsoids((64, 64, 64), n=12, seed=7, device=cuda) * 0.02
    held = learned.tv_pairs(P, [ph], niter=3, crops=4, size=size, seed=1, **asd)
    pre = torch.stack([a for a, _ in held])
    post = torch.stack([b for _, b in held])
    out = net.forward(pre, net.scale)
    err_net = float(((out - post) ** 2).mean())
    err_id = float(((pre - post) ** 2).mean())
    print("held-out TV-step imitation: mse identity %.3e network %.3e" % (err_id, err_net))
    assert err_net < err_id
    proj0 = P.forward(ph)
    norms = iterative.normalisers(P)
    _, r_plain, _ = iterative.asd_pocs(P, proj0, niter=6, norms=norms, phantom=ph, **asd)
    prox = learned.LearnedProx(net, P, proj0, tol=0.01)
    _, r_learn, _ = iterative.asd_pocs(P, proj0, niter=6, norms=norms, phantom=ph, prox=prox, **asd)
    print("rmse plain %.4e learned %.4e accepted %d rejected %d"
          % (r_plain[-1], r_learn[-1], prox.accepted, prox.rejected))
    assert prox.accepted + prox.rejected == 6
    assert r_learn[-1] <= 1.05 * r_plain[-1]
