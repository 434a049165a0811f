"""The allocation-free forward projection (ctgb_forward_static).

Some callers of this library cannot allocate device memory where they call
the projector: an application whose own memory pool owns the whole device
budget and gives plugins no allocation rights, or a latency-bound
reconstruction loop that cannot take cudaMalloc's device-wide
synchronisation.  ctgb_forward_static serves them by keeping its scratch (the
[nz][nx][ny] copy of the volume) in a fixed 16 MiB __device__ array.

This file is collected last, so a failure here comes after every other test
has run.  It checks, through the C ABI, that two consecutive calls (the
second sees the array the first one left behind) match ctgb_forward with a
caller-allocated copy, within the suite's parity tolerance, and that an
oversize volume is refused before anything is launched.
"""
import ctypes

import numpy as np
import pytest
import torch

from ctreconstruction_gb300 import Projector, _lib
from _util import cone_params, rel_err

pytestmark = pytest.mark.gpu


def _call_static(P, vol, out):
    _lib.call("ctgb_forward_static", ctypes.byref(P.c), ctypes.c_void_p(P.table.data_ptr()),
              ctypes.c_void_p(vol.data_ptr()), ctypes.c_void_p(out.data_ptr()), 0, P.params.NumberOfViews,
              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def _call_forward(P, vol, xzy, out):
    nz, ny, nx = P.volume_shape
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("ctgb_transpose_xy", ctypes.c_void_p(vol.data_ptr()), ctypes.c_void_p(xzy.data_ptr()), nx, ny, nz,
              stream)
    _lib.call("ctgb_forward", ctypes.byref(P.c), ctypes.c_void_p(P.table.data_ptr()),
              ctypes.c_void_p(vol.data_ptr()), ctypes.c_void_p(xzy.data_ptr()), ctypes.c_void_p(out.data_ptr()), 0,
              P.params.NumberOfViews, stream)


@pytest.mark.parametrize("shape", [(40, 36, 24), (30, 26, 17)])
def test_static_forward_matches_forward_twice(cuda, shape):
    p = cone_params(n=shape, nviews=16, nu=64, nv=40, dx=0.7)
    P = Projector(p, device=cuda)
    gen = torch.Generator(device=cuda).manual_seed(11)
    for call in range(2):
        vol = torch.rand(P.volume_shape, device=cuda, generator=gen)
        want = torch.empty(P.proj_shape(), device=cuda)
        got = torch.full(P.proj_shape(), float("nan"), device=cuda)
        xzy = torch.empty((shape[2], shape[0], shape[1]), device=cuda)
        _call_forward(P, vol, xzy, want)
        _call_static(P, vol, got)
        torch.cuda.synchronize()
        assert torch.isfinite(got).all(), "call %d" % call
        # Same kernels on the same data: the results are bit-identical.
        assert torch.equal(got, want), "call %d: max rel err %.3e" % (call, rel_err(got.cpu().numpy(),
                                                                                    want.cpu().numpy()))


def test_static_forward_rejects_oversize_volume(cuda):
    n = 176   # 176^3 > 2^22 voxels
    p = cone_params(n=n, nviews=2, nu=8, nv=8)
    P = Projector(p, device=cuda)
    vol = torch.zeros((8,), device=cuda)
    out = torch.zeros((8,), device=cuda)
    with pytest.raises(ValueError, match="exceeds the static scratch"):
        _call_static(P, vol, out)
