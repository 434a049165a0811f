"""A serial CPU stand-in for the small part of ``numba`` that the reference's
numba flavour uses (``cuda.jit`` kernels and device functions, ``cuda.atomic.add``,
``cuda.to_device`` / ``device_array`` / ``copy_to_host``).

Test infrastructure only: ``make_golden.py`` installs it into ``sys.modules`` so
that the reference's unmodified ``Reconstruction_numba.py`` and
``GPUFuncs_numba.py`` run on the CPU and produce golden vectors.  Kernels run
one emulated thread after another, which is exact for the reference's kernels
(their only cross-thread interaction is ``atomic.add``).

Typing follows the kernel signature strings: ``float32`` scalar arguments and
device-function results are rounded to ``numpy.float32``, ``int32``/``int16``
to ``int``; array arguments stay ``float32`` arrays.
"""
import re
import sys
import types

import numpy as np


class _Dim:
    __slots__ = ("x", "y", "z")

    def __init__(self):
        self.x = self.y = self.z = 0


class _DeviceArray(np.ndarray):
    def copy_to_host(self):
        return np.array(self, copy=True).view(np.ndarray)

    def copy_to_device(self, src):
        self[...] = np.asarray(src, dtype=self.dtype).reshape(self.shape)


def _to_device(arr):
    return np.array(arr, copy=True).view(_DeviceArray)


def _device_array(shape, dtype=np.float32):
    return np.zeros(shape, dtype=dtype).view(_DeviceArray)


def _parse_sig(sig):
    m = re.match(r"\s*(\w+)\s*\((.*)\)\s*$", sig)
    ret, args = m.group(1), m.group(2)
    kinds = [a.strip() for a in re.split(r",(?![^\[]*\])", args) if a.strip()]
    return ret, kinds


def _caster(kind):
    if kind.endswith("[:]"):
        return lambda v: v
    if kind.startswith("float"):
        return np.float32
    if kind.startswith("int") or kind.startswith("uint"):
        return int
    return lambda v: v


class _Kernel:
    def __init__(self, fn, casts):
        self.fn = fn
        self.casts = casts

    def __getitem__(self, cfg):
        grid, block = cfg
        grid = tuple(grid) + (1,) * (3 - len(tuple(grid))) if isinstance(grid, tuple) else (grid, 1, 1)
        block = tuple(block) + (1,) * (3 - len(tuple(block))) if isinstance(block, tuple) else (block, 1, 1)

        def launch(*args):
            if self.casts is not None:
                args = tuple(c(a) for c, a in zip(self.casts, args))
            cu = _cuda
            cu.gridDim.x, cu.gridDim.y, cu.gridDim.z = grid
            cu.blockDim.x, cu.blockDim.y, cu.blockDim.z = block
            for bz in range(grid[2]):
                for by in range(grid[1]):
                    for bx in range(grid[0]):
                        cu.blockIdx.x, cu.blockIdx.y, cu.blockIdx.z = bx, by, bz
                        for tz in range(block[2]):
                            for ty in range(block[1]):
                                for tx in range(block[0]):
                                    cu.threadIdx.x, cu.threadIdx.y, cu.threadIdx.z = tx, ty, tz
                                    self.fn(*args)
        return launch


def _jit(sig=None, device=False, **kw):
    casts = ret_cast = None
    if isinstance(sig, str):
        ret, kinds = _parse_sig(sig)
        casts = [_caster(k) for k in kinds]
        ret_cast = _caster(ret) if ret != "void" else None

    def deco(fn):
        if device:
            def dev(*args):
                if casts is not None:
                    args = tuple(c(a) for c, a in zip(casts, args))
                r = fn(*args)
                return ret_cast(r) if ret_cast is not None else r
            dev.__name__ = fn.__name__
            return dev
        return _Kernel(fn, casts)

    if callable(sig) and not isinstance(sig, str):
        return deco(sig)
    return deco


def _atomic_add(arr, idx, val):
    arr[idx] += val


class _Device:
    MAX_THREADS_PER_BLOCK = 1024
    MAX_GRID_DIM_X = 2 ** 31 - 1


_cuda = types.ModuleType("numba.cuda")
_cuda.threadIdx, _cuda.blockIdx, _cuda.blockDim, _cuda.gridDim = _Dim(), _Dim(), _Dim(), _Dim()
_cuda.jit = _jit
_cuda.atomic = types.SimpleNamespace(add=_atomic_add)
_cuda.to_device = _to_device
_cuda.device_array = _device_array
_cuda.get_current_device = lambda: _Device()
_cuda.synchronize = lambda: None


def install():
    """Register the stand-ins as ``numba``, ``numba.cuda`` and ``matplotlib``."""
    numba = types.ModuleType("numba")
    numba.cuda = _cuda
    numba.jit = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
    sys.modules["numba"] = numba
    sys.modules["numba.cuda"] = _cuda
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = types.ModuleType("matplotlib.pyplot")
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", mpl.pyplot)
