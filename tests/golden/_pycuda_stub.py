"""A CPU stand-in for the part of ``pycuda`` that the reference's pycuda
flavour uses.  ``SourceModule(...).get_function(name)`` dispatches to the
reference's own CUDA-C kernels compiled as host code
(``oracle/_ref/libctref.so``, built by ``oracle/build_ref.py``), so the
reference's unmodified ``Reconstruction_pycuda.py`` runs on the CPU.

Test infrastructure only (``make_golden.py``).
"""
import ctypes
import sys
import types

import numpy as np


class GPUArray(np.ndarray):
    def get(self):
        return np.array(self, copy=True).view(np.ndarray)

    def set(self, src):
        self[...] = np.asarray(src, dtype=self.dtype).reshape(self.shape)


def _to_gpu(a):
    return np.ascontiguousarray(np.array(a, copy=True)).view(GPUArray)


def _zeros(shape, dtype=np.float32):
    return np.zeros(shape, dtype=dtype).view(GPUArray)


def _ptr(a):
    a = np.asarray(a)
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class _Module:
    def __init__(self, lib, nthreads):
        self.lib = lib
        self.nthreads = nthreads

    def get_function(self, name):
        lib, nt = self.lib, self.nthreads
        if name in ("distance_project_on_x3", "distance_project_on_y3", "distance_project_on_z3"):
            axis = {"x": 0, "y": 1, "z": 2}[name[len("distance_project_on_")]]

            def fwd(*args, block=None, grid=None):
                param = np.asarray(args[14])
                n_slices = int(param[3 + axis])
                lib.ref_dd_forward3(axis, *[_ptr(a) for a in args], n_slices, nt)
            return fwd
        if name == "flat_distance_backproj_arb2":
            def bp(*args, block=None, grid=None):
                params = np.asarray(args[7])
                nvox = int(params[3]) * int(params[4]) * int(params[5])
                lib.ref_backproj_arb2(*[_ptr(a) for a in args], ctypes.c_long(0), ctypes.c_long(nvox), nt)
            return bp
        raise NotImplementedError("kernel %s has no CPU launcher" % name)


def install(lib_path, nthreads=8):
    lib = ctypes.CDLL(lib_path)
    lib.ref_dd_forward3.restype = None
    lib.ref_backproj_arb2.restype = None

    attr = types.SimpleNamespace(MAX_THREADS_PER_BLOCK="MAX_THREADS_PER_BLOCK", MAX_GRID_DIM_X="MAX_GRID_DIM_X")

    class _Device:
        def __init__(self, i):
            pass

        def get_attributes(self):
            return {"MAX_THREADS_PER_BLOCK": 1024, "MAX_GRID_DIM_X": 2 ** 31 - 1}

    pycuda = types.ModuleType("pycuda")
    drv = types.ModuleType("pycuda.driver")
    drv.Device = _Device
    drv.In = lambda a: a
    autoinit = types.ModuleType("pycuda.autoinit")
    autoinit.context = types.SimpleNamespace(synchronize=lambda: None)
    compiler = types.ModuleType("pycuda.compiler")
    compiler.SourceModule = lambda src, *a, **k: _Module(lib, nthreads)
    gpuarray = types.ModuleType("pycuda.gpuarray")
    gpuarray.to_gpu = _to_gpu
    gpuarray.zeros = _zeros
    gpuarray.zeros_like = lambda a: _zeros(a.shape, a.dtype)
    pycuda.driver, pycuda.autoinit, pycuda.compiler, pycuda.gpuarray = drv, autoinit, compiler, gpuarray
    pycuda._driver = types.SimpleNamespace(device_attribute=attr)
    for name, mod in (("pycuda", pycuda), ("pycuda.driver", drv), ("pycuda.autoinit", autoinit),
                      ("pycuda.compiler", compiler), ("pycuda.gpuarray", gpuarray)):
        sys.modules[name] = mod
