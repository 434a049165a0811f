"""ctypes binding of libctgb.so (the C ABI declared in include/ctgb.h).

The library is loaded from the package's in-tree build directory.  There is no
fallback: if the library is missing, every projector call raises.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libctgb.so")

CTGB_OK = 0
FLAVOUR_NUMBA = 0
FLAVOUR_PYCUDA = 1
FILTER_TYPES = {'ram-lak': 0, 'shepp-logan': 1, 'cosine': 2, 'hamming': 3, 'hann': 4}


class CtgbParams(ctypes.Structure):
    """Mirror of ``ctgb_params`` (include/ctgb.h)."""
    _fields_ = [("nu", ctypes.c_int32), ("nv", ctypes.c_int32), ("du", ctypes.c_double), ("dv", ctypes.c_double),
                ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("nviews", ctypes.c_int32), ("start_angle", ctypes.c_double), ("end_angle", ctypes.c_double),
                ("source_init", ctypes.c_double * 3), ("detector_init", ctypes.c_double * 3),
                ("rotation_origin", ctypes.c_double * 3), ("phantom_center", ctypes.c_double * 3),
                ("recon_center", ctypes.c_double * 3), ("detector_offset", ctypes.c_double * 2),
                ("pitch", ctypes.c_double), ("curved", ctypes.c_int32), ("flavour", ctypes.c_int32)]


class CtgbConeBeamParams(ctypes.Structure):
    """Mirror of ``ctgb_conebeam_params`` (include/ctgb.h)."""
    _fields_ = [("source_to_axis", ctypes.c_double), ("source_to_detector", ctypes.c_double),
                ("pixel_width", ctypes.c_double), ("pixel_height", ctypes.c_double),
                ("det_width", ctypes.c_int32), ("det_height", ctypes.c_int32), ("nviews", ctypes.c_int32),
                ("angle_coverage", ctypes.c_double), ("recon_x", ctypes.c_int32), ("recon_y", ctypes.c_int32),
                ("recon_z", ctypes.c_int32), ("arc", ctypes.c_int32)]


class CtgbFanSlice(ctypes.Structure):
    """Mirror of ``ctgb_fan_slice`` (include/ctgb.h)."""
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("x0", ctypes.c_float), ("dx", ctypes.c_float),
                ("y0", ctypes.c_float), ("dy", ctypes.c_float), ("R", ctypes.c_float), ("D", ctypes.c_float),
                ("g0", ctypes.c_float), ("dg", ctypes.c_float), ("nch", ctypes.c_int32), ("nviews", ctypes.c_int32),
                ("theta0", ctypes.c_float), ("dtheta", ctypes.c_float), ("arc", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("sino_offset", ctypes.c_int64), ("image_offset", ctypes.c_int64)]


class CtgbFwdJob(ctypes.Structure):
    """Mirror of ``ctgb_fwd_job`` (include/ctgb.h): one scan of a batched forward launch."""
    _fields_ = [("params", ctypes.POINTER(CtgbParams)), ("table", ctypes.c_void_p), ("vol", ctypes.c_void_p),
                ("vol_xzy", ctypes.c_void_p), ("out", ctypes.c_void_p), ("view0", ctypes.c_int32),
                ("nviews", ctypes.c_int32), ("epilogue", ctypes.c_int32), ("eps", ctypes.c_float),
                ("p0", ctypes.c_void_p), ("a1", ctypes.c_void_p)]


class CtgbBpJob(ctypes.Structure):
    """Mirror of ``ctgb_bp_job`` (include/ctgb.h): one scan of a batched backprojection launch."""
    _fields_ = [("params", ctypes.POINTER(CtgbParams)), ("table", ctypes.c_void_p), ("proj", ctypes.c_void_p),
                ("vol", ctypes.c_void_p), ("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_size_t),
                ("view0", ctypes.c_int32), ("nviews", ctypes.c_int32), ("scale", ctypes.c_float),
                ("accumulate", ctypes.c_int32), ("epilogue", ctypes.c_int32), ("coef", ctypes.c_float),
                ("eps", ctypes.c_float), ("x", ctypes.c_void_p), ("n1", ctypes.c_void_p)]


FWD_STORE, FWD_SART_RESIDUAL, FWD_POCS_RESIDUAL, FWD_EM_RATIO = 0, 1, 2, 3
BP_STORE, BP_SART_UPDATE, BP_EM_UPDATE, BP_POCS_UPDATE = 0, 1, 2, 3

# (name, argtypes); every entry point returns int status except the string getters.
_P = ctypes.POINTER(CtgbParams)
_vp, _i32, _f32, _sz = ctypes.c_void_p, ctypes.c_int32, ctypes.c_float, ctypes.c_size_t
SIGNATURES = {
    "ctgb_table_bytes": [_P, ctypes.POINTER(_sz)],
    "ctgb_table_build": [_P, _vp, _sz],
    "ctgb_forward": [_P, _vp, _vp, _vp, _vp, _i32, _i32, _vp],
    "ctgb_forward_static": [_P, _vp, _vp, _vp, _i32, _i32, _vp],
    "ctgb_transpose_xy": [_vp, _vp, _i32, _i32, _i32, _vp],
    "ctgb_backproject_fdk": [_P, _vp, _vp, _vp, _i32, _i32, _f32, _i32, _vp],
    "ctgb_backproject_fdk_orbit_size": [_P, ctypes.POINTER(_i32)],
    "ctgb_backproject_fdk_orbits": [_P, _vp, _vp, _vp, _i32, _i32, _f32, _i32, _vp],
    "ctgb_backproject_matched": [_P, _vp, _vp, _vp, _i32, _i32, _f32, _i32, _vp],
    "ctgb_backproject_fdk_workspace_bytes": [_P, _i32, ctypes.POINTER(_sz)],
    "ctgb_backproject_fdk_ws": [_P, _vp, _vp, _vp, _i32, _i32, _f32, _i32, _vp, _sz, _vp],
    "ctgb_backproject_matched_ws": [_P, _vp, _vp, _vp, _i32, _i32, _f32, _i32, _vp, _sz, _vp],
    "ctgb_integrate_projections": [_P, _vp, _i32, _vp, _sz, _vp],
    "ctgb_forward_launches": [_P, _i32, _i32, ctypes.POINTER(_i32)],
    "ctgb_forward_tile_rows": [_P, ctypes.POINTER(_i32)],
    "ctgb_ray_forward": [_P, _vp, _vp, _vp, _i32, _i32, _vp],
    "ctgb_ray_backproject": [_P, _vp, _vp, _vp, _i32, _i32, _f32, _i32, _vp],
    "ctgb_unet_conv3d": [_vp, _i32, _vp, _i32, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp],
    "ctgb_unet_input": [_vp, _vp, _vp, _i32, ctypes.c_int64, _vp],
    "ctgb_unet_first": [_vp, _vp, _vp, _i32, _vp, _vp, _i32, _i32, _i32, _i32, _vp],
    "ctgb_unet_pool2": [_vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp],
    "ctgb_unet_up2": [_vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp],
    "ctgb_unet_relu_grad": [_vp, _i32, _i32, _vp, _vp, ctypes.c_int64, _i32, _vp],
    "ctgb_unet_pool2_grad": [_vp, _vp, _i32, _i32, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp],
    "ctgb_unet_up2_grad": [_vp, _i32, _i32, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp],
    "ctgb_unet_head": [_vp, _vp, _vp, _vp, _vp, _i32, ctypes.c_int64, _vp],
    "ctgb_unet_head_grad_blocks": [ctypes.c_int64, ctypes.POINTER(_i32)],
    "ctgb_unet_head_grad": [_vp, _vp, _vp, _vp, _vp, _vp, _i32, ctypes.c_int64, _vp],
    "ctgb_unet_wgrad_chunks": [_i32, _i32, _i32, _i32, ctypes.POINTER(_i32)],
    "ctgb_unet_wgrad": [_vp, _i32, _vp, _i32, _vp, _i32, _i32, _i32, _i32, _vp],
    "ctgb_unet_colsum": [_vp, _i32, ctypes.c_int64, _vp, _i32, _vp],
    "ctgb_backproject_fdk_integrated": [_P, _vp, _vp, _vp, _i32, _i32, _f32, _i32, _vp],
    "ctgb_filter_bytes": [_P, ctypes.POINTER(_sz)],
    "ctgb_filter_build": [_P, _i32, ctypes.c_double, _vp, _sz],
    "ctgb_fdk_filter": [_P, _vp, _vp, _i32, _vp],
    "ctgb_device_status": [ctypes.POINTER(_i32), _i32],
    "ctgb_selftest_bounded_wait": [_i32, _vp],
    "ctgb_partials_count": [ctypes.c_int64, ctypes.POINTER(_i32)],
    "ctgb_sart_residual": [_vp, _vp, _vp, _f32, _vp, ctypes.c_int64, _vp],
    "ctgb_sart_update": [_vp, _vp, _vp, _f32, _f32, _vp, ctypes.c_int64, _vp],
    "ctgb_em_ratio": [_vp, _vp, _f32, _vp, ctypes.c_int64, _vp],
    "ctgb_em_update": [_vp, _vp, _vp, _vp, ctypes.c_int64, _vp],
    "ctgb_pocs_residual": [_vp, _vp, _vp, _f32, _vp, ctypes.c_int64, _vp],
    "ctgb_pocs_update": [_vp, _vp, _vp, _f32, _f32, _vp, ctypes.c_int64, _vp],
    "ctgb_tv_step": [_vp, _vp, _i32, _i32, _i32, _f32, _f32, _vp, _vp],
    "ctgb_sqdist": [_vp, _vp, ctypes.c_int64, _vp, _vp, _vp],
    "ctgb_conebeam_table_bytes": [ctypes.POINTER(CtgbConeBeamParams), ctypes.POINTER(_sz)],
    "ctgb_conebeam_table_build": [ctypes.POINTER(CtgbConeBeamParams), _vp, _sz],
    "ctgb_conebeam_backproject": [ctypes.POINTER(CtgbConeBeamParams), _vp, _vp, _vp, _i32, _i32, _i32, _vp],
    "ctgb_standalone_filter_bytes": [ctypes.POINTER(CtgbConeBeamParams), ctypes.POINTER(_sz)],
    "ctgb_standalone_filter_build": [ctypes.POINTER(CtgbConeBeamParams), _i32, _i32, ctypes.c_double, _vp, _sz],
    "ctgb_filter_apply": [_vp, _i32, _vp, ctypes.c_int64, _vp],
    "ctgb_filter_zpl": [_vp, ctypes.POINTER(_i32)],
    "ctgb_fan_batch_bytes": [ctypes.POINTER(CtgbFanSlice), _i32, _i32, _i32, ctypes.POINTER(_sz)],
    "ctgb_fan_batch_build": [ctypes.POINTER(CtgbFanSlice), _i32, _i32, _i32, _vp, _sz],
    "ctgb_fan_backproject": [_vp, _i32, _vp, _vp, _i32, _i32, _i32, _i32, _vp],
    "ctgb_batch_forward_plan_bytes": [ctypes.POINTER(CtgbFwdJob), _i32, ctypes.POINTER(_sz)],
    "ctgb_batch_forward_plan": [ctypes.POINTER(CtgbFwdJob), _i32, _vp, _sz],
    "ctgb_batch_forward": [_vp, _vp, _i32, _vp],
    "ctgb_batch_backproject_plan_bytes": [ctypes.POINTER(CtgbBpJob), _i32, ctypes.POINTER(_sz)],
    "ctgb_batch_backproject_plan": [ctypes.POINTER(CtgbBpJob), _i32, _i32, _vp, _sz],
    "ctgb_batch_backproject": [_vp, _vp, _i32, _vp],
}
STRING_FUNCS = ("ctgb_last_error", "ctgb_version")

_lib = None


class CtgbError(RuntimeError):
    pass


def load():
    """Load libctgb.so (building it first if this checkout has not yet)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    for name in STRING_FUNCS:
        fn = getattr(lib, name)
        fn.argtypes = []
        fn.restype = ctypes.c_char_p
    _lib = lib
    return lib


def call(name, *args):
    """Call an entry point; raise ValueError/CtgbError on a non-zero status."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != CTGB_OK:
        msg = lib.ctgb_last_error().decode()
        if st in (-1, -3):
            raise ValueError("%s: %s" % (name, msg))
        raise CtgbError("%s failed (%d): %s" % (name, st, msg))
    return st
