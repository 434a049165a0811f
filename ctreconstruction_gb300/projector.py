"""Device-resident DD projectors over one scan geometry.

``Projector`` owns the geometry table (built once on the host in float64 by
``ctgb_table_build`` and kept in device memory) and calls the C ABI on torch's
current CUDA stream.  Inputs and outputs are float32 CUDA tensors in the
reference's layouts: volume ``[nz, ny, nx]``, projections ``[nviews, nv, nu]``.
There is no CPU path: a CPU tensor or a missing library raises.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .geometry import ReconstructionParams


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class Projector:
    def __init__(self, params, device=None, flavour=None):
        self.params = ReconstructionParams.from_dict(params, flavour)
        if not torch.cuda.is_available():
            raise RuntimeError("ctreconstruction_gb300 needs a CUDA device (no CPU fallback)")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.c = self.params.to_ctgb()
        n = ctypes.c_size_t(0)
        _lib.call("ctgb_table_bytes", ctypes.byref(self.c), ctypes.byref(n))
        host = np.zeros(n.value // 4, dtype=np.float32)
        _lib.call("ctgb_table_build", ctypes.byref(self.c), host.ctypes.data_as(ctypes.c_void_p), n.value)
        self.table = torch.from_numpy(host).to(self.device)
        self._filters = {}
        self._xzy = None
        self._ws = None

    # -- helpers --------------------------------------------------------------
    def _check(self, t, shape, name):
        if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
            raise ValueError("%s must be a CUDA tensor" % name)
        if t.dtype != torch.float32:
            raise ValueError("%s must be float32, got %s" % (name, t.dtype))
        if tuple(t.shape) != tuple(shape):
            raise ValueError("%s has shape %s, expected %s" % (name, tuple(t.shape), tuple(shape)))
        if not t.is_contiguous():
            raise ValueError("%s must be contiguous" % name)

    def _views(self, view0, nviews):
        nv = self.params.NumberOfViews - view0 if nviews is None else nviews
        return int(view0), int(nv)

    @property
    def volume_shape(self):
        return self.params.volume_shape

    def proj_shape(self, nviews=None):
        p = self.params
        return (p.NumberOfViews if nviews is None else nviews, p.nv, p.nu)

    # -- projectors -----------------------------------------------------------
    def forward(self, vol, out=None, view0=0, nviews=None, transposed=None):
        """proj = A vol (distance_forward).  ``transposed``: optional [nz,nx,ny]
        copy of vol; made here (workspace kept between calls) when omitted."""
        view0, nviews = self._views(view0, nviews)
        self._check(vol, self.volume_shape, "vol")
        if out is None:
            out = torch.empty(self.proj_shape(nviews), dtype=torch.float32, device=vol.device)
        self._check(out, self.proj_shape(nviews), "out")
        if transposed is None:
            transposed = self.transpose(vol)
        _lib.call("ctgb_forward", ctypes.byref(self.c), _ptr(self.table), _ptr(vol), _ptr(transposed), _ptr(out),
                  view0, nviews, _stream())
        return out

    def transpose(self, vol, out=None):
        nz, ny, nx = self.volume_shape
        if out is None:
            if self._xzy is None or self._xzy.device != vol.device:
                self._xzy = torch.empty((nz, nx, ny), dtype=torch.float32, device=vol.device)
            out = self._xzy
        _lib.call("ctgb_transpose_xy", _ptr(vol), _ptr(out), nx, ny, nz, _stream())
        return out

    def backproject_fdk(self, proj, out=None, view0=0, nviews=None, scale=None, accumulate=False):
        """vol = scale * sum_v BP_v(proj) with the FDK distance weight
        (distance_backproj); scale defaults to dtheta as in backward()."""
        view0, nviews = self._views(view0, nviews)
        self._check(proj, self.proj_shape(nviews), "proj")
        if out is None:
            out = torch.empty(self.volume_shape, dtype=torch.float32, device=proj.device)
            accumulate = False
        self._check(out, self.volume_shape, "out")
        sc = self.params.dtheta if scale is None else float(scale)
        ws = self._workspace(nviews)
        if ws is None:
            _lib.call("ctgb_backproject_fdk", ctypes.byref(self.c), _ptr(self.table), _ptr(proj), _ptr(out), view0,
                      nviews, sc, int(bool(accumulate)), _stream())
        else:
            _lib.call("ctgb_backproject_fdk_ws", ctypes.byref(self.c), _ptr(self.table), _ptr(proj), _ptr(out),
                      view0, nviews, sc, int(bool(accumulate)), _ptr(ws), ws.numel() * 4, _stream())
        return out

    def orbit_size(self):
        """Rotation-orbit size (4, 2 or 1) the FDK backprojector shares its
        per-view set-up over for a call on every view of this scan."""
        n = ctypes.c_int32(0)
        _lib.call("ctgb_backproject_fdk_orbit_size", ctypes.byref(self.c), ctypes.byref(n))
        return n.value

    def backproject_fdk_orbits(self, proj, out, base0, nbase, scale=None, accumulate=False):
        """backproject_fdk over base views [base0, base0 + nbase) of the
        symmetric orbit (each base view b stands for the views b + k * views /
        orbit_size()); proj holds every view of the scan."""
        self._check(proj, self.proj_shape(), "proj")
        self._check(out, self.volume_shape, "out")
        sc = self.params.dtheta if scale is None else float(scale)
        _lib.call("ctgb_backproject_fdk_orbits", ctypes.byref(self.c), _ptr(self.table), _ptr(proj), _ptr(out),
                  int(base0), int(nbase), sc, int(bool(accumulate)), _stream())
        return out

    def ray_forward(self, vol, out=None, view0=0, nviews=None):
        """Siddon ray sums to every pixel centre (the `Method: 'Ray'` projector)."""
        view0, nviews = self._views(view0, nviews)
        self._check(vol, self.volume_shape, "vol")
        if out is None:
            out = torch.empty(self.proj_shape(nviews), dtype=torch.float32, device=vol.device)
        self._check(out, self.proj_shape(nviews), "out")
        _lib.call("ctgb_ray_forward", ctypes.byref(self.c), _ptr(self.table), _ptr(vol), _ptr(out), view0, nviews,
                  _stream())
        return out

    def ray_backproject(self, proj, out=None, view0=0, nviews=None, scale=1.0, accumulate=False):
        """vol = scale * transpose of ray_forward (exact adjoint up to float
        rounding; atomics make the summation order run-dependent)."""
        view0, nviews = self._views(view0, nviews)
        self._check(proj, self.proj_shape(nviews), "proj")
        if out is None:
            out = torch.empty(self.volume_shape, dtype=torch.float32, device=proj.device)
            accumulate = False
        self._check(out, self.volume_shape, "out")
        _lib.call("ctgb_ray_backproject", ctypes.byref(self.c), _ptr(self.table), _ptr(proj), _ptr(out), view0,
                  nviews, float(scale), int(bool(accumulate)), _stream())
        return out

    def forward_launches(self, view0=0, nviews=None):
        """Kernel launches one forward() call makes over this view range."""
        view0, nviews = self._views(view0, nviews)
        n = ctypes.c_int32(0)
        _lib.call("ctgb_forward_launches", ctypes.byref(self.c), view0, nviews, ctypes.byref(n))
        return n.value

    def forward_tile_rows(self):
        """Detector rows per tile of the forward kernel for this geometry (32,
        or 16 where a detector row spans more than 1.3 voxel rows)."""
        n = ctypes.c_int32(0)
        _lib.call("ctgb_forward_tile_rows", ctypes.byref(self.c), ctypes.byref(n))
        return n.value

    def integrate(self, proj, nviews=None, out=None):
        """Integrated projections of the first nviews views of proj (running
        sum along v, value) as the float2 workspace the FDK backprojector
        reads; returns the workspace tensor (flat float32)."""
        nviews = self.params.NumberOfViews if nviews is None else int(nviews)
        self._check(proj, self.proj_shape(nviews), "proj")
        n = ctypes.c_size_t(0)
        _lib.call("ctgb_backproject_fdk_workspace_bytes", ctypes.byref(self.c), nviews, ctypes.byref(n))
        if out is None or out.numel() * 4 < n.value:
            out = torch.empty((n.value + 3) // 4, dtype=torch.float32, device=proj.device)
        _lib.call("ctgb_integrate_projections", ctypes.byref(self.c), _ptr(proj), nviews, _ptr(out), out.numel() * 4,
                  _stream())
        return out

    def backproject_fdk_integrated(self, integrated, out=None, view0=0, nviews=None, scale=None, accumulate=False):
        """backproject_fdk from projections already integrated by integrate()."""
        view0, nviews = self._views(view0, nviews)
        if out is None:
            out = torch.empty(self.volume_shape, dtype=torch.float32, device=integrated.device)
            accumulate = False
        self._check(out, self.volume_shape, "out")
        n = ctypes.c_size_t(0)
        _lib.call("ctgb_backproject_fdk_workspace_bytes", ctypes.byref(self.c), nviews, ctypes.byref(n))
        if integrated.numel() * 4 < n.value or integrated.dtype != torch.float32 or not integrated.is_cuda:
            raise ValueError("integrated: need a CUDA float32 tensor of at least %d bytes" % n.value)
        sc = self.params.dtheta if scale is None else float(scale)
        _lib.call("ctgb_backproject_fdk_integrated", ctypes.byref(self.c), _ptr(self.table), _ptr(integrated),
                  _ptr(out), view0, nviews, sc, int(bool(accumulate)), _stream())
        return out

    # Integrated-projection workspace of the FDK backprojector: all views when
    # that fits in WORKSPACE_CAP bytes, else chunks of views.
    WORKSPACE_CAP = 6 << 30

    def _workspace(self, nviews):
        if nviews == 0 or self.params.nu < 4:
            return None
        n = ctypes.c_size_t(0)
        _lib.call("ctgb_backproject_fdk_workspace_bytes", ctypes.byref(self.c), 1, ctypes.byref(n))
        per_view = n.value
        want = min(nviews * per_view, max(per_view, self.WORKSPACE_CAP // per_view * per_view))
        if self._ws is None or self._ws.numel() * 4 < want:
            self._ws = torch.empty((want + 3) // 4, dtype=torch.float32, device=self.device)
        return self._ws

    def backproject_matched(self, proj, out=None, view0=0, nviews=None, scale=1.0, accumulate=False):
        """vol = scale * A^T proj (exact adjoint of forward)."""
        view0, nviews = self._views(view0, nviews)
        self._check(proj, self.proj_shape(nviews), "proj")
        if out is None:
            out = torch.empty(self.volume_shape, dtype=torch.float32, device=proj.device)
            accumulate = False
        self._check(out, self.volume_shape, "out")
        ws = self._workspace(nviews)
        if ws is None:
            _lib.call("ctgb_backproject_matched", ctypes.byref(self.c), _ptr(self.table), _ptr(proj), _ptr(out),
                      view0, nviews, float(scale), int(bool(accumulate)), _stream())
        else:
            _lib.call("ctgb_backproject_matched_ws", ctypes.byref(self.c), _ptr(self.table), _ptr(proj), _ptr(out),
                      view0, nviews, float(scale), int(bool(accumulate)), _ptr(ws), ws.numel() * 4, _stream())
        return out

    # -- FDK filtering --------------------------------------------------------
    def filter_table(self, filter_type=None, cutoff=None):
        ft = self.params.FilterType if filter_type is None else filter_type
        co = float(self.params.cutoff if cutoff is None else cutoff)
        if ft not in _lib.FILTER_TYPES:
            raise ValueError("unknown FilterType %r" % ft)
        if not co > 0:
            raise ValueError("cutoff must be positive, got %r" % co)
        if co > 1:
            # Reconstruction.Filter (Reconstruction_numba.py:196-200) reports and carries on.
            print("Cutoff have to be pose between 0 and 0.5")
        key = (ft, co)
        if key not in self._filters:
            n = ctypes.c_size_t(0)
            _lib.call("ctgb_filter_bytes", ctypes.byref(self.c), ctypes.byref(n))
            host = np.zeros(n.value // 4, dtype=np.float32)
            _lib.call("ctgb_filter_build", ctypes.byref(self.c), _lib.FILTER_TYPES[ft], co,
                      host.ctypes.data_as(ctypes.c_void_p), n.value)
            self._filters[key] = torch.from_numpy(host).to(self.device)
        return self._filters[key]

    def filter(self, proj, filter_type=None, cutoff=None):
        """In-place FDK cosine weight + ramp filter (Filtering)."""
        if not isinstance(proj, torch.Tensor) or proj.dim() != 3 or tuple(proj.shape[1:]) != self.proj_shape()[1:]:
            raise ValueError("proj must be a CUDA tensor [nviews, nv, nu]")
        self._check(proj, proj.shape, "proj")
        f = self.filter_table(filter_type, cutoff)
        _lib.call("ctgb_fdk_filter", ctypes.byref(self.c), _ptr(f), _ptr(proj), proj.shape[0], _stream())
        return proj
