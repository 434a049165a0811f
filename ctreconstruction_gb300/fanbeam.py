"""Batched 2-D fan-beam filtered backprojection with tile autotuning.

A batch holds many slices — each its own image grid, scan geometry and
sinogram — and reconstructs all of them with one filtering pass per
filter geometry and one persistent backprojection launch over a work list of
(slice, tile) items (``ctgb_fan_backproject``).  The tile shape of that
launch is chosen by ``TileAutotuner``: the first batch of a given shape
signature times every candidate tile on the device (CUDA events) and caches
the fastest, so later batches of the same signature reuse it.

Per-slice semantics follow python/FanBeam.py:82-138 (equispaced "line"
detector) and matlab/FanBeamReconArc.m:20-47 (equiangular "arc" detector);
see ``fan_slice`` for the geometry of one slice.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from .projector import _ptr, _stream

TILE_CANDIDATES = ((16, 16), (32, 8), (32, 16), (64, 4), (8, 32), (32, 32))


def fan_slice(nx, ny, half_x, half_y, geom, arc=False, theta0=0.0):
    """Descriptor of one slice.

    nx, ny: image size; the pixel centres span [-half_x, half_x] x
    [-half_y, half_y] (FanBeam.py: linspace(-fov/2, fov/2, n)).  geom is a
    CtgbConeBeamParams-like object with source_to_axis, source_to_detector,
    pixel_width (channel pitch on the detector), det_width (channels),
    nviews and angle_coverage (radians)."""
    s = _lib.CtgbFanSlice()
    s.nx, s.ny = int(nx), int(ny)
    s.dx = 2 * half_x / (nx - 1) if nx > 1 else 0.0
    s.dy = 2 * half_y / (ny - 1) if ny > 1 else 0.0
    s.x0, s.y0 = -half_x, -half_y
    R = float(geom.source_to_axis)
    sdd = float(geom.source_to_detector)
    s.R = R
    s.D = sdd - R
    n = int(geom.det_width)
    if arc:
        dg = float(geom.pixel_width) / sdd             # channel angle
    else:
        dg = float(geom.pixel_width) * R / sdd          # iso-scaled channel pitch (FanBeam.py:113-114)
    s.g0 = -(n - 1) / 2.0 * dg
    s.dg = dg
    s.nch = n
    s.nviews = int(geom.nviews)
    s.theta0 = float(theta0)
    s.dtheta = float(geom.angle_coverage) / s.nviews
    s.arc = 1 if arc else 0
    return s


def slice_from_grid(nx, ny, pixel, geom, arc=False):
    """A slice whose pixel centres sit on a regular grid of the given pitch,
    centred on the rotation axis (the batched benchmark's 0.8 mm grids)."""
    return fan_slice(nx, ny, (nx - 1) / 2.0 * pixel, (ny - 1) / 2.0 * pixel, geom, arc)


class TileAutotuner:
    """Per-signature cache of the fastest backprojection tile (measured)."""

    def __init__(self, candidates=TILE_CANDIDATES, reps=2):
        self.candidates = candidates
        self.reps = reps
        self.cache = {}
        self.last_timings = {}

    def best(self, key, run):
        if key in self.cache:
            return self.cache[key]
        timings = {}
        for tile in self.candidates:
            run(tile)                     # warm (and validate) once
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(self.reps):
                run(tile)
            b.record()
            b.synchronize()
            timings[tile] = a.elapsed_time(b) / self.reps
        best = min(timings, key=timings.get)
        self.cache[key] = best
        self.last_timings[key] = timings
        return best


AUTOTUNER = TileAutotuner()


class FanBatch:
    def __init__(self, slices, device=None, filter_type='hann', cutoff=0.3, autotuner=AUTOTUNER, tile=None,
                 arc_kernel='reference'):
        """arc_kernel: 'reference' filters arc-detector slices with
        matlab/FilterArc.m's kernel; 'balanced' with the Kak & Slaney
        equiangular kernel (quantitative reconstructions)."""
        if arc_kernel not in ('reference', 'balanced'):
            raise ValueError("arc_kernel must be 'reference' or 'balanced'")
        self.arc_kernel = arc_kernel
        self.slices = list(slices)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.filter_type = filter_type
        self.cutoff = cutoff
        self.autotuner = autotuner
        self.fixed_tile = tile
        # sinogram / image offsets: slices packed back to back
        so = io = 0
        for s in self.slices:
            s.sino_offset, s.image_offset = so, io
            so += s.nviews * s.nch
            io += s.nx * s.ny
        self.sino_floats, self.image_floats = so, io
        self.max_views = max(s.nviews for s in self.slices)
        self._tables = {}
        self._batches = {}
        props = torch.cuda.get_device_properties(self.device)
        self.sms = props.multi_processor_count

    # -- filtering ---------------------------------------------------------------
    def _filter(self, s):
        key = (s.arc, s.nch, round(s.R, 6), round(s.R + s.D, 6), round(s.dg, 12))
        if key not in self._tables:
            c = _lib.CtgbConeBeamParams()
            c.source_to_axis = s.R
            c.source_to_detector = s.R + s.D
            # pixel_width is the detector pitch: undo fan_slice's scaling
            c.pixel_width = s.dg * (s.R + s.D) if s.arc else s.dg * (s.R + s.D) / s.R
            c.pixel_height = c.pixel_width
            c.det_width, c.det_height, c.nviews = s.nch, 1, s.nviews
            c.angle_coverage = s.dtheta * s.nviews
            c.recon_x = c.recon_y = c.recon_z = 1
            n = ctypes.c_size_t(0)
            _lib.call("ctgb_standalone_filter_bytes", ctypes.byref(c), ctypes.byref(n))
            host = np.zeros(n.value // 4, dtype=np.float32)
            variant = (3 if self.arc_kernel == 'balanced' else 2) if s.arc else 1
            _lib.call("ctgb_standalone_filter_build", ctypes.byref(c), variant,
                      _lib.FILTER_TYPES[self.filter_type], float(self.cutoff), host.ctypes.data_as(ctypes.c_void_p),
                      n.value)
            zpl = ctypes.c_int32(0)
            _lib.call("ctgb_filter_zpl", host.ctypes.data_as(ctypes.c_void_p), ctypes.byref(zpl))
            self._tables[key] = (torch.from_numpy(host).to(self.device), zpl.value)
        return self._tables[key]

    def filter(self, sino):
        """Filter the packed sinograms in place, one call per run of slices that
        share a filter geometry."""
        i = 0
        n = len(self.slices)
        while i < n:
            table, zpl = self._filter(self.slices[i])
            j = i + 1
            while j < n and self._filter(self.slices[j])[0] is table:
                j += 1
            a = self.slices[i].sino_offset
            rows = sum(self.slices[k].nviews for k in range(i, j))
            _lib.call("ctgb_filter_apply", _ptr(table), zpl, ctypes.c_void_p(sino.data_ptr() + 4 * a), rows,
                      _stream())
            i = j
        return sino

    # -- backprojection ------------------------------------------------------------
    def _batch(self, tile):
        if tile not in self._batches:
            arr = (_lib.CtgbFanSlice * len(self.slices))(*self.slices)
            n = ctypes.c_size_t(0)
            _lib.call("ctgb_fan_batch_bytes", arr, len(self.slices), tile[0], tile[1], ctypes.byref(n))
            host = np.zeros((n.value + 3) // 4, dtype=np.int32)
            _lib.call("ctgb_fan_batch_build", arr, len(self.slices), tile[0], tile[1],
                      host.ctypes.data_as(ctypes.c_void_p), n.value)
            self._batches[tile] = torch.from_numpy(host).to(self.device)
        return self._batches[tile]

    def signature(self):
        return tuple(sorted({(s.nx, s.ny, s.nviews, s.nch, s.arc) for s in self.slices}))

    def backproject(self, sino, images=None, tile=None):
        if images is None:
            images = torch.empty(self.image_floats, dtype=torch.float32, device=self.device)

        def run(t):
            batch = self._batch(t)
            blocks = self.sms * max(1, 2048 // (t[0] * t[1]))
            _lib.call("ctgb_fan_backproject", _ptr(batch), self.max_views, _ptr(sino), _ptr(images), t[0], t[1],
                      blocks, 0, _stream())

        t = tile or self.fixed_tile or self.autotuner.best(self.signature(), run)
        run(t)
        self.tile = t
        return images

    def pack(self, sinos):
        flat = torch.empty(self.sino_floats, dtype=torch.float32, device=self.device)
        for s, q in zip(self.slices, sinos):
            flat[s.sino_offset:s.sino_offset + s.nviews * s.nch].copy_(q.reshape(-1))
        return flat

    def unpack(self, images):
        return [images[s.image_offset:s.image_offset + s.nx * s.ny].view(s.ny, s.nx) for s in self.slices]

    def reconstruct(self, sinos):
        """sinos: one [nviews, nch] tensor per slice.  Returns one [ny, nx]
        image per slice."""
        flat = self.pack(sinos)
        self.filter(flat)
        return self.unpack(self.backproject(flat))
