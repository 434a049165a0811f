"""The standalone FDK / fan-beam reconstructors of the reference, on the GPU.

* ``ConeBeam``: python/ConeBeam.py and python/ConeBeamGPU.py — parameters from
  a "key: value" text file, projections loaded from raw files, voxel-driven
  FDK with bilinear detector interpolation.
* ``FanBeam``: python/FanBeam.py — per-slice 2-D fan-beam FBP on an
  equispaced ("line") detector; ``detector='arc'`` gives the equiangular
  variant of matlab/FanBeamReconArc.m.

Layouts follow the reference: ``ConeBeam.proj`` is [DetectorHeight,
DetectorWidth, NumberOfViews] (views last) and ``recon`` is the raw
[Z][Y][X]-ordered volume viewed as [ReconX, ReconY, ReconZ], as
ConeBeamGPU.py:315-317 does; ``FanBeam.sino`` is [NumberOfViews,
DetectorWidth, DetectorHeight] and ``recon`` is [ReconX, ReconY,
DetectorHeight].  Filtering, interpolation and accumulation run in libctgb.
"""
import ctypes
import glob
import math
import os

import numpy as np
import torch

from . import _lib
from .projector import _ptr, _stream

_CB_KEYS = ('SourceToDetector', 'SourceToAxis', 'DataPath', 'precision', 'AngleCoverage', 'ReconX', 'ReconY',
            'ReconZ', 'DetectorPixelHeight', 'DetectorPixelWidth', 'DetectorWidth', 'DetectorHeight',
            'NumberOfViews', 'fov', 'fovz', 'Mode')
_FB_KEYS = ('SourceToDetector', 'SourceToAxis', 'DataPath', 'precision', 'AngleCoverage', 'ReconX', 'ReconY',
            'DetectorPixelWidth', 'DetectorWidth', 'DetectorHeight', 'NumberOfViews', 'fov', 'fovz')


class ErrorDescription(Exception):
    _MSG = {1: 'Unknown variables', 2: 'Unknown data precision',
            3: 'Number of file is different from number of projection data required',
            4: 'Cutoff have to be pose between 0 and 0.5', 5: 'Smooth have to be pose between 0 and 1',
            6: 'Recon volume is too big for GPU'}

    def __init__(self, value):
        self.msg = self._MSG.get(value, 'Unknown error')
        super().__init__(self.msg)

    def __str__(self):
        return self.msg


def read_params_txt(filename, keys=_CB_KEYS, volume_dims=3):
    """ConeBeam.__init__ / FanBeam.__init__ parser (ConeBeam.py:57-84):
    'key: value' lines; AngleCoverage in degrees (stored in radians);
    ReconVolume 'X*Y*Z'; DataPath and precision kept as strings, the rest as
    floats.  An unknown key stops the parse and prints 'Unknown variables'."""
    params = {k: 0 for k in keys}
    params['DataPath'] = ''
    params['precision'] = ''
    with open(filename) as f:
        for line in f:
            if not line.strip():
                continue
            key = line.split(':')[0].strip()
            if key not in params and key != 'ReconVolume':
                print(ErrorDescription(1))
                break
            value = line.split(':', 1)[1].strip()
            if key == 'AngleCoverage':
                params[key] = float(value) * np.pi / 180.0
            elif key == 'ReconVolume':
                v = value.split('*')
                params['ReconX'], params['ReconY'] = int(v[0]), int(v[1])
                if volume_dims == 3:
                    params['ReconZ'] = int(v[2])
            elif key in ('DataPath', 'precision'):
                params[key] = value
            else:
                params[key] = float(value)
    return params


_PRECISION = {'float32': np.float32, 'float64': np.float64, 'int32': np.int32, 'int64': np.int64}


def _load_stack(path, n, shape, precision):
    """Sorted raw files of one projection/sinogram each (ConeBeam.LoadData)."""
    if precision not in _PRECISION:
        raise ErrorDescription(2)
    files = sorted(glob.glob(path + '*.dat'))
    if len(files) != n:
        raise ErrorDescription(3)
    return [np.fromfile(f, dtype=_PRECISION[precision]).reshape(shape) for f in files]


def _cparams(p, arc=False, fan=False):
    c = _lib.CtgbConeBeamParams()
    c.source_to_axis = float(p['SourceToAxis'])
    c.source_to_detector = float(p['SourceToDetector'])
    c.pixel_width = float(p['DetectorPixelWidth'])
    c.pixel_height = float(p.get('DetectorPixelHeight', 0) or p['DetectorPixelWidth'])
    c.det_width = int(p['DetectorWidth'])
    c.det_height = int(p['DetectorHeight'])
    c.nviews = int(p['NumberOfViews'])
    c.angle_coverage = float(p['AngleCoverage'])
    c.recon_x, c.recon_y = int(p['ReconX']), int(p['ReconY'])
    c.recon_z = int(p['DetectorHeight']) if fan else int(p['ReconZ'])
    c.arc = 1 if arc else 0
    return c


def _filter_table(c, variant, filter_type, cutoff, device):
    n = ctypes.c_size_t(0)
    _lib.call("ctgb_standalone_filter_bytes", ctypes.byref(c), ctypes.byref(n))
    host = np.zeros(n.value // 4, dtype=np.float32)
    _lib.call("ctgb_standalone_filter_build", ctypes.byref(c), variant, _lib.FILTER_TYPES[filter_type], float(cutoff),
              host.ctypes.data_as(ctypes.c_void_p), n.value)
    zpl = ctypes.c_int32(0)
    _lib.call("ctgb_filter_zpl", host.ctypes.data_as(ctypes.c_void_p), ctypes.byref(zpl))
    return torch.from_numpy(host).to(device), zpl.value


class ConeBeam:
    def __init__(self, filename, device=None):
        self.params = read_params_txt(filename, _CB_KEYS, 3)
        p = self.params
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.proj = np.zeros([int(p['DetectorHeight']), int(p['DetectorWidth']), int(p['NumberOfViews'])])
        self.recon = np.zeros([p['ReconX'], p['ReconY'], p['ReconZ']])

    def LoadData(self):
        p = self.params
        ny, nx, ns = int(p['DetectorHeight']), int(p['DetectorWidth']), int(p['NumberOfViews'])
        stack = _load_stack(p['DataPath'], ns, [ny, nx], p['precision'])
        for c, img in enumerate(stack):
            self.proj[:, :, c] = img

    def Reconstruction(self, savefile=None, filter_type='ram-lak', cutoff=0.3):
        """ConeBeamGPU.Reconstruction (:203-321): filter, then voxel-driven
        weighted backprojection of every view; recon [X, Y, Z] view of the
        [Z][Y][X] result, written raw to savefile when given."""
        p = self.params
        c = _cparams(p)
        dev = self.device
        ny, nx, ns = c.det_height, c.det_width, c.nviews
        proj = self.proj if isinstance(self.proj, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(np.moveaxis(np.asarray(self.proj, dtype=np.float32), 2, 0)))
        q = proj.to(dev, dtype=torch.float32).contiguous()
        if q.shape != (ns, ny, nx):
            raise ValueError("projections must be [DetectorHeight, DetectorWidth, NumberOfViews]")
        filt, zpl = _filter_table(c, 0, filter_type, cutoff, dev)
        _lib.call("ctgb_filter_apply", _ptr(filt), zpl, _ptr(q), ns * ny, _stream())
        n = ctypes.c_size_t(0)
        _lib.call("ctgb_conebeam_table_bytes", ctypes.byref(c), ctypes.byref(n))
        host = np.zeros(n.value // 4, dtype=np.float32)
        _lib.call("ctgb_conebeam_table_build", ctypes.byref(c), host.ctypes.data_as(ctypes.c_void_p), n.value)
        table = torch.from_numpy(host).to(dev)
        recon = torch.empty((c.recon_z, c.recon_y, c.recon_x), dtype=torch.float32, device=dev)
        _lib.call("ctgb_conebeam_backproject", ctypes.byref(c), _ptr(table), _ptr(q), _ptr(recon), 0, ns, 0,
                  _stream())
        out = recon.cpu().numpy()
        self.recon = out.reshape([c.recon_x, c.recon_y, c.recon_z])
        if savefile:
            out.tofile(savefile, sep='', format='')
        return recon


class FanBeam:
    def __init__(self, filename, device=None):
        self.params = read_params_txt(filename, _FB_KEYS, 2)
        p = self.params
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        nx, ny, ns = int(p['DetectorWidth']), int(p['DetectorHeight']), int(p['NumberOfViews'])
        self.proj = np.zeros([ny, nx, ns])
        self.sino = np.zeros([ns, nx, ny])
        self.recon = np.zeros([p['ReconX'], p['ReconY'], ny])

    def LoadData(self):
        p = self.params
        ny, nx, ns = int(p['DetectorHeight']), int(p['DetectorWidth']), int(p['NumberOfViews'])
        stack = _load_stack(p['DataPath'], ns, [ny, nx], p['precision'])
        for c, img in enumerate(stack):
            self.proj[:, :, c] = img
            self.sino[c, :, :] = img.T

    def Reconstruction(self, savefile=None, detector='line', filter_type='hann', cutoff=0.3):
        """FanBeam.Reconstruction (:82-138): per slice, cosine-weighted ramp
        filter, then voxel-driven backprojection with 1/U^2 (line) or 1/L^2
        (arc) weights.  recon is [ReconX, ReconY, DetectorHeight]."""
        from .fanbeam import FanBatch, fan_slice
        p = self.params
        arc = detector == 'arc'
        c = _cparams(p, arc=arc, fan=True)
        ns, nx, ny = c.nviews, c.det_width, c.det_height
        sino = self.sino if isinstance(self.sino, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(np.moveaxis(np.asarray(self.sino, dtype=np.float32), 2, 0)))
        sino = sino.to(self.device, dtype=torch.float32).contiguous()    # [slices][views][channels]
        if sino.shape != (ny, ns, nx):
            raise ValueError("sinogram must be [NumberOfViews, DetectorWidth, DetectorHeight]")
        R, D = c.source_to_axis, c.source_to_detector - c.source_to_axis
        fov = 2 * R * math.sin(math.atan(nx * c.pixel_width / 2 / (D + R)))
        slices = [fan_slice(c.recon_x, c.recon_y, fov / 2, fov / 2, c, arc) for _ in range(ny)]
        batch = FanBatch(slices, device=self.device, filter_type=filter_type, cutoff=cutoff)
        images = batch.reconstruct([sino[j] for j in range(ny)])
        vol = torch.stack(images)            # [slices][Y][X]
        out = vol.permute(1, 2, 0).cpu().numpy() if c.recon_x == c.recon_y else \
            np.stack([im.cpu().numpy().reshape(c.recon_x, c.recon_y) for im in images], axis=2)
        self.recon = np.ascontiguousarray(out)
        if savefile:
            self.recon.astype(np.float32).tofile(savefile, sep='', format='')
        return vol
