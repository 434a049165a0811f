"""Scan geometry: the reference's ``params`` dict as a validated dataclass.

Keys and meaning follow ``Reconstruction.__init__``
(python/Reconstruction_numba.py:57-90, python/Reconstruction_pycuda.py:64-99).
Differences from the reference, all additive:

* missing keys get the reference's own default values
  (Reconstruction_numba.py:58-62) instead of raising ``KeyError``;
* the old key ``Origin`` (used by SART.py/EM.py/ASD_POCS.py) is accepted as
  ``RotationOrigin``;
* ``flavour`` selects the numba (default) or pycuda conventions, which differ
  in forward-plane centre (PhantomCenter vs ReconCenter), DetectorOffset and the
  weight clamp.
"""
from dataclasses import dataclass, field
import math

import numpy as np

from . import _lib

_DEFAULTS = {'SourceInit': [0.0, 0.0, 0.0], 'DetectorInit': [0.0, 0.0, 0.0], 'StartAngle': 0.0, 'EndAngle': 0.0,
             'NumberOfDetectorPixels': [0, 0], 'DetectorPixelSize': [0.0, 0.0], 'NumberOfViews': 0,
             'ImagePixelSpacing': [0.0, 0.0, 0.0], 'NumberOfImage': [0, 0, 0], 'PhantomCenter': [0.0, 0.0, 0.0],
             'RotationOrigin': [0.0, 0.0, 0.0], 'ReconCenter': [0.0, 0.0, 0.0], 'Method': 'Distance',
             'FilterType': 'ram-lak', 'cutoff': 1.0, 'GPU': 1, 'DetectorShape': 'Flat', 'Pitch': 0.0,
             'DetectorOffset': [0.0, 0.0]}


def _vec(v, n, key):
    a = [float(x) for x in v]
    if len(a) != n:
        raise ValueError("%s must have %d entries, got %r" % (key, n, v))
    return a


@dataclass
class ReconstructionParams:
    SourceInit: list
    DetectorInit: list
    StartAngle: float
    EndAngle: float
    NumberOfDetectorPixels: list
    DetectorPixelSize: list
    NumberOfViews: int
    ImagePixelSpacing: list
    NumberOfImage: list
    PhantomCenter: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    RotationOrigin: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    ReconCenter: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    Method: str = 'Distance'
    FilterType: str = 'ram-lak'
    cutoff: float = 1.0
    GPU: int = 1
    DetectorShape: str = 'Flat'
    Pitch: float = 0.0
    DetectorOffset: list = field(default_factory=lambda: [0.0, 0.0])
    flavour: str = 'numba'

    @classmethod
    def from_dict(cls, params, flavour=None):
        if isinstance(params, ReconstructionParams):
            return params
        d = dict(_DEFAULTS)
        d.update(params)
        if 'RotationOrigin' not in params and 'Origin' in params:
            d['RotationOrigin'] = params['Origin']
        d.pop('Origin', None)
        fl = flavour or params.get('flavour') or ('pycuda' if 'DetectorOffset' in params else 'numba')
        d.pop('flavour', None)
        known = set(_DEFAULTS)
        extra = sorted(set(d) - known)
        if extra:
            raise ValueError("unknown params keys: %s" % ", ".join(extra))
        p = cls(**d, flavour=fl)
        p.validate()
        return p

    def validate(self):
        self.SourceInit = _vec(self.SourceInit, 3, 'SourceInit')
        self.DetectorInit = _vec(self.DetectorInit, 3, 'DetectorInit')
        self.PhantomCenter = _vec(self.PhantomCenter, 3, 'PhantomCenter')
        self.RotationOrigin = _vec(self.RotationOrigin, 3, 'RotationOrigin')
        self.ReconCenter = _vec(self.ReconCenter, 3, 'ReconCenter')
        self.DetectorOffset = _vec(self.DetectorOffset, 2, 'DetectorOffset')
        self.ImagePixelSpacing = _vec(self.ImagePixelSpacing, 3, 'ImagePixelSpacing')
        self.DetectorPixelSize = _vec(self.DetectorPixelSize, 2, 'DetectorPixelSize')
        self.NumberOfImage = [int(v) for v in self.NumberOfImage]
        self.NumberOfDetectorPixels = [int(v) for v in self.NumberOfDetectorPixels]
        self.NumberOfViews = int(self.NumberOfViews)
        if len(self.NumberOfImage) != 3 or min(self.NumberOfImage) < 1:
            raise ValueError("NumberOfImage must be three positive sizes")
        if len(self.NumberOfDetectorPixels) != 2 or min(self.NumberOfDetectorPixels) < 1:
            raise ValueError("NumberOfDetectorPixels must be two positive sizes")
        if self.NumberOfViews < 1:
            raise ValueError("NumberOfViews must be positive")
        if min(self.ImagePixelSpacing) <= 0 or min(self.DetectorPixelSize) <= 0:
            raise ValueError("pixel and voxel spacings must be positive")
        if self.DetectorShape not in ('Flat', 'Curved'):
            raise ValueError("Detector shape is not supported: %r" % self.DetectorShape)
        if self.Method not in ('Distance', 'Ray'):
            raise ValueError("Method must be 'Distance' or 'Ray', got %r" % self.Method)
        if self.flavour not in ('numba', 'pycuda'):
            raise ValueError("flavour must be 'numba' or 'pycuda'")
        if self.sdd <= 0:
            raise ValueError("SourceInit and DetectorInit coincide")
        return self

    # derived quantities (Reconstruction_numba.py:75-80)
    @property
    def sad(self):
        return math.sqrt(sum((a - b) ** 2 for a, b in zip(self.SourceInit, self.RotationOrigin)))

    @property
    def sdd(self):
        return math.sqrt(sum((a - b) ** 2 for a, b in zip(self.SourceInit, self.DetectorInit)))

    @property
    def nu(self):
        return self.NumberOfDetectorPixels[0]

    @property
    def nv(self):
        return self.NumberOfDetectorPixels[1]

    @property
    def volume_shape(self):
        nx, ny, nz = self.NumberOfImage
        return (nz, ny, nx)

    @property
    def proj_shape(self):
        return (self.NumberOfViews, self.nv, self.nu)

    @property
    def angles(self):
        return np.linspace(self.StartAngle, self.EndAngle, self.NumberOfViews + 1)[:-1]

    @property
    def dtheta(self):
        a = self.angles
        return float(a[1] - a[0]) if len(a) > 1 else 0.0

    def to_ctgb(self):
        c = _lib.CtgbParams()
        c.nu, c.nv = self.NumberOfDetectorPixels
        c.du, c.dv = self.DetectorPixelSize
        c.nx, c.ny, c.nz = self.NumberOfImage
        c.dx, c.dy, c.dz = self.ImagePixelSpacing
        c.nviews = self.NumberOfViews
        c.start_angle, c.end_angle = float(self.StartAngle), float(self.EndAngle)
        c.source_init[:] = self.SourceInit
        c.detector_init[:] = self.DetectorInit
        c.rotation_origin[:] = self.RotationOrigin
        c.phantom_center[:] = self.PhantomCenter
        c.recon_center[:] = self.ReconCenter
        c.detector_offset[:] = self.DetectorOffset
        c.pitch = float(self.Pitch)
        c.curved = 1 if self.DetectorShape == 'Curved' else 0
        c.flavour = _lib.FLAVOUR_PYCUDA if self.flavour == 'pycuda' else _lib.FLAVOUR_NUMBA
        return c

    def as_dict(self):
        d = {k: getattr(self, k) for k in _DEFAULTS}
        return d
