"""Drop-in ``Reconstruction`` class: the call surface of the reference's
``Reconstruction`` (python/Reconstruction_numba.py:55-1614 and
python/Reconstruction_pycuda.py:62-1513) on top of the GB300 projectors.

``image`` is ``[nz, ny, nx]`` float32 and ``proj`` is ``[nViews, nv, nu]``
float32, as in the reference.  Either may be a NumPy array (results come back
as NumPy, like the reference) or a CUDA tensor (results stay on the device, no
host round trip).  All arithmetic runs in libctgb's CUDA kernels.
"""
import numpy as np
import torch

from .geometry import ReconstructionParams
from .projector import Projector


class ErrorDescription(Exception):
    """Error codes of the reference (Reconstruction_numba.py:36-52)."""
    _MSG = {1: 'Unknown variables', 2: 'Unknown data precision',
            3: 'Number of file is different from number of projection data required',
            4: 'Cutoff have to be pose between 0 and 0.5', 5: 'Smooth have to be pose between 0 and 1'}

    def __init__(self, value):
        self.msg = self._MSG.get(value, 'Unknown error')
        super().__init__(self.msg)

    def __str__(self):
        return self.msg


def _to_device(a, device):
    if isinstance(a, torch.Tensor):
        t = a.to(device=device, dtype=torch.float32, non_blocking=bool(not a.is_cuda and a.is_pinned()))
        return t.contiguous()
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(device, non_blocking=False)


def _on_host(a):
    return not (isinstance(a, torch.Tensor) and a.is_cuda)


class Reconstruction:
    def __init__(self, params, flavour=None, device=None):
        self.p = ReconstructionParams.from_dict(params, flavour)
        self.params = self.p.as_dict()
        p = self.p
        self.nu, self.nv = p.NumberOfDetectorPixels
        self.du, self.dv = p.DetectorPixelSize
        self.nx, self.ny, self.nz = p.NumberOfImage
        self.dx, self.dy, self.dz = p.ImagePixelSpacing
        self.Origin = np.array(p.RotationOrigin)
        self.PhantomCenter = np.array(p.PhantomCenter)
        self.ReconCenter = p.ReconCenter
        self.cutoff = p.cutoff
        self.DetectorShape = p.DetectorShape
        self.P = p.Pitch
        self.Source = np.array(p.SourceInit, dtype=np.float64)
        self.Detector = np.array(p.DetectorInit, dtype=np.float64)
        self.SAD = p.sad
        self.SDD = p.sdd
        self.HelicalTrans = self.P * (self.nv * self.dv) * self.SAD / self.SDD
        self.nView = p.NumberOfViews
        self.sAngle, self.eAngle = p.StartAngle, p.EndAngle
        self.Method = p.Method
        self.FilterType = p.FilterType
        self.DetectorOffset = p.DetectorOffset
        self.GPU = True
        self.projector = Projector(p, device=device)
        self.image = None
        self.proj = None

    # -- raw float32 I/O (Reconstruction_numba.py:92-104) ------------------------
    def LoadProj(self, filename, dtype=np.float32):
        self.proj = np.fromfile(filename, dtype=dtype).reshape([self.nView, self.nv, self.nu])

    def LoadRecon(self, filename, dtype=np.float32):
        self.image = np.fromfile(filename, dtype=dtype).reshape([self.nz, self.ny, self.nx])

    def SaveProj(self, filename):
        _host(self.proj).tofile(filename, sep='', format='')

    def SaveRecon(self, filename):
        _host(self.image).tofile(filename, sep='', format='')

    def FlipProj(self, dir):
        """dir 0 flips each view along v, 1 along u (Reconstruction_numba.py:106-119)."""
        if dir not in (0, 1):
            print(ErrorDescription(4))
            return
        axis = 1 if dir == 0 else 2
        if isinstance(self.proj, torch.Tensor):
            self.proj = torch.flip(self.proj, dims=[axis]).contiguous()
        else:
            self.proj = np.ascontiguousarray(np.flip(self.proj, axis=axis))

    # -- host results ---------------------------------------------------------------
    def _to_host(self, t, src, key):
        """Result of a call whose input was on the host: NumPy in -> NumPy out
        (as the reference); a CPU tensor in -> a pinned CPU tensor out, copied
        asynchronously into a buffer the object reuses for that attribute
        (copy it before the next call to keep it)."""
        if isinstance(src, torch.Tensor):
            cache = self.__dict__.setdefault("_pinned", {})
            out = _pinned_like(cache, key, t)
            out.copy_(t, non_blocking=True)
            torch.cuda.current_stream(t.device).synchronize()
            return out
        return _host(t)

    # -- pipelined host transfers ---------------------------------------------------
    # Pinned host tensors go through the projectors in chunks of views: each
    # chunk's device-to-host (forward) or host-to-device (backward) copy runs
    # on a second stream while the kernels of the neighbouring chunk run, so
    # the copies hide behind the projector instead of adding to it.
    CHUNKS = 8

    def _chunks(self, n):
        k = max(1, min(self.CHUNKS, n))
        step = (n + k - 1) // k
        return [(a, min(step, n - a)) for a in range(0, n, step)]

    def _device_buffer(self, key, shape):
        cache = self.__dict__.setdefault("_dev", {})
        buf = cache.get(key)
        if buf is None or tuple(buf.shape) != tuple(shape):
            buf = torch.empty(shape, dtype=torch.float32, device=self.projector.device)
            cache[key] = buf
        return buf

    def _streams(self):
        dev = self.projector.device
        if self.__dict__.get("_copy_stream") is None:
            self._copy_stream = torch.cuda.Stream(device=dev)
        return torch.cuda.current_stream(dev), self._copy_stream

    def _forward_pinned(self, src):
        P = self.projector
        compute, copy = self._streams()
        if tuple(src.shape) != tuple(P.volume_shape):
            raise ValueError("image must have shape %s, got %s" % (tuple(P.volume_shape), tuple(src.shape)))
        vol = self._device_buffer("vol", P.volume_shape)
        vol.copy_(src, non_blocking=True)
        xzy = P.transpose(vol)
        shape = P.proj_shape()
        dev = self._device_buffer("proj", shape)
        out = _pinned_like(self.__dict__.setdefault("_pinned", {}), "proj", dev)
        for v0, n in self._chunks(shape[0]):
            P.forward(vol, out=dev[v0:v0 + n], view0=v0, nviews=n, transposed=xzy)
            done = torch.cuda.Event()
            done.record(compute)
            copy.wait_event(done)
            with torch.cuda.stream(copy):
                out[v0:v0 + n].copy_(dev[v0:v0 + n], non_blocking=True)
        copy.synchronize()
        return out

    def _backward_pinned(self, src):
        P = self.projector
        compute, copy = self._streams()
        shape = P.proj_shape()
        if tuple(src.shape) != tuple(shape):
            raise ValueError("proj must have shape %s, got %s" % (shape, tuple(src.shape)))
        q = self._device_buffer("proj_in", shape)
        vol = self._device_buffer("vol", P.volume_shape)
        # Symmetric orbits: each chunk is a range of base views, whose nc
        # slabs (one per 1/nc turn) are copied before its launch.
        nc = P.orbit_size()
        if nc == 1:
            for i, (v0, n) in enumerate(self._chunks(shape[0])):
                with torch.cuda.stream(copy):
                    q[v0:v0 + n].copy_(src[v0:v0 + n], non_blocking=True)
                landed = torch.cuda.Event()
                landed.record(copy)
                compute.wait_event(landed)
                P.backproject_fdk(q[v0:v0 + n], out=vol, view0=v0, nviews=n, accumulate=i > 0)
            return self._to_host(vol, src, "image")
        period = shape[0] // nc
        for i, (b0, n) in enumerate(self._chunks(period)):
            with torch.cuda.stream(copy):
                for k in range(nc):
                    v0 = b0 + k * period
                    q[v0:v0 + n].copy_(src[v0:v0 + n], non_blocking=True)
            landed = torch.cuda.Event()
            landed.record(copy)
            compute.wait_event(landed)
            P.backproject_fdk_orbits(q, vol, b0, n, accumulate=i > 0)
        return self._to_host(vol, src, "image")

    # -- projectors ----------------------------------------------------------------
    def forward(self):
        """self.proj = forward projection of self.image: DD (distance_forward)
        for Method 'Distance', Siddon ray sums for Method 'Ray' (a stub in
        the reference, Reconstruction_numba.py:799-801)."""
        if self.Method not in ('Distance', 'Ray'):
            return
        src = self.image
        host = _on_host(src)
        if host and self.Method == 'Distance' and isinstance(src, torch.Tensor) and src.is_pinned():
            self.proj = self._forward_pinned(src)
            return
        vol = _to_device(src, self.projector.device)
        proj = self.projector.forward(vol) if self.Method == 'Distance' else self.projector.ray_forward(vol)
        self.proj = self._to_host(proj, src, "proj") if host else proj

    def backward(self):
        """self.image = FDK-weighted DD backprojection of self.proj * dtheta
        (distance_backproj) for Method 'Distance'; for Method 'Ray' (a stub
        in the reference, :266-268) the transpose of the ray projector times
        dtheta."""
        if self.Method not in ('Distance', 'Ray'):
            return
        src = self.proj
        host = _on_host(src)
        if host and self.Method == 'Distance' and isinstance(src, torch.Tensor) and src.is_pinned():
            self.image = self._backward_pinned(src)
            return
        q = _to_device(src, self.projector.device)
        if self.Method == 'Distance':
            vol = self.projector.backproject_fdk(q)
        else:
            vol = self.projector.ray_backproject(q, scale=self.projector.params.dtheta)
        self.image = self._to_host(vol, src, "image") if host else vol

    def Filtering(self):
        """In-place cosine pre-weight and ramp filter of self.proj (Filtering)."""
        src = self.proj
        host = _on_host(src)
        q = _to_device(src, self.projector.device)
        self.projector.filter(q, self.FilterType, self.cutoff)
        self.proj = self._to_host(q, src, "proj") if host else q


def _pinned_like(cache, key, t):
    buf = cache.get(key)
    if buf is None or buf.shape != t.shape:
        buf = torch.empty(t.shape, dtype=torch.float32, pin_memory=True)
        cache[key] = buf
    return buf


def _host(a):
    if isinstance(a, torch.Tensor):
        return a.detach().to("cpu").numpy()
    return a
