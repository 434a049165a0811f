"""Sharding hooks for running the path on several GPUs (one process each).

The DD path partitions without data exchange:
* the forward projection by views — each rank projects the full volume onto
  its own contiguous view range (``view_shard``);
* the backprojections by z slabs — each rank reconstructs its own slab of the
  volume from all views (``slab_params`` gives the slab's own geometry, so a
  Projector built from it is an ordinary scan).
Results are disjoint pieces of the output; gathering them is the caller's
choice (nothing here issues a collective).
"""
from .geometry import ReconstructionParams


def shard_range(n, rank, world):
    """Contiguous split of range(n) into `world` parts: (start, count) of `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside world %d" % (rank, world))
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def view_shard(params, rank, world):
    """(view0, nviews) of this rank's forward-projection shard."""
    p = ReconstructionParams.from_dict(params)
    return shard_range(p.NumberOfViews, rank, world)


def slab_params(params, z0, nz, flavour=None):
    """Geometry of the z slab [z0, z0 + nz) of the volume: the same scan with
    NumberOfImage z = nz and the volume centres moved so that the slab's voxel
    centres and boundary planes coincide with the full volume's
    (Reconstruction_numba.py:834-840, :409-411 place voxel i at
    centre + (i - (n-1)/2) * (-dz))."""
    p = ReconstructionParams.from_dict(params, flavour)
    nx, ny, nz_full = p.NumberOfImage
    if not (0 <= z0 and nz >= 1 and z0 + nz <= nz_full):
        raise ValueError("slab [%d, %d) outside [0, %d)" % (z0, z0 + nz, nz_full))
    dz = p.ImagePixelSpacing[2]
    shift = -((z0 + (nz - 1) / 2.0) - (nz_full - 1) / 2.0) * dz
    d = p.as_dict()
    d['NumberOfImage'] = [nx, ny, nz]
    d['PhantomCenter'] = [p.PhantomCenter[0], p.PhantomCenter[1], p.PhantomCenter[2] + shift]
    d['ReconCenter'] = [p.ReconCenter[0], p.ReconCenter[1], p.ReconCenter[2] + shift]
    return ReconstructionParams.from_dict(d, p.flavour)


def slab_shard(params, rank, world):
    """(z0, nz, slab params) of this rank's backprojection shard."""
    p = ReconstructionParams.from_dict(params)
    z0, nz = shard_range(p.NumberOfImage[2], rank, world)
    return z0, nz, slab_params(p, z0, nz)
