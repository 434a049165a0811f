"""GB300-native CT projection/backprojection (distance-driven), a drop-in for
the hot path of leehoy/CTReconstruction.

Public API:
  Reconstruction          the reference's call surface (forward/backward/Filtering, raw I/O)
  ReconstructionParams    the reference's params dict, validated
  Projector               device-resident projectors on CUDA tensors
"""
from .geometry import ReconstructionParams
from .projector import Projector
from .reconstruction import Reconstruction, ErrorDescription

__all__ = ["Reconstruction", "ReconstructionParams", "Projector", "ErrorDescription"]
