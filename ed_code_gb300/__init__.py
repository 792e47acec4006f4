"""GB300-native momentum-sector exact diagonalisation (the H*v hot path of
hiteshjc/ED_Code), behind a C ABI (include/edgpu.h).

Modules:
  lattice  -- torus generators and the reference input format
  sector   -- GpuSector: basis + H*v on the GPU through libedgpu.so
  build    -- compiles libedgpu.so for sm_103a
"""
from . import lattice  # noqa: F401

__all__ = ["lattice"]
