"""spatial_cell_gb300: the per-step simulation hot path of spatial_cell_sim
(justgos/spatial-cell) on GB300 (sm_103a), behind the C ABI of
include/spatialcell.h.

* ``abi`` -- the reference's byte layouts (particles, reduced frame records,
  rule / type tables) as numpy dtypes, and the config struct;
* ``native`` -- ctypes binding of libspatialcell.so (``Simulation``);
* ``scenes`` -- seeded synthetic states of the measured workloads;
* ``build`` -- in-tree nvcc build of the library.
"""
from . import abi  # noqa: F401

__all__ = ["abi", "native", "scenes", "build"]
