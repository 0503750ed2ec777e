"""GB300 lattice-Boltzmann solver step (host side over the C ABI).

``capi``: ctypes mirror of include/aeros_lbm.h; ``solver``: one device domain;
``geometry``: seeded meshes and solver configurations; ``batch`` / ``serve``:
many domains stepped together and the continuous-batching request loop.
"""
from . import batch, capi, geometry, serve, solver  # noqa: F401
from .batch import Batch  # noqa: F401
from .solver import Solver, voxel_grid, voxelize  # noqa: F401
