"""GB300-native segregated finite-volume solid solver (solids4foam hot path).

The compute path is libs4g.so (hand-written CUDA for sm_103a behind the C ABI
of include/s4g.h); this package is its host-side mirror of the reference's
solidModel / mechanicalLaw interface.
"""
from . import _lib
from ._lib import S4GError, lib
from .cases import box_mesh, cantilever_case, cube_case
from .foam_case import read_case, read_relaxation
from .post import derived_fields, point_displacement
from .solid_model import Context, Server, SolidModel, solve_batch

__all__ = ["S4GError", "lib", "box_mesh", "cantilever_case", "cube_case", "Context",
           "Server", "SolidModel", "read_case", "read_relaxation", "point_displacement",
           "derived_fields", "solve_batch", "_lib"]
