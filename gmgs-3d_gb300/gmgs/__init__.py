"""GB300-native GMGS-3D solve: geometric-multigrid-preconditioned CG for
static linear elasticity on Cartesian voxel meshes (libgmgs.so + ctypes)."""
from . import mesh, synthetic
from ._lib import GMGSLibraryMissing, load
from .solver import GMGSError, Session, Solver

__all__ = ["Solver", "Session", "GMGSError", "GMGSLibraryMissing", "load", "mesh", "synthetic"]
