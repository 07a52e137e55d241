"""helmholtz.jl_gb300: GB300-native shifted-Laplacian multigrid Helmholtz solver.

The compute path is the CUDA library ``libhelmgpu.so`` (sources in ``csrc/``,
C ABI in ``include/helmgpu.h``); this package is the host-side mirror of the
Helmholtz.jl API on top of it (see ``api.py``).  The directory name holds a
dot, so load it with ``load_package()`` from ``__graft_entry__`` or with
importlib; it registers itself as ``helmholtz_jl_gb300``.
"""
from .api import *  # noqa: F401,F403
from .api import (GetHelmholtzOperator, GetHelmholtzShiftOP, HelmholtzOperator, HelmholtzParam, MGparam,
                  RegularMesh, ShiftedLaplacianMultigridSolver, clear_, copySolver, getABL, getAcousticPointSource,
                  getHelmholtzFun, getMaximalFrequency, getMGparam, getMidPointSrc, getRegularMesh,
                  getShiftedHelmholtzParam, getShiftedLaplacianMultigridSolver, getSommerfeldBC, getTopPointSrc,
                  helmholtz_mass, loc2cs, solveLinearSystem, solveLinearSystemInPlace)
from . import _lib  # noqa: F401
from . import learned  # noqa: F401

__all__ = [
    "GetHelmholtzOperator", "GetHelmholtzShiftOP", "HelmholtzOperator", "HelmholtzParam", "MGparam", "RegularMesh",
    "ShiftedLaplacianMultigridSolver", "clear_", "copySolver", "getABL", "getAcousticPointSource", "getHelmholtzFun",
    "getMaximalFrequency", "getMGparam", "getMidPointSrc", "getRegularMesh", "getShiftedHelmholtzParam",
    "getShiftedLaplacianMultigridSolver", "getSommerfeldBC", "getTopPointSrc", "helmholtz_mass", "loc2cs",
    "solveLinearSystem", "solveLinearSystemInPlace",
]
