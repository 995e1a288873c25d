"""semgb300 — host-side mirror of SpectralElements.jl's operator/solve API over
libsem_b200.so (GB300, sm_103a).

Names and argument meanings follow the reference: ``Mesh``, ``generateMask``,
``ABu``, ``lapl``, ``mass``, ``hlmz``, ``gatherScatter``, ``mask``, ``pcg``,
``pcg_`` (pcg!), ``Diffusion``.  Fields are CUDA float64 tensors in the
reference's column-major local layout.
"""
from ._lib import (SEM_F32, SEM_F64, SEM_F64_DF, SEM_GS, SEM_MASK, SEM_MIXED, SEM_MIXED_RR,  # noqa: F401
                   SEM_BDF_MAX_ORDER, SEM_PATH_AUTO, SEM_PATH_CHUNKED, SEM_PATH_SMALL, NotConverged, SemError, build, load)
from .host import bdfExtK, derivMat, fixU, gausslobatto, interpMat, ndgrid, semmesh, semq_index  # noqa: F401
from .mesh import Mesh, QQt, as_local, generateMask, local_empty  # noqa: F401
from .ops import ABu, advect, gatherScatter, grad, gradT, hlmz, lapl, mask, mass  # noqa: F401
from . import spectral  # noqa: F401
from .solver import (BatchSolver, Diffusion, HelmholtzOp, Jacobi, TimeStepper, identity,  # noqa: F401
                     linsolve, linsolve_varcoef, pcg, pcg_, transient_varcoef,
                     PcgSolver, VarCoefProblem)

__all__ = ["Mesh", "QQt", "generateMask", "ABu", "lapl", "mass", "hlmz", "gatherScatter", "mask",
           "grad", "gradT", "advect",
           "pcg", "pcg_", "HelmholtzOp", "Jacobi", "identity", "Diffusion", "TimeStepper",
           "linsolve_varcoef", "linsolve", "VarCoefProblem", "PcgSolver", "gausslobatto", "derivMat", "interpMat", "semmesh", "ndgrid",
           "semq_index", "bdfExtK", "fixU", "as_local", "local_empty", "build", "load",
           "SemError", "NotConverged", "SEM_F64", "SEM_F64_DF", "SEM_F32", "SEM_MIXED",
           "SEM_GS", "SEM_MASK", "SEM_MIXED_RR", "SEM_PATH_AUTO", "SEM_PATH_CHUNKED", "SEM_PATH_SMALL",
           "SEM_BDF_MAX_ORDER"]
