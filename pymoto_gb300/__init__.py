"""pymoto_gb300 -- pyMOTO's structured-grid topology-optimisation hot path on GB300 (sm_103a).

Drop-in GPU Modules and LinearSolvers with pyMOTO's API:
  DensityFilter, FilterConv, OverhangFilter, SIMP, MathExpression (any sympy expression; the SIMP form on its kernels),
  AssembleStiffness, AssembleMass, AssemblePoisson, LinSolve, EinSum,
  CG, GeometricMultigrid, DampedJacobi, DenseCholesky, MixedPrecisionCG, OC, MMA (MMA1987 / MMA2007 / GCMMA), Scaling,
  WriteToVTI (VoxelDomain.write_to_vti), ScalarToFile, finite_difference, minimize_oc, minimize_mma.
The arithmetic runs in hand-written CUDA kernels of libpymoto_gb300.so through its C ABI
(include/pymoto_gb300.h); there is no CPU fallback.
"""
from . import _lib
from .core import HOST_RUNTIME, Module, Network, Signal
from .domain import VoxelDomain
from .modules import (AssembleMass, AssemblePoisson, AssembleStiffness, DensityFilter, DeviceDyad, EinSum, FilterConv, LinSolve, MathExpression,
                      SIMP, Scaling)
from .operators import (Grid, ScalarOperator, StencilOperator, StiffnessOperator, element_stiffness,
                        operator_kernel, set_operator_kernel)
from .optimizers import OC
from .mma import MMA
from .solvers import (CG, Chebyshev, DampedJacobi, DenseCholesky, GeometricMultigrid, LinearSolver,
                      MixedPrecisionCG, Preconditioner)
from .autograd import ComplianceObjective
from .vti import WriteToVTI
from .scalars import DesignLog, ScalarToFile
from .overhang import OverhangFilter
from .checkpoint import load_checkpoint, save_checkpoint
from .routines import finite_difference, minimize_mma, minimize_oc

__version__ = "0.1.0"

__all__ = ["AssembleMass", "AssemblePoisson", "AssembleStiffness", "DensityFilter", "DeviceDyad", "EinSum", "FilterConv", "LinSolve", "MathExpression",
           "SIMP", "Grid", "ScalarOperator", "StencilOperator", "StiffnessOperator", "element_stiffness", "OC", "CG", "Chebyshev", "DampedJacobi",
           "DenseCholesky", "GeometricMultigrid", "LinearSolver", "MixedPrecisionCG", "Preconditioner",
           "VoxelDomain", "Module", "Network", "Signal", "HOST_RUNTIME", "ComplianceObjective", "WriteToVTI", "Scaling",
           "MMA", "ScalarToFile", "finite_difference",
           "minimize_oc", "minimize_mma", "OverhangFilter",
           "save_checkpoint", "load_checkpoint", "DesignLog", "set_operator_kernel", "operator_kernel"]
