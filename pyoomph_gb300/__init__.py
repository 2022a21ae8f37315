"""pyoomph_gb300: GB300-native (sm_103a) residual/Jacobian assembly for
pyoomph-style finite-element problems.

The element kernels are generated from the weak form (``codegen``),
compiled with nvrtc for sm_103a and run through the C-ABI library
``libfe_gb300.so`` (``include/fe_gb300.h``).  There is no CPU fallback:
without the native library or a GPU the calls raise.
"""
from .equations import (DiffusionEquation, DirichletBC, Equations, NavierStokesEquations,
                        NonlinearDiffusionEquation, PoissonEquation, PressureFixation, StokesEquations)
from .expressions import (div, dot, exp, gaussian_source, grad, identity_matrix, material_derivative, partial_t,
                          parameter, sym, testfunction, var, var_and_test, weak)
from .meshes import CuboidBrickMesh, RectangularQuadMesh
from .assembly import CustomAssemblyBase, GB300Assembler
from .problem import NewtonSolverError, Problem

__all__ = ["CustomAssemblyBase", "GB300Assembler", "Problem", "NewtonSolverError", "Equations", "PoissonEquation", "DiffusionEquation", "NonlinearDiffusionEquation",
           "StokesEquations", "NavierStokesEquations", "DirichletBC", "PressureFixation", "RectangularQuadMesh",
           "CuboidBrickMesh", "var", "testfunction", "var_and_test", "grad", "div", "dot", "sym", "weak", "exp",
           "identity_matrix", "material_derivative", "partial_t", "parameter", "gaussian_source"]
