"""GB300-native batched per-voxel Levenberg-Marquardt fitter.

Drop-in for the fitter of turbotage/pycompute (``pycompute.cuda.lsqnonlin``):
a sympy model expression is generated into straight-line residual, Jacobian
and Hessian code, and every voxel runs its own second-order LM loop with GMW81
modified-Cholesky damped solves inside one sm_103a kernel launch.
"""
from .lsqnonlin import (F, Expr, F_GradF, GMW81Solver, RandomSearch, SearchStep,  # noqa: F401
                        SecondOrderLevenbergMarquardt, SecondOrderRandomSearch)

__all__ = ["Expr", "F_GradF", "F", "SecondOrderLevenbergMarquardt", "GMW81Solver", "SearchStep", "RandomSearch",
           "SecondOrderRandomSearch"]
