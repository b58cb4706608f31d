"""Python numerical path (fem / topopt) on the GB300 engine."""
from .fem import (MaterialProperties, apply_stiffness, compute_element_compliance, get_element_dof_indices,
                  get_element_stiffness_matrix, solve_fem)
from .topopt import SIMPOptimizer, SIMPParams, TOResult, threshold_density

__all__ = ["MaterialProperties", "apply_stiffness", "compute_element_compliance", "get_element_dof_indices",
           "get_element_stiffness_matrix", "solve_fem", "SIMPOptimizer", "SIMPParams", "TOResult",
           "threshold_density"]
