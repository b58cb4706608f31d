"""FEM primitives of the Python numerical path, on the GB300 engine.

Mirrors src/am/numerical/fem.py: ``MaterialProperties`` (:18-40),
``get_element_stiffness_matrix`` (:43-135), ``get_element_dof_indices``
(:138-172), ``solve_fem`` (:251-325) and ``compute_element_compliance``
(:328-383).  ``assemble_global_stiffness`` (:175-248) has no counterpart: the
engine never forms K; ``apply_stiffness`` gives K(rho) u matrix-free.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np

from .. import _native as nat


@dataclass
class MaterialProperties:
    E: float = 113.8e9
    nu: float = 0.342
    rho: float = 4430.0

    @property
    def lame_lambda(self) -> float:
        return self.E * self.nu / ((1 + self.nu) * (1 - 2 * self.nu))

    @property
    def lame_mu(self) -> float:
        return self.E / (2 * (1 + self.nu))


def get_element_stiffness_matrix(element_size: float, material: MaterialProperties) -> np.ndarray:
    """24x24 KE of a cubic hex8 element (the operator the kernels apply)."""
    return nat.element_stiffness(material.E, material.nu, element_size)


_NODE_OFFSETS = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)])


def get_element_dof_indices(element_ijk: Tuple[int, int, int], grid_shape: Tuple[int, int, int]) -> np.ndarray:
    i, j, k = element_ijk
    nx, ny, nz = grid_shape
    n = ((i + _NODE_OFFSETS[:, 0]) * (ny + 1) + (j + _NODE_OFFSETS[:, 1])) * (nz + 1) + (k + _NODE_OFFSETS[:, 2])
    return (3 * n[:, None] + np.arange(3)[None, :]).ravel().astype(np.int64)


def _config(penalty, E_min, precision, tol):
    return nat.default_config(nat.VARIANT_PY, penalty=float(penalty), E_min=float(E_min), precision=precision,
                              cg_tol=float(tol), warm_start=0)


def apply_stiffness(domain_grid: np.ndarray, density: np.ndarray, u: np.ndarray, element_size: float,
                    material: MaterialProperties, penalty: float = 3.0, E_min: float = 1e-9,
                    precision: int = nat.PREC_FP64) -> np.ndarray:
    """K(rho) u with the scale rules of assemble_global_stiffness (void skipped,
    fixed cells full stiffness, design E_min + rho^p (E - E_min))."""
    grid = np.asarray(domain_grid)
    p = nat.Problem(grid.shape, element_size, material.E, material.nu, grid=grid)
    try:
        return p.ku(_config(penalty, E_min, precision, 1e-8), density, u, precision)
    finally:
        p.close()


def solve_fem(domain_grid: np.ndarray, density: np.ndarray, F: np.ndarray, constrained_dofs: np.ndarray,
              element_size: float, material: MaterialProperties, penalty: float = 3.0, E_min: float = 1e-9,
              tol: float = 1e-10, precision: int = nat.PREC_FP64) -> np.ndarray:
    """u with K_ff u_f = F_f; constrained and orphan DOFs (zero stiffness) get 0.

    The reference signature takes an assembled K; here the operator is defined
    by (grid, density, material) instead.  Raises ValueError on NaN/Inf like
    fem.py:316-319."""
    grid = np.asarray(domain_grid)
    p = nat.Problem(grid.shape, element_size, material.E, material.nu, grid=grid)
    try:
        p.set_loads([F], [np.asarray(constrained_dofs, dtype=np.int64)])
        u, st = p.solve(_config(penalty, E_min, precision, tol), density)
    except nat.AmError as e:
        raise ValueError(f"FEM solve failed: {e}") from e
    finally:
        p.close()
    if not np.all(np.isfinite(u)):
        raise ValueError("FEM solution contains NaN or Inf")
    return u


def compute_element_compliance(u: np.ndarray, domain_grid: np.ndarray, density: np.ndarray, element_size: float,
                               material: MaterialProperties, penalty: float = 3.0,
                               E_min: float = 1e-9) -> Tuple[float, np.ndarray]:
    """(sum, per-element) of E_ratio * u_e^T KE u_e over non-void cells."""
    grid = np.asarray(domain_grid)
    p = nat.Problem(grid.shape, element_size, material.E, material.nu, grid=grid)
    try:
        cfg = _config(penalty, E_min, nat.PREC_FP64, 1e-8)
        _, ce, total = p.sensitivities(cfg, density, u)
    finally:
        p.close()
    rho = np.asarray(density, dtype=np.float64).ravel()
    g = grid.ravel()
    ratio = np.where(g == 0, E_min / material.E + rho ** penalty * (1 - E_min / material.E), 1.0)
    per = np.where(g == -1, 0.0, ratio * ce).reshape(grid.shape)
    return float(total), per
