"""SIMP optimizer of the Python numerical path, on the GB300 engine.

Drop-in for src/am/numerical/topopt.py: ``SIMPParams`` (:30-52), ``TOResult``
(:55-81), ``SIMPOptimizer(domain, load_cases, material, params,
verbose).run(callback)`` (:84-411) and ``threshold_density`` (:414-428).  The
loop runs on the device (variant AM_VARIANT_PY of include/am_gpu.h): density
pre-filter and clip, per-load-case solve / compliance / sensitivities, the
normalised reflect-mode cone filter of dc*rho / max(rho, 1e-3), the OC
bisection with the Python constants.  The direct sparse solve of the reference
is replaced by PCG to ``cg_tol`` (FP64) or mixed precision (FP32 PCG with FP64
residual replacement, every solve accepted on its FP64 residual).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Callable, List, Optional

import numpy as np

from .. import _native as nat
from ..core import LoadCase, VoxelDomain
from .fem import MaterialProperties


@dataclass
class SIMPParams:
    volume_fraction: float = 0.25
    penalty: float = 3.0
    filter_radius: float = 2.0
    move_limit: float = 0.2
    rho_min: float = 0.01
    max_iterations: int = 100
    convergence_tol: float = 0.01
    E_min: float = 1e-9
    # engine knobs (no counterpart in the reference, which solves directly)
    precision: int = nat.PREC_FP64
    cg_tol: float = 1e-8
    cg_max_iterations: int = 100000
    warm_start: bool = True


@dataclass
class TOResult:
    density: np.ndarray
    compliance_history: List[float] = field(default_factory=list)
    volume_history: List[float] = field(default_factory=list)
    iterations: int = 0
    converged: bool = False
    elapsed_time: float = 0.0
    solver_iterations: List[int] = field(default_factory=list)

    @property
    def final_compliance(self) -> float:
        return self.compliance_history[-1] if self.compliance_history else 0.0

    @property
    def final_volume(self) -> float:
        return self.volume_history[-1] if self.volume_history else 0.0


class SIMPOptimizer:
    def __init__(self, domain: VoxelDomain, load_cases: List[LoadCase], material: Optional[MaterialProperties] = None,
                 params: Optional[SIMPParams] = None, verbose: bool = True):
        self.domain = domain
        self.load_cases = list(load_cases)
        self.material = material or MaterialProperties()
        self.params = params or SIMPParams()
        self.verbose = verbose
        self.nx, self.ny, self.nz = domain.shape
        self.n_elements = domain.n_elements
        self.element_size = domain.resolution_mm / 1000.0
        self.density = np.ones((self.nx, self.ny, self.nz)) * self.params.volume_fraction
        self.design_mask = domain.grid == 0
        n_dofs = 3 * (self.nx + 1) * (self.ny + 1) * (self.nz + 1)
        self._problem = nat.Problem(domain.shape, self.element_size, self.material.E, self.material.nu,
                                    grid=domain.grid)
        self._problem.set_loads([lc.get_force_vector(n_dofs) for lc in self.load_cases],
                                [lc.get_constrained_dofs() for lc in self.load_cases])

    def _config(self) -> nat.SimpConfig:
        p = self.params
        return nat.default_config(
            nat.VARIANT_PY, volume_fraction=float(p.volume_fraction), penalty=float(p.penalty),
            filter_radius=float(p.filter_radius), move_limit=float(p.move_limit), rho_min=float(p.rho_min),
            E_min=float(p.E_min), convergence_tol=float(p.convergence_tol), max_iterations=int(p.max_iterations),
            precision=int(p.precision), cg_tol=float(p.cg_tol), cg_max_iterations=int(p.cg_max_iterations),
            warm_start=int(bool(p.warm_start)))

    def run(self, callback: Optional[Callable] = None) -> TOResult:
        t0 = time.time()
        cfg = self._config()
        P = self._problem
        P.simp_begin(cfg, None)
        ch, vh, its = [], [], []
        converged = False
        iteration = 0
        for iteration in range(self.params.max_iterations):
            r = P.simp_step()
            ch.append(r.compliance)
            vh.append(r.volume_fraction)
            its.append(r.solver_iterations)
            if self.verbose:
                print(f"Iter {iteration + 1:3d} | Compliance: {r.compliance:.4e} | Volume: {r.volume_fraction:.4f} | "
                      f"Change: {r.max_density_change:.4f} | PCG: {r.solver_iterations}")
            if callback:
                callback(iteration, P.simp_density().reshape(self.domain.shape), r.compliance)
            if r.max_density_change < self.params.convergence_tol:
                converged = True
                break
        density = P.simp_density().reshape(self.domain.shape)
        self.density = density
        return TOResult(density=density, compliance_history=ch, volume_history=vh, iterations=iteration + 1,
                        converged=converged, elapsed_time=time.time() - t0, solver_iterations=its)


def threshold_density(density: np.ndarray, threshold: float = 0.5) -> np.ndarray:
    return (np.asarray(density) >= threshold).astype(np.float64)
