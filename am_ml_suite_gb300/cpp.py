"""Python surface of the C++ engine, on the GB300 engine.

The reference's notebook (visualize_results.ipynb cells 23-24) imports a
``src.am.cpp`` binding whose source is not in the reference tree:
``CPPTopologyOptimizer(nx, ny, nz, element_size, material, config)`` with
``.run(initial_density, forces, fixed_dofs)`` and ``.run_iteration(...)``,
``MaterialProperties``, ``SIMPConfig``, ``get_max_threads()``,
``is_available()``.  This module provides that surface over the C ABI, with
TopologyOptimizer semantics (cpp_engine/src/topology_optimizer.cpp:294-520,
variant AM_VARIANT_CPP): relative E_min, design mask from the initial density,
sum w rho dc / sum w rho filter, OC 1e-20/1e20 to 1e-4, compliance u.F.
The density list is x-fastest (``iz*nx*ny + iy*nx + ix``), the index the C++
optimizer uses (topology_optimizer.hpp:218-232).
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field
from typing import Callable, List, Optional

import numpy as np

from . import _native as nat


@dataclass
class MaterialProperties:
    E: float = 113.8e9
    nu: float = 0.342
    rho: float = 4430.0


@dataclass
class SIMPConfig:
    """SIMPConfig of topology_optimizer.hpp:49-59 plus the engine's solver knobs."""

    volume_fraction: float = 0.25
    penalty: float = 3.0
    filter_radius: float = 2.0
    move_limit: float = 0.2
    rho_min: float = 0.01
    E_min: float = 1e-6
    max_iterations: int = 100
    convergence_tol: float = 0.01
    verbose: bool = True
    # solver (TopologyOptimizer uses tolerance 1e-6, topology_optimizer.cpp:35-40)
    cg_tol: float = 1e-6
    cg_max_iterations: int = 100000
    precision: int = nat.PREC_MIXED
    warm_start: bool = True
    # True: element stiffness scales read the density list with the reference
    # assembler's z-fastest index (global_assembler.hpp:162-164) like the reference
    # engine, to replay its runs; False: every density at its own element
    reference_assembly_index: bool = False


@dataclass
class IterationResult:
    compliance: float = 0.0
    volume_fraction: float = 0.0
    max_density_change: float = 0.0
    solver_iterations: int = 0
    assembly_time_s: float = 0.0
    solve_time_s: float = 0.0
    sensitivity_time_s: float = 0.0
    update_time_s: float = 0.0


@dataclass
class OptimizationResult:
    final_density: List[float] = field(default_factory=list)
    compliance_history: List[float] = field(default_factory=list)
    volume_history: List[float] = field(default_factory=list)
    iterations: int = 0
    converged: bool = False
    elapsed_time_s: float = 0.0


def is_available() -> bool:
    return nat.is_available()


def get_max_threads() -> int:
    """Streaming multiprocessors of the current device (the OpenMP thread count
    of the reference engine has no GPU meaning)."""
    sm = ctypes.c_int(0)
    nat.check(nat.load().am_device_info(ctypes.byref(sm), None, None), "am_device_info")
    return sm.value


class CPPTopologyOptimizer:
    def __init__(self, nx: int, ny: int, nz: int, element_size: float, material: MaterialProperties,
                 config: Optional[SIMPConfig] = None):
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.config = config or SIMPConfig()
        self.material = material
        self.element_size = float(element_size)
        self._p = nat.Problem((nx, ny, nz), element_size, material.E, material.nu, layout=nat.LAYOUT_XFASTEST)
        self._loads_key = None
        self._begun = False

    def num_elements(self) -> int:
        return self.nx * self.ny * self.nz

    def num_dofs(self) -> int:
        return 3 * (self.nx + 1) * (self.ny + 1) * (self.nz + 1)

    def _cfg(self) -> nat.SimpConfig:
        c = self.config
        return nat.default_config(
            nat.VARIANT_CPP, volume_fraction=float(c.volume_fraction), penalty=float(c.penalty),
            filter_radius=float(c.filter_radius), move_limit=float(c.move_limit), rho_min=float(c.rho_min),
            E_min=float(c.E_min), convergence_tol=float(c.convergence_tol), max_iterations=int(c.max_iterations),
            precision=int(c.precision), cg_tol=float(c.cg_tol), cg_max_iterations=int(c.cg_max_iterations),
            warm_start=int(bool(c.warm_start)), layout=nat.LAYOUT_XFASTEST,
            cpp_assembly_index=int(bool(c.reference_assembly_index)))

    def _set_loads(self, forces, fixed_dofs):
        F = np.ascontiguousarray(forces, dtype=np.float64).ravel()
        fx = np.ascontiguousarray(fixed_dofs, dtype=np.int64).ravel()
        key = (F.tobytes(), fx.tobytes())
        if key != self._loads_key:
            self._p.set_loads([F], [fx])
            self._loads_key = key

    def run(self, initial_density, forces, fixed_dofs,
            callback: Optional[Callable] = None) -> OptimizationResult:
        t0 = time.time()
        rho0 = np.asarray(initial_density, dtype=np.float64).ravel()
        if rho0.size != self.num_elements():
            # the reference silently resets to volume_fraction (topology_optimizer.cpp:403-405)
            rho0 = np.full(self.num_elements(), self.config.volume_fraction)
        self._set_loads(forces, fixed_dofs)
        cfg = self._cfg()
        self._p.simp_begin(cfg, rho0)
        self._begun = True
        res = OptimizationResult()
        for it in range(self.config.max_iterations):
            r = self._p.simp_step()
            res.compliance_history.append(r.compliance)
            res.volume_history.append(r.volume_fraction)
            res.iterations = it + 1
            if self.config.verbose:
                print(f"{it:6d} {r.compliance:14.4e} {r.volume_fraction:10.3f} {r.max_density_change:12.2e} "
                      f"{r.solver_iterations:10d}")
            if callback is not None:
                ir = IterationResult(r.compliance, r.volume_fraction, r.max_density_change, r.solver_iterations,
                                     r.assembly_time_s, r.solve_time_s, r.sensitivity_time_s, r.update_time_s)
                if not callback(it, list(self._p.simp_density()), ir):
                    break
            if r.max_density_change < self.config.convergence_tol:
                res.converged = True
                break
        res.final_density = list(self._p.simp_density())
        res.elapsed_time_s = time.time() - t0
        return res

    def run_iteration(self, density, forces, fixed_dofs) -> IterationResult:
        """One iteration (TopologyOptimizer::runIteration).  The density list is
        updated in place when it is a mutable list or array."""
        rho = np.asarray(density, dtype=np.float64).ravel()
        self._set_loads(forces, fixed_dofs)
        self._p.simp_begin(self._cfg(), rho)
        r = self._p.simp_step()
        new = self._p.simp_density()
        if isinstance(density, np.ndarray) and density.dtype == np.float64 and density.size == new.size:
            density.reshape(-1)[:] = new
        elif isinstance(density, list):
            density[:] = list(new)
        return IterationResult(r.compliance, r.volume_fraction, r.max_density_change, r.solver_iterations,
                               r.assembly_time_s, r.solve_time_s, r.sensitivity_time_s, r.update_time_s)
