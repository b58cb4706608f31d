"""Problem-definition types of the SIMP entry points.

Same names, fields and index conventions as the reference's input types
(src/am/core/geometry.py:16-76 ``VoxelDomain``; src/am/core/loads.py:16-156
``DOF``, ``BoundaryCondition``, ``PointLoad``, ``DistributedLoad``,
``LoadCase``) so that code building a domain and load cases for the reference
builds them for this engine unchanged.  Node index of (i, j, k):
``i*(ny+1)*(nz+1) + j*(nz+1) + k``; DOF ``3*node + d``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from enum import Enum
from typing import List, Tuple

import numpy as np

VOID, DESIGN, FIXED = -1, 0, 1


@dataclass
class VoxelDomain:
    """Voxel grid with cell tags -1 void, 0 design, 1 fixed (non-design solid)."""

    grid: np.ndarray
    resolution_mm: float
    origin: Tuple[float, float, float] = (0.0, 0.0, 0.0)

    @property
    def shape(self) -> Tuple[int, int, int]:
        return tuple(int(s) for s in self.grid.shape)

    @property
    def size_mm(self) -> Tuple[float, float, float]:
        return tuple(s * self.resolution_mm for s in self.shape)

    @property
    def n_elements(self) -> int:
        return int(np.prod(self.shape))

    @property
    def n_design(self) -> int:
        return int(np.count_nonzero(self.grid == DESIGN))

    @property
    def n_fixed(self) -> int:
        return int(np.count_nonzero(self.grid == FIXED))

    def get_design_indices(self) -> np.ndarray:
        return np.argwhere(self.grid == DESIGN)

    def get_fixed_indices(self) -> np.ndarray:
        return np.argwhere(self.grid == FIXED)

    def voxel_to_coords(self, indices: np.ndarray) -> np.ndarray:
        """Voxel-centre coordinates in mm."""
        return (np.asarray(indices) + 0.5) * self.resolution_mm + np.asarray(self.origin)


class DOF(Enum):
    UX = 0
    UY = 1
    UZ = 2


@dataclass
class BoundaryCondition:
    """Homogeneous Dirichlet constraint of the listed DOFs of the listed nodes."""

    node_indices: np.ndarray
    constrained_dofs: List[DOF] = field(default_factory=lambda: [DOF.UX, DOF.UY, DOF.UZ])
    prescribed_values: float = 0.0

    @property
    def n_nodes(self) -> int:
        return len(self.node_indices)

    def get_dof_indices(self, dofs_per_node: int = 3) -> np.ndarray:
        nodes = np.asarray(self.node_indices, dtype=np.int64).reshape(-1, 1)
        comps = np.array([d.value for d in self.constrained_dofs], dtype=np.int64).reshape(1, -1)
        return (nodes * dofs_per_node + comps).ravel()


@dataclass
class PointLoad:
    node_index: int
    force_vector: np.ndarray

    def __post_init__(self):
        self.force_vector = np.asarray(self.force_vector, dtype=np.float64)
        if self.force_vector.shape != (3,):
            raise ValueError("force_vector must have shape (3,)")


@dataclass
class DistributedLoad:
    """Total force split uniformly over the listed nodes."""

    node_indices: np.ndarray
    total_force: np.ndarray
    distribution: str = "uniform"

    def __post_init__(self):
        self.node_indices = np.asarray(self.node_indices, dtype=np.int64)
        self.total_force = np.asarray(self.total_force, dtype=np.float64)

    def get_nodal_forces(self) -> np.ndarray:
        if self.distribution != "uniform":
            raise NotImplementedError(f"Distribution '{self.distribution}' not implemented")
        n = len(self.node_indices)
        return np.tile(self.total_force / n, (n, 1))


@dataclass
class LoadCase:
    name: str
    description: str = ""
    boundary_conditions: List[BoundaryCondition] = field(default_factory=list)
    point_loads: List[PointLoad] = field(default_factory=list)
    distributed_loads: List[DistributedLoad] = field(default_factory=list)

    def get_force_vector(self, n_dofs: int) -> np.ndarray:
        F = np.zeros(n_dofs, dtype=np.float64)
        for pl in self.point_loads:
            F[3 * int(pl.node_index) + np.arange(3)] += pl.force_vector
        for dl in self.distributed_loads:
            f = dl.get_nodal_forces()
            for node, fv in zip(dl.node_indices, f):
                F[3 * int(node) + np.arange(3)] += fv
        return F

    def get_constrained_dofs(self) -> np.ndarray:
        if not self.boundary_conditions:
            return np.zeros(0, dtype=np.int64)
        return np.unique(np.concatenate([bc.get_dof_indices() for bc in self.boundary_conditions]))


def node_index(i: int, j: int, k: int, shape) -> int:
    """Reference node numbering (fem.py:168)."""
    nx, ny, nz = shape
    return (i * (ny + 1) + j) * (nz + 1) + k


# ---------------------------------------------------------------------------
# BRK-A-01 bracket set-up on the device (am_bracket_build in include/am_gpu.h)
# ---------------------------------------------------------------------------
def _bracket_params(shape, resolution_mm, size_mm=(120, 60, 80), base_thickness_mm=5.0, hole_diameter_mm=8.0,
                    eyelet_diameter_mm=12.0, eyelet_offset_mm=4.0):
    from . import _native as nat

    p = nat.BracketParams()
    nat.load().am_bracket_params_default(p, float(resolution_mm))
    p.size_mm[:] = [float(v) for v in size_mm]
    p.base_thickness_mm = float(base_thickness_mm)
    p.hole_diameter_mm = float(hole_diameter_mm)
    p.eyelet_diameter_mm = float(eyelet_diameter_mm)
    p.eyelet_offset_mm = float(eyelet_offset_mm)
    if shape is None:
        shape = tuple(int(s / resolution_mm) for s in size_mm)
    p.nx, p.ny, p.nz = (int(v) for v in shape)
    return p


def create_bracket_domain(size_mm=(120, 60, 80), resolution_mm: float = 1.0, base_thickness_mm: float = 5.0,
                          hole_diameter_mm: float = 8.0, eyelet_diameter_mm: float = 12.0,
                          eyelet_offset_mm: float = 4.0) -> VoxelDomain:
    """The BRK-A-01 design domain (geometry.py:79-196): fixed flange with four void
    holes, fixed eyelet ring with its void hole, fixed pillar between them,
    design space elsewhere.  Built by a device kernel; identical to the
    reference's grid cell for cell."""
    from . import _native as nat

    p = _bracket_params(None, resolution_mm, size_mm, base_thickness_mm, hole_diameter_mm, eyelet_diameter_mm,
                        eyelet_offset_mm)
    grid = np.zeros((p.nx, p.ny, p.nz), dtype=np.int8)
    nat.check(nat.load().am_bracket_build(p, None, nat.LAYOUT_ZFASTEST, nat.ptr(grid, nat._i8p), None, None, None,
                                          None, None, 0), "am_bracket_build")
    return VoxelDomain(grid=grid, resolution_mm=resolution_mm)


def _brk_case(domain_shape, resolution_mm, total_force, name, description) -> LoadCase:
    from . import _native as nat

    p = _bracket_params(domain_shape, resolution_mm)
    nx, ny, nz = p.nx, p.ny, p.nz
    cap = (2 * (int(12.0 / resolution_mm) + 3) + 1) ** 2 + 1
    nodes = np.zeros(cap, dtype=np.int64)
    n_nodes = ctypes.c_int64(0)
    nat.check(nat.load().am_bracket_build(p, None, nat.LAYOUT_ZFASTEST, None, None, None, None,
                                          nat.ptr(nodes, nat._i64p), ctypes.byref(n_nodes), cap),
              "am_bracket_build")
    base = np.array([i * (ny + 1) * (nz + 1) + j * (nz + 1) for i in range(nx + 1) for j in range(ny + 1)],
                    dtype=np.int64)
    return LoadCase(name=name, description=description,
                    boundary_conditions=[BoundaryCondition(node_indices=base)],
                    distributed_loads=[DistributedLoad(node_indices=nodes[:n_nodes.value].copy(),
                                                       total_force=np.asarray(total_force, dtype=np.float64))])


def create_brk_a_01_static_case_1(domain_shape, resolution_mm: float = 1.0) -> LoadCase:
    """Static case 1 (loads.py:163-264): base nodes (z = 0) clamped, 15 kN in -z
    spread over the eyelet's load ring (ring nodes found on the device)."""
    return _brk_case(domain_shape, resolution_mm, [0.0, 0.0, -15000.0], "BRK-A-01_Static_1",
                     "Vertical 15 kN on the eyelet, base clamped")


def create_brk_a_01_static_case_2(domain_shape, resolution_mm: float = 1.0) -> LoadCase:
    """Static case 2 (loads.py:267-300): the same ring, 10 kN inclined 30 degrees
    from -z towards +x."""
    angle = np.radians(30)
    return _brk_case(domain_shape, resolution_mm, [10000.0 * np.sin(angle), 0.0, -10000.0 * np.cos(angle)],
                     "BRK-A-01_Static_2", "10 kN inclined 30 degrees on the eyelet, base clamped")


def bracket_force_vector(domain_shape, resolution_mm: float, total_force) -> np.ndarray:
    """The force vector of a BRK-A-01 load case formed on the device."""
    from . import _native as nat

    p = _bracket_params(domain_shape, resolution_mm)
    F = np.zeros(3 * (p.nx + 1) * (p.ny + 1) * (p.nz + 1))
    tf = np.ascontiguousarray(total_force, dtype=np.float64)
    nat.check(nat.load().am_bracket_build(p, nat.ptr(tf), nat.LAYOUT_ZFASTEST, None, nat.ptr(F), None, None, None,
                                          None, 0), "am_bracket_build")
    return F


def bracket_fixed_dofs(domain_shape, resolution_mm: float = 1.0) -> np.ndarray:
    """The base constraints of the BRK-A-01 load cases formed on the device."""
    from . import _native as nat

    p = _bracket_params(domain_shape, resolution_mm)
    n = ctypes.c_int64(0)
    out = np.zeros(3 * (p.nx + 1) * (p.ny + 1), dtype=np.int64)
    nat.check(nat.load().am_bracket_build(p, None, nat.LAYOUT_ZFASTEST, None, None, nat.ptr(out, nat._i64p),
                                          ctypes.byref(n), None, None, 0), "am_bracket_build")
    return out[:n.value]
