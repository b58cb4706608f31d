"""Problem-definition types of the SIMP entry points.

Same names, fields and index conventions as the reference's input types
(src/am/core/geometry.py:16-76 ``VoxelDomain``; src/am/core/loads.py:16-156
``DOF``, ``BoundaryCondition``, ``PointLoad``, ``DistributedLoad``,
``LoadCase``) so that code building a domain and load cases for the reference
builds them for this engine unchanged.  Node index of (i, j, k):
``i*(ny+1)*(nz+1) + j*(nz+1) + k``; DOF ``3*node + d``.
"""
from __future__ import annotations

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
