"""AIOptimizer: the inference pipeline of src/am/ai/inference.py:18-133 -- encode a
problem (voxel domain + load cases) as a 4-channel tensor, predict the density
with the U-Net, post-process, and validate against the numerical SIMP solution
(IoU, compliance error, volume error)."""
from __future__ import annotations

from pathlib import Path
from typing import List, Optional, Union

import numpy as np

from .. import _native as nat
from ..core import LoadCase, VoxelDomain
from .model import TopOptUNet, load_pretrained


def element_loads(domain: VoxelDomain, load_cases: List[LoadCase]) -> np.ndarray:
    """(3, nx, ny, nz): the summed load cases' nodal forces averaged onto the
    elements (each element the mean over its 8 nodes), scaled to a largest
    magnitude of 1."""
    nx, ny, nz = domain.shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    F = np.zeros(N)
    for lc in load_cases:
        F += lc.get_force_vector(N)
    f = F.reshape(nx + 1, ny + 1, nz + 1, 3)
    e = np.zeros((nx, ny, nz, 3))
    for di in (0, 1):
        for dj in (0, 1):
            for dk in (0, 1):
                e += f[di:di + nx, dj:dj + ny, dk:dk + nz]
    e /= 8.0
    m = np.abs(e).max()
    if m > 0:
        e /= m
    return np.moveaxis(e, -1, 0)


def element_constraints(domain: VoxelDomain, load_cases: List[LoadCase]) -> np.ndarray:
    """(3, nx, ny, nz): per element and component, the fraction of its 8 nodes
    whose DOF of that component is constrained in some load case."""
    nx, ny, nz = domain.shape
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    fixed = np.zeros(3 * nn)
    for lc in load_cases:
        idx = np.asarray(lc.get_constrained_dofs(), dtype=np.int64)
        fixed[idx[(idx >= 0) & (idx < 3 * nn)]] = 1.0
    f = fixed.reshape(nx + 1, ny + 1, nz + 1, 3)
    e = np.zeros((nx, ny, nz, 3))
    for di in (0, 1):
        for dj in (0, 1):
            for dk in (0, 1):
                e += f[di:di + nx, dj:dj + ny, dk:dk + nz]
    return np.moveaxis(e / 8.0, -1, 0)


class AIOptimizer:
    """Density prediction by a trained TopOptUNet (inference.py:18-113).

    The encoding: channel 0 the domain (-1 void, 0 design, 1 fixed), channels 1-3
    the loads on the elements (element_loads), channels 4-6 of a 7-channel model
    the constrained DOFs (element_constraints).  A model predicts designs for the
    SIMP parameters it was trained with (volume fraction, filter radius, penalty:
    stored in the checkpoint)."""

    def __init__(self, model_path: Optional[Union[str, Path]] = None, device: str = "cuda"):
        if device not in ("cuda", "cuda:0"):
            raise ValueError("the engine runs on the CUDA device only")
        self.device = device
        self.model: Optional[TopOptUNet] = None
        if model_path is not None:
            self.load_model(model_path)

    def load_model(self, model_path: Union[str, Path]) -> None:
        self.model = load_pretrained(str(model_path))

    def encode_problem(self, domain: VoxelDomain, load_cases: List[LoadCase],
                       channels: Optional[int] = None) -> np.ndarray:
        """Input tensor (C, nx, ny, nz), the layout inference.py:61-79 of the
        reference sets out: channel 0 the domain, channels 1-3 the loads and, for a
        7-channel model, channels 4-6 the constrained DOFs (element_constraints).
        C is the loaded model's in_channels (4 without a model) unless given."""
        if channels is None:
            channels = self.model.in_channels if self.model is not None else 4
        if channels not in (4, 7):
            raise ValueError("the encoding has 4 or 7 channels")
        g = np.asarray(domain.grid, dtype=np.float32)
        parts = [g[None], element_loads(domain, load_cases).astype(np.float32)]
        if channels == 7:
            parts.append(element_constraints(domain, load_cases).astype(np.float32))
        return np.concatenate(parts, axis=0)

    def predict(self, domain: VoxelDomain, load_cases: List[LoadCase],
                threshold: Optional[float] = 0.5) -> np.ndarray:
        """Predicted density field (nx, ny, nz): void cells 0, fixed cells 1; with a
        threshold the design cells are binarised (density >= threshold -> 1)."""
        if self.model is None:
            raise RuntimeError("no model loaded (AIOptimizer(model_path=...) or load_model)")
        rho = self.model.predict(self.encode_problem(domain, load_cases)).astype(np.float64)
        g = np.asarray(domain.grid)
        rho = np.where(g == -1, 0.0, np.where(g == 1, 1.0, rho))
        if threshold is not None:
            rho = np.where(g == 0, (rho >= threshold).astype(np.float64), rho)
        return rho

    def validate_against_numerical(self, domain: VoxelDomain, load_cases: List[LoadCase],
                                   numerical_density: Optional[np.ndarray] = None) -> dict:
        """IoU of the thresholded designs, relative compliance error of the predicted
        design, and its volume error, against the SIMP solution of the engine
        (run here unless numerical_density is given)."""
        from ..numerical.fem import MaterialProperties
        from ..numerical.topopt import SIMPOptimizer, SIMPParams

        meta = self.model.meta if self.model else {}
        prm = SIMPParams(volume_fraction=float(meta.get("volume_fraction", 0.3)),
                         filter_radius=float(meta.get("filter_radius", 1.5)),
                         max_iterations=int(meta.get("simp_iterations", 40)), convergence_tol=0.0,
                         precision=nat.PREC_MIXED, cg_tol=1e-6)
        mat = MaterialProperties(E=1.0, nu=0.3)
        if numerical_density is None:
            numerical_density = SIMPOptimizer(domain, load_cases, mat, prm, verbose=False).run().density
        pred = self.predict(domain, load_cases, threshold=None)
        design = np.asarray(domain.grid) == 0
        a, b = pred[design] >= 0.5, numerical_density[design] >= 0.5
        iou = float((a & b).sum() / max((a | b).sum(), 1))
        # compliance of each design under the same loads (SIMP stiffness rho^p)
        comp = []
        p = nat.Problem(domain.shape, domain.resolution_mm / 1000.0, mat.E, mat.nu, grid=domain.grid)
        nx, ny, nz = domain.shape
        N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
        p.set_loads([lc.get_force_vector(N) for lc in load_cases], [lc.get_constrained_dofs() for lc in load_cases])
        cfg = nat.default_config(nat.VARIANT_PY, E_min=1e-9, penalty=3.0, precision=nat.PREC_MIXED, cg_tol=1e-8,
                                 warm_start=0)
        for rho in (pred, numerical_density):
            c = 0.0
            for k, lc in enumerate(load_cases):
                u, _ = p.solve(cfg, np.clip(rho, 0.01, 1.0), load_case=k)
                c += float(lc.get_force_vector(N) @ u)
            comp.append(c)
        p.close()
        vol_pred, vol_num = float(pred[design].mean()), float(numerical_density[design].mean())
        return {"iou": iou, "compliance_ai": comp[0], "compliance_numerical": comp[1],
                "compliance_error": (comp[0] - comp[1]) / comp[1], "volume_ai": vol_pred,
                "volume_numerical": vol_num, "volume_error": vol_pred - vol_num}


def run_ai_optimization(domain: VoxelDomain, load_cases: List[LoadCase],
                        model_path: Optional[str] = None) -> np.ndarray:
    """Convenience wrapper (inference.py:116-133): the thresholded prediction."""
    if model_path is None:
        raise ValueError("a trained model checkpoint is required (python -m am_ml_suite_gb300.ai.train)")
    return AIOptimizer(model_path=model_path).predict(domain, load_cases)
