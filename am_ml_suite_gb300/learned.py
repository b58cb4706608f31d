"""Training set, training and stored weights of the learned preconditioner.

The network (``am_precond_*`` in include/am_gpu.h, csrc/precond.cu) is a 3-D
convolutional encoder-decoder -- 4 levels of 16/32/64/128 channels, 3x3x3
kernels, skip connections, BF16 weights and activations with FP32 accumulate --
that maps a residual to a correction of the Jacobi step.  It has no counterpart
in the reference, whose ``am.ai`` package is an unrelated placeholder
(src/am/ai/model.py:18-67).

The training set follows the 64x32x32 cantilever workload: residual/error pairs
harvested from the engine's own Jacobi-PCG solves at densities taken from SIMP
trajectories (iterations 1-80) of cantilevers clamped at x = 0 with three seeded
point loads of magnitude U(0.5, 1.5) in random unit directions on the top face;
Adam, lr 1e-3, batch 8, 20 epochs.

    python -m am_ml_suite_gb300.learned [out.npy]

trains the network on the GPU and writes its weights (BF16 bit patterns, the
precision the network computes in) to ``weights/precond_cantilever64.npy``.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

from . import _native as nat

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "precond_cantilever64.npy")

SHAPE = (64, 32, 32)
SIMP_ITERATIONS = 80
HARVEST_ITERS = (0, 16, 64, 256, 1024)  # PCG iteration counts whose (r_k, e_k) become samples
N_TRAJECTORIES = 10                      # 10 x 80 densities x 5 counts = 4000 pairs


def cantilever_loads(shape, rng):
    """Clamped x = 0 face; three point loads on the top face (k = nz) at seeded
    random nodes, magnitude U(0.5, 1.5), direction uniform on the sphere.
    Returns (F in the reference DOF order, constrained DOFs)."""
    nx, ny, nz = shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)

    def node(i, j, k):
        return (i * (ny + 1) + j) * (nz + 1) + k

    base = np.array([node(0, j, k) for j in range(ny + 1) for k in range(nz + 1)])
    fixed = (3 * base[:, None] + np.arange(3)).ravel()
    F = np.zeros(N)
    ij = rng.integers(0, [nx + 1, ny + 1], size=(3, 2))
    mag = rng.uniform(0.5, 1.5, size=3)
    d = rng.normal(size=(3, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    for (a, b), m, v in zip(ij, mag, d):
        F[3 * node(int(a), int(b), nz) + np.arange(3)] += m * v
    return F, fixed


def simp_config(max_iterations=SIMP_ITERATIONS, **kw):
    """C++-variant SIMP of the training trajectories: vf 0.3, rmin 1.5, move 0.2."""
    return nat.default_config(nat.VARIANT_CPP, volume_fraction=0.3, filter_radius=1.5, move_limit=0.2,
                              rho_min=0.01, E_min=1e-9, convergence_tol=0.0, max_iterations=max_iterations,
                              cg_tol=1e-6, **kw)


def trajectory_densities(shape, F, fixed, iterations):
    """Densities after each SIMP iteration in `iterations` (1-based) of one
    trajectory from the uniform density 0.3, solved with the multigrid solver
    (the densities, not the solver, are what the samples need).  Returns
    (problem, {iteration: density})."""
    p = nat.Problem(shape)
    p.set_loads([F], [fixed])
    p.simp_begin(simp_config(max(iterations), preconditioner=nat.PRECOND_MG), np.full(shape, 0.3))
    out = {}
    for it in range(1, max(iterations) + 1):
        p.simp_step()
        if it in iterations:
            out[it] = p.simp_density().copy()
    return p, out


def harvest(pre, n_trajectories=N_TRAJECTORIES, seed=4, shape=SHAPE, iters=HARVEST_ITERS, verbose=False):
    """Adds n_trajectories x SIMP_ITERATIONS x len(iters) samples to `pre`."""
    rng = np.random.default_rng(seed)
    cfg = nat.default_config(nat.VARIANT_CPP, rho_min=0.01, E_min=1e-9, cg_tol=1e-6)
    t0 = time.time()
    for t in range(n_trajectories):
        F, fixed = cantilever_loads(shape, rng)
        p, dens = trajectory_densities(shape, F, fixed, set(range(1, SIMP_ITERATIONS + 1)))
        for it in range(1, SIMP_ITERATIONS + 1):
            pre.harvest(p, cfg, dens[it], list(iters))
        p.close()
        if verbose:
            print(f"trajectory {t}: {pre.num_samples} samples, {time.time() - t0:.1f} s", flush=True)


def train(epochs=20, batch=8, lr=1e-3, loss=0, n_trajectories=N_TRAJECTORIES, seed=0, verbose=False):
    """Harvests the training set and trains a fresh network; returns
    (Preconditioner, per-epoch mean loss)."""
    cap = n_trajectories * SIMP_ITERATIONS * len(HARVEST_ITERS)
    pre = nat.Preconditioner(seed=seed, capacity=cap)
    harvest(pre, n_trajectories=n_trajectories, verbose=verbose)
    losses = pre.train(epochs=epochs, batch=batch, lr=lr, loss=loss, verbose=int(verbose))
    return pre, losses


def to_bf16_bits(w):
    """FP32 -> BF16 bit patterns (round to nearest even)."""
    u = np.ascontiguousarray(w, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def from_bf16_bits(b):
    return (np.ascontiguousarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def save_weights(pre, path=WEIGHTS):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.save(path, to_bf16_bits(pre.get_params()))


def load_weights(path=WEIGHTS):
    """FP32 weights (exact BF16 values) of the trained network, or None."""
    if not os.path.exists(path):
        return None
    return from_bf16_bits(np.load(path))


if __name__ == "__main__":
    nat.load()
    out = sys.argv[1] if len(sys.argv) > 1 else WEIGHTS
    pre, losses = train(verbose=True)
    save_weights(pre, out)
    print("epoch losses", [round(float(v), 5) for v in losses])
