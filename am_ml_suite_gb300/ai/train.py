"""Training set and training of the density-predicting U-Net.

    python -m am_ml_suite_gb300.ai.train out.npz [n_train] [f0] [epochs] [channels: 4 or 7]

The samples are BRK-A-01 brackets at 5 mm (24 x 12 x 16 elements, the resolution of
the reference's recorded run data/brk_a_01) with the eyelet load of static case 1
turned to a random direction within 60 degrees of -z, each optimised by this
engine's own SIMP (Python variant, volume fraction 0.3, filter radius 1.5, 40
iterations).  The network learns encoding -> final density on the design cells;
held-out problems report IoU, compliance error and volume error against their
SIMP solutions."""
from __future__ import annotations

import json
import sys
import time

import numpy as np

from .. import _native as nat
from ..core import LoadCase, create_bracket_domain, create_brk_a_01_static_case_1
from .inference import AIOptimizer
from .model import TopOptUNet, _pad8

RESOLUTION_MM = 5.0
VOLUME_FRACTION = 0.3
FILTER_RADIUS = 1.5
SIMP_ITERATIONS = 40


def random_case(domain_shape, rng) -> LoadCase:
    """Static case 1's ring and constraints with the 15 kN load turned by up to
    60 degrees from -z in a random azimuth."""
    lc = create_brk_a_01_static_case_1(domain_shape, RESOLUTION_MM)
    th, ph = np.radians(60.0) * np.sqrt(rng.uniform()), rng.uniform(0, 2 * np.pi)
    lc.distributed_loads[0].total_force = 15000.0 * np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph),
                                                              -np.cos(th)])
    return lc


def make_samples(n: int, seed: int, verbose=False, channels=4):
    from ..numerical.fem import MaterialProperties
    from ..numerical.topopt import SIMPOptimizer, SIMPParams

    rng = np.random.default_rng(seed)
    dom = create_bracket_domain(resolution_mm=RESOLUTION_MM)
    enc = AIOptimizer()
    prm = SIMPParams(volume_fraction=VOLUME_FRACTION, filter_radius=FILTER_RADIUS, max_iterations=SIMP_ITERATIONS,
                     convergence_tol=0.0, precision=nat.PREC_MIXED, cg_tol=1e-6)
    X, T, cases = [], [], []
    t0 = time.time()
    for i in range(n):
        lc = random_case(dom.shape, rng)
        res = SIMPOptimizer(dom, [lc], MaterialProperties(E=1.0, nu=0.3), prm, verbose=False).run()
        X.append(enc.encode_problem(dom, [lc], channels=channels))
        T.append(res.density)
        cases.append(lc)
        if verbose and (i + 1) % 16 == 0:
            print(f"{i + 1} samples, {time.time() - t0:.1f} s", flush=True)
    return dom, np.stack(X), np.stack(T), cases


def padded(dom, X, T):
    nx, ny, nz = dom.shape
    S = X.shape[0]
    g = (_pad8(nx), _pad8(ny), _pad8(nz))
    x = np.zeros((S,) + g + (X.shape[1],), np.float32)
    x[:, :nx, :ny, :nz] = np.moveaxis(X, 1, -1)
    t = np.zeros((S,) + g, np.float32)
    t[:, :nx, :ny, :nz] = T
    m = np.zeros((S,) + g, np.uint8)
    m[:, :nx, :ny, :nz] = (dom.grid == 0)
    return x, t, m


def train(n_train=160, n_test=16, f0=32, epochs=60, batch=8, lr=1e-3, seed=0, verbose=False, channels=4):
    dom, X, T, cases = make_samples(n_train + n_test, seed, verbose, channels)
    x, t, m = padded(dom, X[:n_train], T[:n_train])
    model = TopOptUNet(channels, 1, (f0, 2 * f0, 4 * f0, 8 * f0), seed=seed)
    model.net.set_data(x, t, m)
    t0 = time.time()
    losses = model.net.train(epochs=epochs, batch=batch, lr=lr, seed=seed, verbose=int(verbose))
    train_s = time.time() - t0
    model.meta = {"volume_fraction": VOLUME_FRACTION, "filter_radius": FILTER_RADIUS,
                  "simp_iterations": SIMP_ITERATIONS, "resolution_mm": RESOLUTION_MM}
    ai = AIOptimizer()
    ai.model = model
    held = []
    for i in range(n_train, n_train + n_test):
        held.append(ai.validate_against_numerical(dom, [cases[i]], numerical_density=T[i]))
    summary = {"n_train": n_train, "n_test": n_test, "f0": f0, "channels": channels, "epochs": epochs,
               "train_s": train_s,
               "mse_first": float(losses[0]), "mse_last": float(losses[-1]),
               "held_out_iou_mean": float(np.mean([h["iou"] for h in held])),
               "held_out_compliance_error_mean": float(np.mean([h["compliance_error"] for h in held])),
               "held_out_volume_error_mean": float(np.mean([h["volume_error"] for h in held]))}
    return model, summary, held


if __name__ == "__main__":
    nat.load()
    out = sys.argv[1] if len(sys.argv) > 1 else "topopt_unet_brk5mm.npz"
    n = int(sys.argv[2]) if len(sys.argv) > 2 else 160
    f0 = int(sys.argv[3]) if len(sys.argv) > 3 else 32
    ep = int(sys.argv[4]) if len(sys.argv) > 4 else 60
    ch = int(sys.argv[5]) if len(sys.argv) > 5 else 4
    model, summary, held = train(n_train=n, f0=f0, epochs=ep, verbose=True, channels=ch)
    model.save(out)
    print(json.dumps(summary))
