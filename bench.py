#!/usr/bin/env python
"""SIMP iterations/s and PCG solve ms at relative residual 1e-6 on GB300:
learned vs Jacobi PCG.

Workload (default ``cantilever256``): the 256x128x128 cantilever -- 4,194,304
hex8 elements, 12,830,211 DOF, E0 = 1, nu = 0.3, E_min = 1e-9, p = 3, vf = 0.25,
rmin = 2.5 cone sensitivity filter, move 0.2, clamped x = 0 face, a -z load of
total magnitude 1 spread over the 33x33 nodes of the central 32x32 element patch
of the x = 256 face.  ``bracket192`` is the 192x96x96 bracket (void cylinder,
four passive bolt-pad columns, 3 seeded point loads); ``batch256`` the 256
seeded cantilevers of uneven sizes solved together.

One step = one SIMP iteration (solve, sensitivities, filter, OC update).  The
solver arms (``--arms``; jacobi, learned, mg) each time SIMP steps 1..K of a
fresh problem from the same initial density after W warm-up steps on a
throwaway problem; every solve is accepted on its FP64 residual at 1e-6.
``value``: iterations/s of the primary arm (Jacobi PCG, the method the reference
arm runs on the CPU), timed with CUDA events on the library's stream;
``arms`` holds every arm's rate, PCG solve ms, iterations and agreement with the
Jacobi arm.  ``e2e``: the primary arm through the public C ABI from pinned host
buffers (loads, network weights, am_simp_run for K iterations, density read
back).  The working set of a step (solver vectors + element arrays, > 1 GB)
exceeds the 129 MB L2; the roofline probes flush L2 before each launch.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (shape, rmin, vf, description)
    "bracket192": ((192, 96, 96), 2.0, 0.3, "192x96x96 bracket, void cylinder r=16 through y, 4 bolt-pad columns, "
                                            "3 seeded point loads on the top face"),
    "cantilever256": ((256, 128, 128), 2.5, 0.25, "256x128x128 cantilever, -z load 1 on the central 32x32 patch of x=max"),
    "cantilever48": ((48, 24, 12), 1.5, 0.3, "48x24x12 cantilever, -z unit line load along x=48, z=6"),
}


def build_workload(name):
    shape, rmin, vf, desc = WORKLOADS[name]
    nx, ny, nz = shape
    N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
    node = lambda i, j, k: (i * (ny + 1) + j) * (nz + 1) + k  # noqa: E731
    base = np.array([node(0, j, k) for j in range(ny + 1) for k in range(nz + 1)])
    fixed = (3 * base[:, None] + np.arange(3)).ravel()
    F = np.zeros(N)
    rho0 = np.full(shape, vf)
    if name == "bracket192":
        i = np.arange(nx)[:, None, None] + 0.5
        k = np.arange(nz)[None, None, :] + 0.5
        cyl = (i - nx / 2) ** 2 + (k - nz / 2) ** 2 <= 16.0 ** 2
        rho0 = np.where(np.broadcast_to(cyl, shape), 0.0, rho0)
        for x0 in (6, nx - 12):
            for y0 in (6, ny - 12):
                rho0[x0:x0 + 6, y0:y0 + 6, :] = 1.0
        rng = np.random.default_rng(2)
        ij = rng.integers(0, [nx + 1, ny + 1], size=(3, 2))
        mag = rng.uniform(0.5, 1.5, size=3)
        d = rng.normal(size=(3, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        for (a, b), m, v in zip(ij, mag, d):
            F[3 * node(int(a), int(b), nz) + np.arange(3)] += m * v
    elif name == "cantilever256":
        c0j, c0k = ny // 2 - 16, nz // 2 - 16
        nodes = [node(nx, j, k) for j in range(c0j, c0j + 33) for k in range(c0k, c0k + 33)]
        F[3 * np.array(nodes) + 2] = -1.0 / len(nodes)
    else:
        line = [node(nx, j, nz // 2) for j in range(ny + 1)]
        F[3 * np.array(line) + 2] = -1.0 / len(line)
    return dict(shape=shape, rmin=rmin, vf=vf, F=F, fixed=fixed, rho0=rho0, desc=desc)


def build_batch256(n=256, seed=3):
    """256 independent cantilevers: nelx in U{32..96}, nely in U{16..48}, nelz in
    U{8..48}, vf ~ U(0.2, 0.5), rmin ~ U(1.2, 2.5), clamped x = 0 face, one unit load
    at a random node of the x = nelx face in a random unit direction."""
    rng = np.random.default_rng(seed)
    probs = []
    for _ in range(n):
        nx, ny, nz = int(rng.integers(32, 97)), int(rng.integers(16, 49)), int(rng.integers(8, 49))
        vf, rmin = float(rng.uniform(0.2, 0.5)), float(rng.uniform(1.2, 2.5))
        N = 3 * (nx + 1) * (ny + 1) * (nz + 1)
        base = np.array([j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)])
        fixed = (3 * base[:, None] + np.arange(3)).ravel()
        j, k = int(rng.integers(0, ny + 1)), int(rng.integers(0, nz + 1))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        F = np.zeros(N)
        node = nx * (ny + 1) * (nz + 1) + j * (nz + 1) + k
        F[3 * node:3 * node + 3] = d
        probs.append(dict(shape=(nx, ny, nz), vf=vf, rmin=rmin, F=F, fixed=fixed))
    return probs


def batch_config(nat, pr, max_iterations=50):
    return nat.default_config(nat.VARIANT_CPP, volume_fraction=pr["vf"], filter_radius=pr["rmin"], move_limit=0.2,
                              rho_min=0.01, E_min=1e-9, convergence_tol=0.0, max_iterations=max_iterations,
                              cg_tol=1e-6, cg_max_iterations=200000)


def run_batch(args, nat, world, rank, emit=True):
    """Batched workload: one step = one SIMP iteration of every problem.  Prints
    the JSON line when `emit`; returns it."""
    import torch

    probs = build_batch256()
    if world > 1:
        # one share of the problems per rank, no exchange step
        from am_ml_suite_gb300.sharding import partition, problem_cost

        mine = partition([problem_cost(pr["shape"]) for pr in probs], world)[rank]
        probs = [probs[i] for i in mine]
    shapes = [pr["shape"] for pr in probs]
    nel = sum(a * b * c for a, b, c in shapes)
    nodes = sum((a + 1) * (b + 1) * (c + 1) for a, b, c in shapes)
    b = nat.Batch(shapes)
    b.set_loads([pr["F"] for pr in probs], [pr["fixed"] for pr in probs])
    cfgs = [batch_config(nat, pr) for pr in probs]
    b.simp_begin(cfgs)
    plan = b.autotune(reps=5)
    b.set_staged(args.batch_ku == "staged")
    b.set_device_loop(not getattr(args, "host_loop", False))
    for _ in range(args.warmup):
        b.simp_step()
    its0 = b.pcg_iterations.copy()
    stream = torch.cuda.ExternalStream(b.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stepped = 0
    torch.cuda.synchronize()
    l0 = nat.launch_count()
    with ClockSampler(0) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            c, _, _, _ = b.simp_step()
            stepped += int(np.isfinite(c).sum())
        ev1.record(stream)
        torch.cuda.synchronize()
    l1 = nat.launch_count()
    elapsed = ev0.elapsed_time(ev1) * 1e-3
    its_per_step = (b.pcg_iterations - its0) / max(args.steps, 1)
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([elapsed, float(stepped)], dtype=torch.float64)
        tmax = t.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        elapsed, stepped = float(tmax[0]), int(t[1])
    value = stepped / elapsed
    # roofline: the batched FP32 PCG K*u the solve runs (p = D^-1 r + beta p, q =
    # mask(K p), p.q: reads p, r 12 B per node each, D^-1 4 B, constraint bits 1 B,
    # scale 4 B per element; writes p, q 12 B per node each), every problem active
    ku_ms = b.bench_ku(reps=10)
    alg = 53 * nodes + 4 * nel
    peak, peak_kind = measured_peaks()
    achieved = alg / (ku_ms * 1e-3) / 1e9
    b.close()
    e2e = None
    if not args.no_e2e:
        total = args.warmup + args.steps
        q = nat.Batch(shapes)
        if world > 1:
            dist.barrier()
        q.set_staged(args.batch_ku == "staged")
        q.set_device_loop(not getattr(args, "host_loop", False))
        te0 = time.perf_counter()
        q.set_loads([pr["F"] for pr in probs], [pr["fixed"] for pr in probs])
        out = q.simp_run([batch_config(nat, pr, total) for pr in probs])
        te1 = time.perf_counter()
        q.close()
        wall, done = te1 - te0, float(len(probs) * total)
        if world > 1:
            t = torch.tensor([wall, done], dtype=torch.float64)
            tmax = t.clone()
            dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
            wall, done = float(tmax[0]), float(t[1])
        h2d = sum(pr["F"].nbytes + pr["fixed"].nbytes for pr in probs)
        d2h = sum(o["density"].nbytes for o in out)
        e2e = {"value": done / wall, "unit": "problem-iterations/s",
               "h2d_bytes_per_step": int(h2d / total), "d2h_bytes_per_step": int(d2h / total),
               "iterations": total, "wall_s": wall,
               "note": "am_batch_set_loads + am_batch_simp_run from host buffers (plan of the default autotuner "
                       "state, cold start included)"}
    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        import oracle as O

        # the CPU restatement on a bounded sample: 4 problems, CSR assembly + 10
        # Jacobi-PCG iterations each, extrapolated per problem with the GPU's PCG
        # iteration count, scaled by element count to all problems
        t_tot, nel_s = 0.0, 0
        t_iter_per_el, t_fixed_per_el = 0.0, 0.0
        for pr in probs[:4]:
            prm = O.make_params(volume_fraction=pr["vf"], filter_radius=pr["rmin"], move_limit=0.2, rho_min=0.01,
                                E_min=1e-9)
            nx, ny, nz = pr["shape"]
            times, threads = O.baseline_sample(pr["shape"], prm, np.full(nx * ny * nz, pr["vf"]), pr["F"],
                                               pr["fixed"], 10)
            ne = nx * ny * nz
            t_iter_per_el += times["pcg_iteration"]
            t_fixed_per_el += (times["assembly"] + times["pcg_setup"] + times["sensitivities"] + times["filter"] +
                               times["oc"])
            nel_s += ne
        t_iter_per_el /= nel_s
        t_fixed_per_el /= nel_s
        for p, (nx, ny, nz) in enumerate(shapes):
            ne = nx * ny * nz
            t_tot += ne * (t_fixed_per_el + its_per_step[p] * t_iter_per_el)
        cpu = {"value": len(probs) / t_tot, "unit": "problem-iterations/s", "cores": threads, "kind": "port",
               "sample": ("CPU restatement (CSR + Jacobi PCG, OpenMP) timed on 4 of the 256 problems: assembly, "
                          "10 PCG iterations, sensitivities, filter, OC; per-element rates extrapolated to every "
                          "problem with its GPU PCG iteration count per step")}
    if rank == 0:
        line = {
            "metric": "batched SIMP problem-iterations/s @ rel-res 1e-6 (Jacobi PCG)",
            "value": value, "unit": "problem-iterations/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": "batch256", "problems": 256, "problems_rank0": len(probs), "elements_rank0": nel,
                       "nodes_rank0": nodes,
                       "description": build_batch256.__doc__.strip().replace("\n", " "), "cg_tol": 1e-6,
                       "pcg_ku": args.batch_ku,
                       "autotuned_plan": plan, "l2": "working set per step > 129 MB L2",
                       "parallelism": f"problems sharded over {world} ranks (LPT by cost)" if world > 1 else "1 GPU"},
            "pcg_iterations_per_problem_step": float(np.mean(its_per_step)),
            "roofline": {"bound": "hbm",
                         "kernel": ("b_ku3_kernel (batched tensor-copy staged FP32 PCG K*u, 28 x 15-node tiles)"
                                    if args.batch_ku == "staged" else
                                    "b_ku2_kernel<8|4,KU_PCG> (batched warp-row FP32 PCG K*u, tile height per problem)"
                                    if plan["warps"] == 0 else
                                    f"b_ku2_kernel<{plan['warps']},KU_PCG> (batched warp-row FP32 PCG K*u)"),
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": None, "algorithmic_bytes": alg, "avg_ms": ku_ms},
            "gpu_launches": int(l1 - l0), "clocks": clk.summary(), "e2e": e2e, "cpu_baseline": cpu,
        }
        if emit:
            print(json.dumps(line))
        return line
    return None


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([v.strip() for v in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[3:7]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f).get("bf16_tflops", 1900.0))
    return 1900.0


def ku_traffic_per_launch(W, nodes, elements):
    """DRAM bytes per launch of the fused FP32 PCG K*u from the committed ncu
    captures: the capture of this workload's grid if there is one, else the
    largest capture scaled by nodes; None without captures."""
    p = os.path.join(ROOT, "profiles", "ku_pcg_fp32_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        caps = json.load(f)["captures"]
    for c in caps.values():
        if c["nodes"] == nodes and c["elements"] == elements:
            return float(c["dram_bytes_per_launch"])
    c = max(caps.values(), key=lambda c: c["nodes"])
    return c["dram_bytes_per_launch"] * nodes / c["nodes"]


def cpu_baseline(W, steps_gpu_its, pcg_iters_sample=20):
    """The CPU restatement (oracle, OpenMP on all host cores): CSR assembly,
    `pcg_iters_sample` Jacobi-PCG iterations, sensitivities, filter, OC of one
    C++-variant SIMP iteration on the full workload.  The iteration rate is
    extrapolated with the PCG iteration count per SIMP iteration of the GPU run
    (same method, same tolerance)."""
    import oracle as O

    prm = O.make_params(volume_fraction=W["vf"], filter_radius=W["rmin"], move_limit=0.2, rho_min=0.01,
                        E_min=1e-9)
    t0 = time.time()
    times, threads = O.baseline_sample(W["shape"], prm, W["rho0"].ravel(), W["F"], W["fixed"], pcg_iters_sample)
    wall = time.time() - t0
    per_iter = (times["assembly"] + times["pcg_setup"] + steps_gpu_its * times["pcg_iteration"] +
                times["sensitivities"] + times["filter"] + times["oc"])
    return {"value": 1.0 / per_iter, "unit": "SIMP iters/s", "cores": threads, "kind": "port",
            "sample": (f"one C++-variant SIMP iteration of the FP64 CPU restatement on the full workload: "
                       f"CSR assembly + {pcg_iters_sample} Jacobi-PCG iterations timed (s/PCG-it "
                       f"{times['pcg_iteration']:.4f}), extrapolated to {steps_gpu_its:.0f} PCG iterations per SIMP "
                       f"iteration; sample wall {wall:.1f} s"),
            "phases_s": times}




METRIC = "SIMP iters/s and PCG solve ms @ rel-res 1e-6: learned vs Jacobi PCG, 1×GB300"

# Solver arms of one bench line.  jacobi: one FP32 Jacobi-PCG sequence with FP64
# residual replacement; learned: the FP64 flexible CG preconditioned by the trained
# conv3d network (Jacobi PCG its fallback on stagnation); mg: the multigrid V-cycle
# in the FP64 flexible CG.  Every solve of every arm is accepted on its FP64
# residual at rel-res 1e-6.
ARM_DESC = {
    "jacobi": "FP32 Jacobi PCG with FP64 residual replacement (mixed precision)",
    "learned": "FP64 flexible CG preconditioned by the trained conv3d encoder-decoder, FP32 Jacobi-PCG refinement",
    "mg": "FP64 flexible CG preconditioned by the FP32 multigrid V-cycle",
}
_inner_tol = 0.0
_mg_deflation = 1
_mixed_solver = "reliable"
_host_loop = False
MIXED_SOLVER = {"reliable": 0, "flexible": 1}


def simp_config(nat, W, max_iterations=100, arm="jacobi"):
    c = nat.default_config(nat.VARIANT_CPP, volume_fraction=W["vf"], filter_radius=W["rmin"], move_limit=0.2,
                           rho_min=0.01, E_min=1e-9, convergence_tol=0.0, max_iterations=max_iterations,
                           precision=nat.PREC_MIXED, cg_tol=1e-6, warm_start=1, inner_tol=_inner_tol,
                           cg_max_iterations=200000, mixed_solver=MIXED_SOLVER[_mixed_solver],
                           mg_deflation=_mg_deflation)
    if arm == "learned":
        c.preconditioner = nat.PRECOND_LEARNED
        c.mixed_solver = nat.MIXED_FLEXIBLE
    elif arm == "mg":
        c.preconditioner = nat.PRECOND_MG
    return c


def reference_sample(W, n_pcg, pcg_iters_sample=10):
    """Projected seconds of one SIMP iteration of the CPU restatement: one bounded
    sample (CSR assembly, `pcg_iters_sample` Jacobi-PCG iterations, sensitivities,
    filter, OC on the full workload) with the PCG phase scaled to n_pcg iterations."""
    import oracle as O

    prm = O.make_params(volume_fraction=W["vf"], filter_radius=W["rmin"], move_limit=0.2, rho_min=0.01,
                        E_min=1e-9)
    times, threads = O.baseline_sample(W["shape"], prm, W["rho0"].ravel(), W["F"], W["fixed"], pcg_iters_sample)
    s = (times["assembly"] + times["pcg_setup"] + n_pcg * times["pcg_iteration"] + times["sensitivities"] +
         times["filter"] + times["oc"])
    return s, times, threads


def reference_whole_iteration(W):
    """One whole C++-variant SIMP iteration (the first, from the workload's initial
    density) of the CPU restatement: CSR assembly, FP64 Jacobi PCG from zero to
    rel-res 1e-6, sensitivities, filter, OC.  Returns (seconds, PCG iterations)."""
    import oracle as O

    prm = O.make_params(volume_fraction=W["vf"], filter_radius=W["rmin"], move_limit=0.2, rho_min=0.01,
                        E_min=1e-9, convergence_tol=0.0, max_iterations=1, cg_tol=1e-6, cg_maxit=200000,
                        warm_start=0, use_csr=1)
    t0 = time.perf_counter()
    r = O.simp_cpp(W["shape"], 1.0, 1.0, 0.3, prm, W["rho0"], W["F"], W["fixed"])
    return time.perf_counter() - t0, int(r["cg_iters"][0])


def run_reference(args, W):
    """The reference arm: the CPU restatement of the reference's C++ SIMP loop
    (topology_optimizer.cpp:294-520 with Jacobi PCG, the preconditioner the metric
    names) on all host cores.  SIMP iteration 1 is run whole, which gives the PCG
    iteration count of a solve from zero to rel-res 1e-6; each step is then one
    bounded sample projected with that count (the reference solves every
    iteration from zero, linear_solver.cpp:136-155)."""
    t_whole, n_pcg = reference_whole_iteration(W)
    vals = []
    sample = None
    for _ in range(args.warmup):
        reference_sample(W, n_pcg, 2)
    t0 = time.time()
    for _ in range(args.steps):
        s, times, threads = reference_sample(W, n_pcg)
        vals.append(1.0 / s)
        sample = (times, threads)
    wall = time.time() - t0
    value = statistics.median(vals)
    times, threads = sample
    desc = (f"SIMP iteration 1 run whole on the FP64 CPU restatement ({n_pcg} Jacobi-PCG iterations to rel-res "
            f"1e-6, {t_whole:.1f} s); each step a bounded sample (CSR assembly, 10 PCG iterations, sensitivities, "
            f"filter, OC on the full workload) with the PCG phase projected to {n_pcg} iterations")
    line = {"metric": METRIC, "value": value, "unit": "SIMP iters/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "shape": list(W["shape"]), "description": W["desc"],
                       "preconditioner": "jacobi", "cg_tol": 1e-6},
            "projected": True, "pcg_iterations_per_solve": n_pcg, "pcg_solve_ms": 1000.0 * n_pcg *
            times["pcg_iteration"], "whole_iteration_1": {"s": t_whole, "pcg_iterations": n_pcg},
            "cpu_baseline": {"value": value, "unit": "SIMP iters/s", "cores": threads, "kind": "port",
                             "sample": desc, "phases_s": times},
            "e2e": {"value": value, "unit": "SIMP iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))


def time_arm(nat, torch, W, arm, steps, pre=None, keep=False):
    """SIMP steps 1..`steps` of a fresh problem with the arm's solver, timed with
    CUDA events on the library's stream (allocation and set-up of the fresh state
    included).  Returns the per-step results and, if keep, the open problem."""
    p = nat.Problem(W["shape"], 1.0, 1.0, 0.3)
    p.set_device_loop(not _host_loop)
    p.set_loads([W["F"]], [W["fixed"]])
    if pre is not None:
        p.set_preconditioner(pre)
    cfg = simp_config(nat, W, max_iterations=max(steps, 1), arm=arm)
    stream = torch.cuda.ExternalStream(p.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = nat.launch_count()
    ev0.record(stream)
    p.simp_begin(cfg, W["rho0"])
    res = [p.simp_step() for _ in range(steps)]
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = nat.launch_count() - l0
    s = ev0.elapsed_time(ev1) * 1e-3
    rho = p.simp_density()
    out = {"s": s, "value": steps / s, "ms_per_step": 1000.0 * s / steps,
           "pcg_solve_ms": 1000.0 * statistics.mean(r.solve_time_s for r in res),
           "pcg_iterations_per_solve": statistics.mean(r.solver_iterations for r in res),
           "outer_iterations_per_solve": statistics.mean(r.solver_outer_iterations for r in res),
           "learned_applications_per_solve": statistics.mean(r.solver_learned_applications for r in res),
           "solver_residual_max": max(r.solver_residual for r in res),
           "compliance": [r.compliance for r in res], "gpu_launches": int(launches), "density": rho}
    if keep:
        return out, p
    p.close()
    return out, None


def arm_summary(a, ref=None):
    keys = ["value", "ms_per_step", "pcg_solve_ms", "pcg_iterations_per_solve", "outer_iterations_per_solve",
            "learned_applications_per_solve", "solver_residual_max", "gpu_launches"]
    d = {k: a[k] for k in keys}
    d["compliance_last"] = a["compliance"][-1]
    if ref is not None and ref is not a:
        c, cr = np.array(a["compliance"]), np.array(ref["compliance"])
        d["compliance_rel_diff_vs_jacobi_max"] = float(np.max(np.abs(c - cr) / np.abs(cr)))
        d["density_max_abs_diff_vs_jacobi"] = float(np.max(np.abs(a["density"] - ref["density"])))
    return d


def e2e_run(nat, torch, W, arm, iterations, pre_weights=None):
    """The same metric through the C ABI from pinned host buffers: problem loads,
    (the network's weights,) am_simp_run for `iterations` SIMP iterations and the
    density read back, all inside the timed region."""
    def pinned(a, dtype):
        t = torch.empty(a.size, dtype=dtype, pin_memory=True)
        arr = t.numpy()
        arr[:] = a.ravel()
        return arr, t

    nel = int(np.prod(W["shape"]))
    F_h, _tF = pinned(W["F"], torch.float64)
    fx_h, _tx = pinned(W["fixed"].astype(np.int64), torch.int64)
    r0_h, _tr = pinned(W["rho0"], torch.float64)
    out_h, _to = pinned(np.zeros(nel), torch.float64)
    w_h = None
    if pre_weights is not None:
        w_h, _tw = pinned(pre_weights, torch.float32)
    cfg = simp_config(nat, W, max_iterations=iterations, arm=arm)
    q = nat.Problem(W["shape"], 1.0, 1.0, 0.3)
    q.set_device_loop(not _host_loop)
    pre = nat.Preconditioner(seed=0, capacity=0) if w_h is not None else None
    torch.cuda.synchronize()
    te0 = time.perf_counter()
    q.set_loads([F_h], [fx_h])
    if pre is not None:
        pre.set_params(w_h)
        q.set_preconditioner(pre)
    r = q.simp_run(cfg, r0_h)
    out_h[:] = r["density"]
    te1 = time.perf_counter()
    q.close()
    if pre is not None:
        pre.close()
    h2d = F_h.nbytes + fx_h.nbytes + r0_h.nbytes + (0 if w_h is None else w_h.nbytes)
    d2h = out_h.nbytes + 3 * 8 * iterations
    return {"value": iterations / (te1 - te0), "unit": "SIMP iters/s",
            "h2d_bytes_per_step": int(h2d / iterations), "d2h_bytes_per_step": int(d2h / iterations),
            "iterations": iterations, "wall_s": te1 - te0, "arm": arm,
            "note": "am_problem_set_loads" + (" + am_precond_set_params" if w_h is not None else "") +
                    " + am_simp_run from pinned host buffers, density read back; a fresh problem (SIMP steps 1..K)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cantilever256", choices=sorted(WORKLOADS) + ["batch256"])
    ap.add_argument("--arms", default="jacobi,learned,mg",
                    help="comma-separated solver arms timed from the same start: jacobi, learned, mg")
    ap.add_argument("--primary", default="jacobi",
                    help="the arm whose rate is `value` (default jacobi: the method the reference arm runs on the "
                         "CPU, so the two lines compare like for like; the other arms are in `arms`)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="skip the short runs of the bracket (config 2) and the 256-problem batch (config 3) "
                         "reported in `other_workloads`")
    ap.add_argument("--probe", choices=["ku", "resid", "update", "conv", "ku2", "ku3s3", "ku3tile", "ku3b4", "resid_df",
                                        "update_even", "update_odd",
                                        "filter", "oc", "vcycle", "vcycle_defl"],
                    help="only time `reps` launches of one kernel after set-up (bounded command for ncu)")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--compare-mg", action="store_true",
                    help="time --steps SIMP iterations with the Jacobi and the multigrid mixed-precision solvers "
                         "from the same start and report the ratio and the compliance / density agreement")
    ap.add_argument("--compare-fp64", action="store_true",
                    help="time --steps SIMP iterations of --arms' first arm in mixed precision and of FP64 plain "
                         "Jacobi PCG from the same start and report the ratio and the agreement")
    ap.add_argument("--inner-tol", type=float, default=0.0,
                    help="mixed precision: residual reduction between FP64 replacements / per inner solve "
                         "(0: the solver's default, 0.1 reliable / 0.01 flexible)")
    ap.add_argument("--mg-deflation", type=int, default=1, choices=[0, 1],
                    help="multigrid: balance the V-cycle with the rigid-body modes of the passive solid "
                         "inclusions (1, the default) or not (0)")
    ap.add_argument("--mixed-solver", default="reliable", choices=sorted(MIXED_SOLVER),
                    help="jacobi arm: one FP32 PCG with FP64 residual replacement (reliable) or the FP64 "
                         "flexible CG over FP32 inner solves (flexible)")
    ap.add_argument("--batch-ku", default="staged", choices=["staged", "warp-row"],
                    help="batch256: the FP32 PCG K*u kernel (tensor-copy staged, or warp-row with the autotuned plan)")
    ap.add_argument("--host-loop", action="store_true",
                    help="drive every inner PCG solve chunk by chunk from the host instead of the device-side "
                         "graph loop (same results; the measurement baseline of the loop)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    global _mixed_solver, _inner_tol, _mg_deflation, _host_loop
    _host_loop = args.host_loop
    _mixed_solver = args.mixed_solver
    _mg_deflation = args.mg_deflation
    _inner_tol = args.inner_tol
    arms = [a for a in args.arms.split(",") if a]
    for a in arms:
        if a not in ARM_DESC:
            raise SystemExit(f"unknown arm {a}")

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # one independent replica per GPU (the single-domain path does not shard):
        # pin this process to its GPU before the CUDA runtime starts
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local_rank)
        import torch.distributed as dist

        dist.init_process_group("gloo")
    W = build_workload(args.workload) if args.workload != "batch256" else None

    if args.impl == "reference":
        if args.workload == "batch256":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the batched workload has no reference arm; "
                                  "its CPU baseline is reported in the GB300 line"}))
            return
        if rank == 0:
            run_reference(args, W)
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
            dist.destroy_process_group()
        return

    from am_ml_suite_gb300 import _build, _native as nat
    from am_ml_suite_gb300 import learned

    _build.build()
    nat.load()
    if not nat.is_available():
        raise SystemExit("no CUDA device: the GB300 arm needs a GPU")
    if args.workload == "batch256":
        run_batch(args, nat, world, rank)
        return
    import torch

    torch.cuda.init()
    shape = W["shape"]

    weights = learned.load_weights() if "learned" in arms else None
    pre = None
    if weights is not None:
        pre = nat.Preconditioner(seed=0, capacity=0)
        pre.set_params(weights)
    elif "learned" in arms:
        arms.remove("learned")

    if args.compare_mg or args.compare_fp64:
        if args.compare_mg:
            pairs = [("jacobi", "jacobi", nat.PREC_MIXED), ("mg", "mg", nat.PREC_MIXED)]
        else:
            pairs = [(arms[0], arms[0], nat.PREC_MIXED), ("fp64", "jacobi", nat.PREC_FP64)]
        out = {}
        for name, arm, prec in pairs:
            p = nat.Problem(shape, 1.0, 1.0, 0.3)
            p.set_loads([W["F"]], [W["fixed"]])
            if arm == "learned":
                p.set_preconditioner(pre)
            c = simp_config(nat, W, max_iterations=args.steps, arm=arm)
            c.precision = prec
            p.simp_begin(c, W["rho0"])
            st = torch.cuda.ExternalStream(p.stream())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            res = [p.simp_step() for _ in range(args.steps)]
            e1.record(st)
            torch.cuda.synchronize()
            out[name] = dict(s=e0.elapsed_time(e1) * 1e-3, comp=np.array([r.compliance for r in res]),
                             its=[r.solver_iterations for r in res], res=max(r.solver_residual for r in res),
                             rho=p.simp_density())
            p.close()
        (na, a), (nb, b) = list(out.items())
        rel = np.abs(a["comp"] - b["comp"]) / np.abs(b["comp"])
        print(json.dumps({
            "compare": f"{na} vs {nb}", "workload": args.workload, "steps": args.steps,
            f"{na}_s_per_step": a["s"] / args.steps, f"{nb}_s_per_step": b["s"] / args.steps,
            "speedup": b["s"] / a["s"] if na != "jacobi" or nb == "fp64" else a["s"] / b["s"],
            "compliance_rel_diff_max": float(rel.max()), "compliance_rel_diff_final": float(rel[-1]),
            "compliance_final": float(b["comp"][-1]),
            "density_max_abs_diff": float(np.max(np.abs(a["rho"] - b["rho"]))),
            f"pcg_iterations_{na}": a["its"], f"pcg_iterations_{nb}": b["its"],
            f"compliance_{na}": a["comp"].tolist(), f"compliance_{nb}": b["comp"].tolist(),
            "mg_deflation": _mg_deflation, "residual_max": max(a["res"], b["res"])}))
        return

    if args.probe == "conv":
        # forward passes of the learned preconditioner on this workload's node grid
        pc = nat.Preconditioner(seed=0, capacity=0)
        nx, ny, nz = shape
        g = [(v + 1 + 7) // 8 * 8 for v in (nz, ny, nx)]
        ms, flops = pc.bench_forward(1, g[0], g[1], g[2], reps=args.reps)
        peak = measured_bf16_peak()
        tf = flops / (ms * 1e-3) / 1e12
        print(json.dumps({"probe": "conv", "workload": args.workload, "grid_zyx": g, "reps": args.reps,
                          "ms_per_forward": ms, "tflops": tf, "bf16_peak_tflops": peak, "frac": tf / peak}))
        return

    if args.probe:
        # set-up only, then `reps` launches of one kernel (L2 flushed before each)
        p = nat.Problem(shape, 1.0, 1.0, 0.3)
        p.set_loads([W["F"]], [W["fixed"]])
        p.simp_begin(simp_config(nat, W), W["rho0"])
        which = {"ku": 0, "resid": 1, "update": 2, "ku2": 4, "ku3s3": 5, "update_even": 6, "update_odd": 7,
                 "filter": 8, "oc": 9, "vcycle": 10, "vcycle_defl": 11, "ku3tile": 12, "ku3b4": 13, "resid_df": 14}[args.probe]
        if which in (8, 9):
            p.simp_step()  # the filter and OC probes time the state a SIMP step leaves
        avg, mn = p.bench_kernel(which, reps=args.reps, flush_l2=True)
        lay = p.layout_info()
        p.close()
        print(json.dumps({"probe": args.probe, "workload": args.workload, "reps": args.reps, "avg_ms": avg,
                          "min_ms": mn, "nodes": lay["nodes"], "elements": lay["elements"]}))
        return

    primary = args.primary if args.primary in arms else arms[0]
    if primary not in arms:
        raise SystemExit(f"primary arm {primary} is not timed")

    # ---- warm-up: W SIMP steps of every arm on throwaway problems -----------
    for arm in arms:
        time_arm(nat, torch, W, arm, args.warmup, pre=pre if arm == "learned" else None)

    # ---- timed: SIMP steps 1..K of a fresh problem per arm ------------------
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.synchronize()
    results, keep_p = {}, None
    with ClockSampler(0) as clk:
        for arm in arms:
            r, p = time_arm(nat, torch, W, arm, args.steps, pre=pre if arm == "learned" else None,
                            keep=arm == primary)
            results[arm] = r
            if p is not None:
                keep_p = p
    if world > 1:
        dist.barrier()
    elapsed = results[primary]["s"]
    if world > 1:
        t = torch.tensor([elapsed], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * args.steps / elapsed

    # ---- rooflines: the inner PCG's K*u and vector update, the network ------
    lay = keep_p.layout_info()
    nodes, nel = lay["nodes"], lay["elements"]
    ku_ms, ku_min = keep_p.bench_kernel(0, reps=20, flush_l2=True)
    res_ms, _ = keep_p.bench_kernel(1, reps=5, flush_l2=True)
    res_df_ms, _ = keep_p.bench_kernel(14, reps=5, flush_l2=True)
    upd_ms, upd_min = keep_p.bench_kernel(2, reps=20, flush_l2=True)
    kplan = keep_p.ku_plan()
    keep_p.close()
    peak, peak_kind = measured_peaks()
    # ku3: reads p, r (3 x 4 B each per node), dinv (4 B), constraint bits (1 B),
    # scale (4 B per element); writes p, q (3 x 4 B each per node)
    alg_bytes = 53 * nodes + 4 * nel
    ku_roof = {"bound": "hbm",
               "kernel": (f"ku3_kernel<{kplan['warps']},4> (tensor-copy staged p-update + FP32 K*p + p.q; "
                          f"{kplan['tiles']} tiles of 28 x {2 * kplan['warps'] - 1} nodes x {kplan['z_chunk']} planes)"),
               "achieved": alg_bytes / (ku_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
               "frac": alg_bytes / (ku_ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind,
               "traffic": ku_traffic_per_launch(W, nodes, nel), "algorithmic_bytes": alg_bytes,
               "avg_ms": ku_ms, "min_ms": ku_min}
    # the update averaged over its even / odd pair: 40 / 112 B per node
    upd_bytes = 76 * nodes
    upd_roof = {"bound": "hbm",
                "kernel": "pcg_update_df_kernel (double-float iterate folded every 2nd iteration, bulk-copy staged)",
                "achieved": upd_bytes / (upd_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                "frac": upd_bytes / (upd_ms * 1e-3) / 1e9 / peak, "algorithmic_bytes": upd_bytes,
                "avg_ms": upd_ms, "min_ms": upd_min}
    roof = ku_roof
    conv_roof = None
    if "learned" in arms:
        nx, ny, nz = shape
        g = [(v + 1 + 7) // 8 * 8 for v in (nz, ny, nx)]
        fwd_ms, flops = pre.bench_forward(1, g[0], g[1], g[2], reps=5)
        bf16 = measured_bf16_peak()
        tf = flops / (fwd_ms * 1e-3) / 1e12
        conv_roof = {"bound": "tensor", "kernel": "conv3d forward (15 BF16 3x3x3 convolutions of the network)",
                     "achieved": tf, "peak": bf16, "unit": "TFLOP/s", "frac": tf / bf16, "peak_kind": "measured",
                     "traffic": None, "algorithmic_flops": flops, "avg_ms": fwd_ms}
        if primary == "learned":
            la = results["learned"]
            net_s = la["learned_applications_per_solve"] * fwd_ms
            pcg_s = la["pcg_iterations_per_solve"] * (ku_ms + upd_ms)
            if net_s > pcg_s:
                roof = conv_roof

    # ---- end to end through the C ABI from host buffers ---------------------
    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(nat, torch, W, primary, args.steps, pre_weights=weights if primary == "learned" else None)
        e2e["value"] *= world

    cpu = None
    if not args.no_cpu_baseline and rank == 0 and "jacobi" in results:
        cpu = cpu_baseline(W, results["jacobi"]["pcg_iterations_per_solve"])

    # ---- the other benchmark configurations, short runs on this GPU ----------
    other = None
    if rank == 0 and world == 1 and not args.no_other_workloads and args.workload == "cantilever256":
        other = {}
        Wb = build_workload("bracket192")
        time_arm(nat, torch, Wb, "jacobi", 2)
        rb, pb = time_arm(nat, torch, Wb, "jacobi", min(args.steps, 8), keep=True)
        lb = pb.layout_info()
        kb_ms, _ = pb.bench_kernel(0, reps=10, flush_l2=True)
        pb.close()
        bb = 53 * lb["nodes"] + 4 * lb["elements"]
        other["bracket192"] = {
            "config": "192x96x96 bracket (config 2), Jacobi PCG with FP64 residual replacement, rel-res 1e-6, "
                      "SIMP steps 1..K of a fresh problem",
            "value": rb["value"], "unit": "SIMP iters/s", "steps": min(args.steps, 8),
            "pcg_solve_ms": rb["pcg_solve_ms"], "pcg_iterations_per_solve": rb["pcg_iterations_per_solve"],
            "solver_residual_max": rb["solver_residual_max"],
            "roofline_ku": {"achieved": bb / (kb_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                            "frac": bb / (kb_ms * 1e-3) / 1e9 / peak, "avg_ms": kb_ms, "algorithmic_bytes": bb}}
        import types

        lbatch = run_batch(types.SimpleNamespace(steps=3, warmup=2, no_e2e=True, no_cpu_baseline=True,
                                                 batch_ku=args.batch_ku, host_loop=_host_loop), nat, 1, 0,
                           emit=False)
        other["batch256"] = {k: lbatch[k] for k in ("metric", "value", "unit", "ms_per_step",
                                                   "pcg_iterations_per_problem_step", "roofline")}
        other["batch256"]["steps"] = 3
        other["batch256"]["autotuned_plan"] = lbatch["config"]["autotuned_plan"]
        other["batch256"]["pcg_ku"] = lbatch["config"]["pcg_ku"]

    if rank == 0:
        ref = results.get("jacobi")
        line = {
            "metric": METRIC, "value": value, "unit": "SIMP iters/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": args.workload, "shape": list(shape), "dof": 3 * nodes, "elements": nel,
                       "description": W["desc"], "precision": "mixed", "primary_arm": primary,
                       "arms": {a: ARM_DESC[a] for a in arms}, "window": "SIMP steps 1..K of a fresh problem",
                       "cg_tol": 1e-6, "l2": "working set per step > 129 MB L2; roofline probes flush L2",
                       "solver_loop": "host, chunk by chunk" if _host_loop else "device-side CUDA-graph while loop",
                       "parallelism": f"replicas x{world}"},
            "pcg_solve_ms": results[primary]["pcg_solve_ms"],
            "pcg_iterations_per_solve": results[primary]["pcg_iterations_per_solve"],
            "solver_residual_max": max(r["solver_residual_max"] for r in results.values()),
            "compliance_last": results[primary]["compliance"][-1],
            "arms": {a: arm_summary(r, ref) for a, r in results.items()},
            "roofline": roof,
            "kernels_ms": {"ku_pcg_fp32": ku_ms, "ku_resid_double_float": res_df_ms, "ku_resid_fp64": res_ms,
                           "pcg_update_fp32": upd_ms},
            "roofline_ku": ku_roof, "roofline_update": upd_roof, "roofline_conv": conv_roof,
            "gpu_launches": results[primary]["gpu_launches"],
            "clocks": clk.summary(),
            "e2e": e2e,
            "cpu_baseline": cpu,
            "other_workloads": other,
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
