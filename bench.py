#!/usr/bin/env python
"""SIMP iterations/s and PCG solve ms at relative residual 1e-6 on GB300.

Workload (default ``bracket192``): the 192x96x96 bracket -- 1,769,472 hex8
elements, 5,447,811 DOF, E0 = 1, nu = 0.3, E_min = 1e-9, p = 3, vf = 0.3,
rmin = 2.0 cone sensitivity filter, move 0.2, clamped x = 0 face, a passive void
cylinder (radius 16 voxels through y, axis at the x-z centre, rho = 0) and four
passive solid 6x6 bolt-pad columns (full height, inset 6 voxels from the x-y
corners, rho = 1), 3 point loads on the top face at seeded random nodes
(numpy default_rng(2)), magnitude U(0.5, 1.5), direction uniform on the sphere.
FP64 flexible CG to rel-res 1e-6 preconditioned by FP32 Jacobi-PCG inner solves.

One step = one SIMP iteration (solve, sensitivities, filter, OC update).
``value``: iterations/s over the timed steps with the state resident in HBM,
timed with CUDA events on the library's stream.
``e2e``: the same metric through the public C ABI from host buffers
(``am_problem_set_loads`` + ``am_simp_run`` for W+K iterations, density
downloaded).  The working set of a step (solver vectors + element arrays,
~300 MB) exceeds the 129 MB L2, so no explicit flush is needed between steps;
the roofline probe of the dominant kernel flushes L2 before each launch.

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


def run_batch(args, nat, world, rank):
    """Batched workload: one step = one SIMP iteration of every problem."""
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
    # roofline: plain batched FP32 K*u of the chosen plan (u, y: 12 B per node
    # each, scale 4 B per element)
    alg = 24 * nodes + 4 * nel
    peak, peak_kind = measured_peaks()
    achieved = alg / (plan["ms"] * 1e-3) / 1e9
    b.close()
    e2e = None
    if not args.no_e2e:
        total = args.warmup + args.steps
        q = nat.Batch(shapes)
        if world > 1:
            dist.barrier()
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
                       "autotuned_plan": plan, "l2": "working set per step > 129 MB L2",
                       "parallelism": f"problems sharded over {world} ranks (LPT by cost)" if world > 1 else "1 GPU"},
            "pcg_iterations_per_problem_step": float(np.mean(its_per_step)),
            "roofline": {"bound": "hbm", "kernel": f"b_ku2_kernel<{plan['warps']},KU_PLAIN> (batched FP32 K*u)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": None, "algorithmic_bytes": alg, "avg_ms": plan["ms"]},
            "gpu_launches": int(l1 - l0), "clocks": clk.summary(), "e2e": e2e, "cpu_baseline": cpu,
        }
        print(json.dumps(line))


MIXED_SOLVER = {"reliable": 0, "flexible": 1}
PRECOND = {"jacobi": 0, "mg": 2}
_mixed_solver = "reliable"
_inner_tol = 0.0
_precond = "jacobi"
_mg_deflation = 1


def simp_config(nat, W, max_iterations=100):
    return nat.default_config(nat.VARIANT_CPP, volume_fraction=W["vf"], filter_radius=W["rmin"], move_limit=0.2,
                              rho_min=0.01, E_min=1e-9, convergence_tol=0.0, max_iterations=max_iterations,
                              precision=nat.PREC_MIXED, cg_tol=1e-6, warm_start=1, inner_tol=_inner_tol,
                              cg_max_iterations=200000, mixed_solver=MIXED_SOLVER[_mixed_solver],
                              preconditioner=PRECOND[_precond], mg_deflation=_mg_deflation)


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


def ku_traffic_per_launch(W, nodes, elements):
    """DRAM bytes per launch of the fused FP32 PCG K*u from the committed ncu
    summary (measured on a smaller case, scaled by nodes), or None."""
    p = os.path.join(ROOT, "profiles", "ku_pcg_fp32_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d["dram_bytes_per_launch"] * nodes / d["nodes"]


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


def measured_pcg_iterations(workload):
    """PCG iterations per SIMP iteration measured by this GB300 arm on the same
    workload and steps (committed with the profiles), or None."""
    p = os.path.join(ROOT, "profiles", "pcg_iterations.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    e = d.get(workload)
    return None if e is None else float(e["pcg_iterations_per_solve"])


def run_reference(args, W):
    import oracle as O  # noqa: F401

    # bounded sample per step: one timed sample of the CPU restatement per step,
    # extrapolated with the PCG iteration count the GB300 arm measured (same
    # method and tolerance), so both arms do the same number of PCG iterations
    vals = []
    sample = None
    its = measured_pcg_iterations(args.workload)
    if its is None:
        its = float(os.environ.get("AM_BENCH_PCG_ITS", "2000"))
    for _ in range(max(1, args.warmup)):
        cpu_baseline(W, its, 5)
    t0 = time.time()
    for _ in range(args.steps):
        cb = cpu_baseline(W, its, 10)
        vals.append(cb["value"])
        sample = cb
    wall = time.time() - t0
    value = statistics.median(vals)
    line = {"metric": "SIMP iters/s @ rel-res 1e-6 (Jacobi PCG)", "value": value, "unit": "SIMP iters/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "shape": list(W["shape"]), "description": W["desc"]},
            "cpu_baseline": {"value": value, "unit": "SIMP iters/s", "cores": sample["cores"], "kind": "port",
                             "sample": sample["sample"]},
            "e2e": {"value": value, "unit": "SIMP iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="bracket192", choices=sorted(WORKLOADS) + ["batch256"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--probe", choices=["ku", "resid", "update", "conv", "ku2", "ku3s3", "update_even", "update_odd", "filter", "oc",
                                        "vcycle", "vcycle_defl"],
                    help="only time `reps` launches of one kernel after set-up (bounded command for ncu)")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--compare-mg", action="store_true",
                    help="time --steps SIMP iterations with the Jacobi and the multigrid mixed-precision solvers "
                         "from the same start and report the ratio and the compliance / density agreement")
    ap.add_argument("--compare-fp64", action="store_true",
                    help="time --steps SIMP iterations in mixed precision and in FP64 plain Jacobi from the same "
                         "start and report the ratio and the compliance / density agreement")
    ap.add_argument("--inner-tol", type=float, default=0.0,
                    help="mixed precision: residual reduction between FP64 replacements / per inner solve "
                         "(0: the solver's default, 0.1 reliable / 0.01 flexible)")
    ap.add_argument("--precond", default="jacobi", choices=sorted(PRECOND),
                    help="jacobi: Jacobi PCG (the headline); mg: multigrid V-cycle in the FP64 flexible CG")
    ap.add_argument("--mg-deflation", type=int, default=1, choices=[0, 1],
                    help="multigrid: balance the V-cycle with the rigid-body modes of the passive solid "
                         "inclusions (1, the default) or not (0)")
    ap.add_argument("--mixed-solver", default="reliable", choices=sorted(MIXED_SOLVER),
                    help="mixed precision: one FP32 PCG with FP64 residual replacement (reliable) or the FP64 "
                         "flexible CG over FP32 inner solves (flexible)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    global _mixed_solver, _inner_tol, _precond, _mg_deflation
    _mixed_solver = args.mixed_solver
    _mg_deflation = args.mg_deflation
    _inner_tol = args.inner_tol
    _precond = args.precond

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

    _build.build()
    nat.load()
    if not nat.is_available():
        raise SystemExit("no CUDA device: the GB300 arm needs a GPU")
    if args.workload == "batch256":
        run_batch(args, nat, world, rank)
        return
    shape = W["shape"]
    cfg = simp_config(nat, W)

    if args.compare_mg:
        import torch

        out = {}
        for name, pc in (("jacobi", nat.PRECOND_JACOBI), ("mg", nat.PRECOND_MG)):
            p = nat.Problem(shape, 1.0, 1.0, 0.3)
            p.set_loads([W["F"]], [W["fixed"]])
            c = simp_config(nat, W, max_iterations=args.steps)
            c.preconditioner = pc
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
                             outer=[r.solver_outer_iterations for r in res], rho=p.simp_density())
            p.close()
        j, m = out["jacobi"], out["mg"]
        rel = np.abs(m["comp"] - j["comp"]) / np.abs(j["comp"])
        print(json.dumps({
            "metric": "SIMP s/iteration: mixed precision, multigrid vs Jacobi preconditioner, same GPU",
            "workload": args.workload, "steps": args.steps, "jacobi_s_per_step": j["s"] / args.steps,
            "mg_s_per_step": m["s"] / args.steps, "speedup": j["s"] / m["s"],
            "compliance_rel_diff_max": float(rel.max()), "compliance_rel_diff_final": float(rel[-1]),
            "compliance_final": float(j["comp"][-1]),
            "density_max_abs_diff": float(np.max(np.abs(m["rho"] - j["rho"]))),
            "pcg_iterations_jacobi_mean": float(np.mean(j["its"])), "pcg_iterations_mg_mean": float(np.mean(m["its"])),
            "mg_deflation": _mg_deflation, "mg_iterations": m["its"], "mg_outer_iterations": m["outer"],
            "residual_max": max(j["res"], m["res"])}))
        return

    if args.compare_fp64:
        import torch

        out = {}
        for name, prec in (("mixed", nat.PREC_MIXED), ("fp64", nat.PREC_FP64)):
            p = nat.Problem(shape, 1.0, 1.0, 0.3)
            p.set_loads([W["F"]], [W["fixed"]])
            c = simp_config(nat, W)
            c.precision = prec
            if prec == nat.PREC_FP64:
                c.preconditioner = nat.PRECOND_JACOBI  # the plain FP64 Jacobi-PCG GPU path
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
        m, f = out["mixed"], out["fp64"]
        print(json.dumps({
            "metric": "SIMP s/iteration: mixed precision (FP32 PCG with FP64 residual replacement, or the FP64 flexible CG "
                      "over FP32 inner solves: mixed_solver) vs FP64 plain Jacobi PCG, same GPU",
            "mixed_solver": _mixed_solver, "inner_tol": _inner_tol, "preconditioner": _precond,
            "workload": args.workload, "steps": args.steps, "mixed_s_per_step": m["s"] / args.steps,
            "fp64_s_per_step": f["s"] / args.steps, "speedup": f["s"] / m["s"],
            "compliance_rel_diff_max": float(np.max(np.abs(m["comp"] - f["comp"]) / np.abs(f["comp"]))),
            "density_max_abs_diff": float(np.max(np.abs(m["rho"] - f["rho"]))),
            "pcg_iterations_mixed": m["its"], "pcg_iterations_fp64": f["its"],
            "residual_max": max(m["res"], f["res"])}))
        return

    if args.probe == "conv":
        # forward passes of the learned preconditioner on this workload's node grid
        pre = nat.Preconditioner(seed=0, capacity=0)
        nx, ny, nz = shape
        g = [(v + 1 + 7) // 8 * 8 for v in (nz, ny, nx)]
        ms, flops = pre.bench_forward(1, g[0], g[1], g[2], reps=args.reps)
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f).get("bf16_tflops", 1900.0))
        tf = flops / (ms * 1e-3) / 1e12
        print(json.dumps({"probe": "conv", "workload": args.workload, "grid_zyx": g, "reps": args.reps,
                          "ms_per_forward": ms, "tflops": tf, "bf16_peak_tflops": peak, "frac": tf / peak}))
        return

    if args.probe:
        # set-up only, then `reps` launches of one kernel (L2 flushed before each)
        p = nat.Problem(shape, 1.0, 1.0, 0.3)
        p.set_loads([W["F"]], [W["fixed"]])
        p.simp_begin(cfg, W["rho0"])
        # ku: the staged PCG K*u the solver runs; ku2: the register-direct kernel it
        # replaced; ku3s3: the staged kernel with 3 stages instead of 4
        which = {"ku": 0, "resid": 1, "update": 2, "ku2": 4, "ku3s3": 5, "update_even": 6, "update_odd": 7,
                 "filter": 8, "oc": 9, "vcycle": 10, "vcycle_defl": 11}[args.probe]
        if which in (8, 9):
            p.simp_step()  # the filter and OC probes time the state a SIMP step leaves
        avg, mn = p.bench_kernel(which, reps=args.reps, flush_l2=True)
        lay = p.layout_info()
        p.close()
        print(json.dumps({"probe": args.probe, "workload": args.workload, "reps": args.reps, "avg_ms": avg,
                          "min_ms": mn, "nodes": lay["nodes"], "elements": lay["elements"]}))
        return

    import torch

    torch.cuda.init()

    # ---- device-resident timed region --------------------------------------
    p = nat.Problem(shape, 1.0, 1.0, 0.3)
    p.set_loads([W["F"]], [W["fixed"]])
    p.simp_begin(cfg, W["rho0"])
    warm = [p.simp_step() for _ in range(args.warmup)]
    lay = p.layout_info()
    # CUDA events on the stream the library launches on
    lib_stream = torch.cuda.ExternalStream(p.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.synchronize()
    l0 = nat.launch_count()
    with ClockSampler(0) as clk:
        ev0.record(lib_stream)
        res = [p.simp_step() for _ in range(args.steps)]
        ev1.record(lib_stream)
        torch.cuda.synchronize()
    l1 = nat.launch_count()
    if world > 1:
        dist.barrier()
    elapsed = ev0.elapsed_time(ev1) * 1e-3
    if world > 1:
        t = torch.tensor([elapsed], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * args.steps / elapsed
    pcg_ms = 1000.0 * statistics.mean(r.solve_time_s for r in res)
    pcg_its = statistics.mean(r.solver_iterations for r in res)

    # ---- roofline of the dominant kernel (fused FP32 PCG K*u) ---------------
    nodes, nel = lay["nodes"], lay["elements"]
    ku_ms, ku_min = p.bench_kernel(0, reps=20, flush_l2=True)
    # reads p, r (3 x 4 B each per node), dinv (4 B), constraint bits (1 B), scale
    # (4 B per element); writes p, q (3 x 4 B each per node)
    alg_bytes = 53 * nodes + 4 * nel
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (ku_ms * 1e-3) / 1e9
    traffic = ku_traffic_per_launch(W, nodes, nel)
    res_ms, _ = p.bench_kernel(1, reps=5, flush_l2=True)
    upd_ms, upd_min = p.bench_kernel(2, reps=20, flush_l2=True)
    # the other half of a PCG iteration, averaged over the even / odd pair the
    # timed launches alternate between: an even iteration reads r, q (3 x 4 B each
    # per node) and dinv (4 B) and writes r (40 B per node); an odd one also reads
    # the double-float iterate (3 x 8 B), p_prev and p (3 x 4 B each) and writes
    # the iterate (112 B per node)
    upd_bytes = 76 * nodes
    p.close()

    # ---- end to end through the C ABI from host buffers ---------------------
    e2e = None
    if not args.no_e2e:
        total = args.warmup + args.steps
        ecfg = simp_config(nat, W, max_iterations=total)
        try:
            def pinned(a, dtype):
                t = torch.empty(a.size, dtype=dtype, pin_memory=True)
                arr = t.numpy()
                arr[:] = a.ravel()
                return arr, t

            F_h, _tF = pinned(W["F"], torch.float64)
            fx_h, _tx = pinned(W["fixed"].astype(np.int64), torch.int64)
            r0_h, _tr = pinned(W["rho0"], torch.float64)
            out_h, _to = pinned(np.zeros(nel), torch.float64)
        except Exception:
            F_h, fx_h, r0_h, out_h = W["F"], W["fixed"].astype(np.int64), W["rho0"].ravel(), np.zeros(nel)
        q = nat.Problem(shape, 1.0, 1.0, 0.3)
        te0 = time.perf_counter()
        q.set_loads([F_h], [fx_h])
        r = q.simp_run(ecfg, r0_h)
        out_h[:] = r["density"]
        te1 = time.perf_counter()
        q.close()
        h2d = F_h.nbytes + fx_h.nbytes + r0_h.nbytes
        d2h = out_h.nbytes + 3 * 8 * total
        e2e = {"value": world * total / (te1 - te0), "unit": "SIMP iters/s",
               "h2d_bytes_per_step": int(h2d / total), "d2h_bytes_per_step": int(d2h / total),
               "iterations": total, "wall_s": te1 - te0,
               "note": "am_problem_set_loads + am_simp_run from host buffers, cold start included"}

    cpu = None
    # the CPU restatement runs Jacobi PCG: its extrapolation needs Jacobi iteration counts
    if not args.no_cpu_baseline and rank == 0 and _precond == "jacobi":
        cpu = cpu_baseline(W, pcg_its)

    if rank == 0:
        line = {
            "metric": ("SIMP iters/s @ rel-res 1e-6 (Jacobi PCG); PCG solve ms in pcg_solve_ms" if _precond == "jacobi"
                       else "SIMP iters/s @ rel-res 1e-6 (multigrid-preconditioned flexible CG); solve ms in "
                            "pcg_solve_ms"),
            "value": value, "unit": "SIMP iters/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": args.workload, "shape": list(shape), "dof": 3 * nodes, "elements": nel,
                       "description": W["desc"], "precision": "mixed", "mixed_solver": _mixed_solver, "preconditioner": _precond,
                       **({"mg_deflation": _mg_deflation} if _precond == "mg" else {}),
                       "cg_tol": 1e-6, "l2": "working set per step > 129 MB L2; roofline probe flushes L2",
                       "parallelism": f"replicas x{world}"},
            "pcg_solve_ms": pcg_ms, "pcg_iterations_per_solve": pcg_its,
            "solver_residual_max": max(r.solver_residual for r in res),
            "compliance_last": res[-1].compliance,
            "roofline": {"bound": "hbm", "kernel": "ku3_kernel<8,4> (tensor-copy staged p-update + FP32 K*p + p.q)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": traffic, "algorithmic_bytes": alg_bytes,
                         "avg_ms": ku_ms, "min_ms": ku_min},
            "kernels_ms": {"ku_pcg_fp32": ku_ms, "ku_resid_fp64": res_ms, "pcg_update_fp32": upd_ms},
            "roofline_update": {"bound": "hbm", "kernel": "pcg_update_df_kernel (double-float iterate folded every 2nd iteration, bulk-copy staged)",
                                "achieved": upd_bytes / (upd_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                                "frac": upd_bytes / (upd_ms * 1e-3) / 1e9 / peak, "algorithmic_bytes": upd_bytes,
                                "avg_ms": upd_ms, "min_ms": upd_min},
            "gpu_launches": int(l1 - l0),
            "clocks": clk.summary(),
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
