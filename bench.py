"""Benchmark of the GB300 LBM time step (one JSON line on rank 0).

Workload (default): D3Q19 flow past a sphere, 512 x 256 x 256 cells, sphere of
radius 24 at (128,128,128) voxelised on cell centres and bounced back,
equilibrium velocity inlet u = 0.05 at x = 0, zero-gradient outlet at x = 511,
free-slip side walls, BGK tau drawn from [0.52, 0.6] by seed.  Inputs are
synthetic (built from the seed); the populations (1.3 GB in FP16, 5.1 GB in
FP64) are larger than L2, so no flush is needed between steps.

A "step" is one time step of the whole box.  ``value`` is MLUPS of the
headline storage (FP16 deviations from the lattice weights, FP32 arithmetic)
with the state resident in HBM, timed over the library's own step call (one
CUDA event pair on the engine's stream around K steps); the roofline's kernel
time comes from K further steps with an event pair around every launch; FP64 (the plain method), FP32 and BF16 are
timed the same way and reported with their velocity L2 error against FP64.
``e2e`` is the same metric through the C ABI with host buffers: the initial
FP64 populations are copied from pinned host memory and every step's residual
is read back to the host inside the timed region.

--impl reference times the reference path on the host CPU.  The reference
cannot run D3Q19 (its 3D neighbour table aborts, src/cartesiangrid.h:488-491),
so its stand-in is the project's FP64 CPU restatement of the same step
(oracle/, OpenMP over all host cores) on a bounded sample of the workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

D3Q19 = 4
B_PER_CELL = {"f64": 2 * 19 * 8 + 1, "f32": 2 * 19 * 4 + 1, "f16dev": 2 * 19 * 2 + 1, "bf16dev": 2 * 19 * 2 + 1,
              "e3m12dev": 2 * 19 * 2 + 1}
METRIC = "MLUPS (D3Q19 sphere 512x256x256, FP16-deviation storage)"
# DRAM bytes (read + write) per launch of the bulk step kernel on this
# workload, averaged over the two step parities: taken from an ncu capture on
# the 512x256x64 slab of the sphere case and scaled by cells to the full box;
# not measured by this script
PROFILED_TRAFFIC_PER_STEP = {"f16dev": 2.32e9}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def sphere_case(nx=512, ny=256, nz=256, radius=24.0, center=(128.0, 128.0, 128.0), seed=2026):
    rng = np.random.default_rng(seed)
    tau = float(rng.uniform(0.52, 0.6))
    flags = np.zeros((nz, ny, nx), dtype=np.uint8)
    lo = [max(0, int(math.floor(c - radius - 1))) for c in center]
    hi = [int(math.ceil(c + radius + 1)) for c in center]
    z, y, x = np.meshgrid(np.arange(lo[2], min(hi[2], nz)), np.arange(lo[1], min(hi[1], ny)), np.arange(lo[0], min(hi[0], nx)),
                          indexing="ij")
    inside = (x + 0.5 - center[0]) ** 2 + (y + 0.5 - center[1]) ** 2 + (z + 0.5 - center[2]) ** 2 < radius * radius
    sub = flags[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
    sub[inside] = 1
    flags[:, :, 0] = 2
    flags[:, :, -1] = 3
    # started from the free stream (the equilibrium at rho = 1 and the inlet
    # velocity in every fluid cell), the usual impulsive start of a flow past
    # an obstacle
    return dict(shape=(nx, ny, nz), tau=tau, flags=flags.reshape(-1),
                faces=("open", "open", "freeslip", "freeslip", "freeslip", "freeslip"), inlet=(0.05, 0.0, 0.0),
                init=(0.05, 0.0, 0.0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join("/tmp", f"lbm_clocks_{os.getpid()}.csv")

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.fh.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons), "samples": len(sm)}


def job_throughput(local_ms: float, cells_per_rank: int, steps: int, dist=None, device="cuda"):
    """Replicas: every rank steps its own copy of the workload.  The job time
    is the slowest rank's (max over ranks); the whole-job MLUPS counts the
    cells of every rank.  Returns (max_ms, mlups)."""
    import torch

    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    world = 1
    if dist is not None and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        world = dist.get_world_size()
    max_ms = float(t.item())
    return max_ms, cells_per_rank * steps * world / (max_ms / 1e3) / 1e6


def cpu_baseline(threads: int, budget_s: float = 12.0):
    """The FP64 CPU restatement (oracle) on a bounded sample of the workload:
    the same geometry scaled to 128 x 64 x 64 cells (sphere radius 6)."""
    import oracle

    case = sphere_case(128, 64, 64, radius=6.0, center=(32.0, 32.0, 32.0))
    o = oracle.BoxOracle(D3Q19, case["shape"], 1.0 / case["tau"], faces=case["faces"], flags=case["flags"],
                         inlet_velocity=case["inlet"])
    o.init_equilibrium(1.0, case["init"])
    t0 = time.perf_counter()
    o.step(2, threads)
    dt = (time.perf_counter() - t0) / 2
    steps = max(2, min(400, int(budget_s / max(dt, 1e-6))))
    t0 = time.perf_counter()
    o.step(steps, threads)
    sec = time.perf_counter() - t0
    cells = int(np.prod(case["shape"]))
    return {"value": cells * steps / sec / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"D3Q19 sphere scaled to 128x64x64 (r=6), {steps} steps, FP64, OpenMP {threads} threads"}


def mass_drift(tau, device, steps=100_000):
    """Relative change of the FP64 mass sum over `steps` steps, per storage,
    on a closed box: the sphere case scaled to 96 x 64 x 64 (radius 8),
    periodic along x instead of inlet / outlet, free-slip sides, started from
    a uniform flow u = 0.05 (bounce-back, periodic wrap and free slip all
    conserve mass, so any change is rounding)."""
    from lbm_gb300.solver import BoxSolver

    shape = (96, 64, 64)
    c = sphere_case(*shape, radius=8.0, center=(32.0, 32.0, 32.0))
    flags = c["flags"].copy()
    flags[flags > 1] = 0  # the inlet and outlet planes become fluid
    out = {}
    for st in ("f64", "f32", "f16dev", "bf16dev", "e3m12dev"):
        s = BoxSolver(D3Q19, shape, 1.0 / tau, st, faces=("periodic", "periodic") + ("freeslip",) * 4, flags=flags,
                      init_velocity=(0.05, 0.0, 0.0), device=device)
        s.initial_condition()
        m0 = s.mass_momentum()[0]
        s.step(steps)
        m1 = s.mass_momentum()[0]
        s.close()
        out[st] = float((m1 - m0) / m0)
    return out


def long_horizon_accuracy(device, steps=5000):
    """Velocity relative L2 of each storage against the plain FP64 method
    after `steps` steps of the sphere case scaled to 256 x 128 x 128 (radius
    12), all started from the free stream: the flow has passed the box twice."""
    from lbm_gb300.solver import BoxSolver

    case = sphere_case(256, 128, 128, radius=12.0, center=(64.0, 64.0, 64.0))
    u = {}
    for st in ("f64", "f32", "f16dev", "bf16dev", "e3m12dev"):
        s = BoxSolver(D3Q19, case["shape"], 1.0 / case["tau"], st, faces=case["faces"], flags=case["flags"],
                      inlet_velocity=case["inlet"], init_velocity=case["init"], device=device)
        s.initial_condition()
        s.step(steps)
        u[st] = s.moments()[1]
        s.close()
    ref = u.pop("f64")
    out = {st: float(np.linalg.norm(v - ref) / np.linalg.norm(ref)) for st, v in u.items()}
    out["case"] = f"D3Q19 sphere 256x128x128 (r=12), {steps} steps from the free stream"
    return out


def accuracy_run(args):
    """Velocity relative L2 against the plain FP64 method of every storage,
    with and without the free-stream shift of the single-precision state,
    at checkpoints of a long run of the sphere case: the 256x128x128 sample
    (r=12) to 50,000 steps and the full 512x256x256 box to 10,000 steps, both
    started from the free stream."""
    from lbm_gb300.solver import BoxSolver

    out = {"metric": "velocity relative L2 vs FP64 (D3Q19 sphere)", "unit": "relative L2", "higher_is_better": False,
           "dtype": "f64 reference; f32 / f16 / bf16 storage with f32 arithmetic", "data": "synthetic", "rows": []}
    spec = {"f64": ("f64", True), "f32": ("f32", True), "f32_noshift": ("f32", False), "f16dev": ("f16dev", True),
            "f16dev_noshift": ("f16dev", False), "bf16dev": ("bf16dev", True), "e3m12dev": ("e3m12dev", True)}
    runs = (((256, 128, 128, 12.0, (64.0, 64.0, 64.0)), (1000, 5000, 20000, 50000)),
            ((512, 256, 256, 24.0, (128.0, 128.0, 128.0)), (2000, 5000, 10000)))
    if args.acc_full_steps:
        # the full box alone, to the given length (the configuration's 50,000)
        full = sorted({c for c in (2000, 5000, 10000, 20000, 50000) if c < args.acc_full_steps} | {args.acc_full_steps})
        runs = (((512, 256, 256, 24.0, (128.0, 128.0, 128.0)), tuple(full)),)
    for (nx, ny, nz, r, c), checkpoints in runs:
        case = sphere_case(nx, ny, nz, radius=r, center=c)
        sol = {}
        for n, (st, sh) in spec.items():
            sol[n] = BoxSolver(D3Q19, case["shape"], 1.0 / case["tau"], st, faces=case["faces"], flags=case["flags"],
                               inlet_velocity=case["inlet"], init_velocity=case["init"], shift=sh)
            sol[n].initial_condition()
        done = 0
        for cp in checkpoints:
            for sv in sol.values():
                sv.step(cp - done)
            done = cp
            u64 = sol["f64"].moments()[1]
            row = {"case": f"{nx}x{ny}x{nz}", "steps": cp}
            for n, sv in sol.items():
                if n != "f64":
                    row[n] = float(np.linalg.norm(sv.moments()[1] - u64) / np.linalg.norm(u64))
            out["rows"].append(row)
            print(json.dumps(row), file=sys.stderr, flush=True)
        for sv in sol.values():
            sv.close()
    out["value"] = next(r["f16dev"] for r in out["rows"] if r["case"] == "512x256x256" and r["steps"] == 5000)
    if args.acc_full_steps:
        out["value_at_end"] = out["rows"][-1]["f16dev"]
    out["config"] = {"workload": "D3Q19 flow past a sphere from the free stream; value: FP16 storage, full box, 5,000 steps",
                     "tau": sphere_case(64, 32, 32)["tau"]}
    return out


def run_variant(storage, case, warmup, steps, device):
    from lbm_gb300.solver import BoxSolver

    s = BoxSolver(D3Q19, case["shape"], 1.0 / case["tau"], storage, faces=case["faces"], flags=case["flags"],
                  inlet_velocity=case["inlet"], init_velocity=case["init"], device=device)
    s.initial_condition()
    s.step(warmup)
    s.synchronize()
    # the product's stepping path (captured per-parity graphs, residual on the
    # last two steps) timed as a whole; then the same number of steps with an
    # event pair around every step-kernel launch, for the kernel time
    tot = s.time_steps(steps)
    _, ker, n = s.profile_steps(steps)
    return s, tot, ker, n


def cavities_run(args, dist=None):
    """The batched cavities (2048 D2Q9 lid-driven cavities, sides 32-512,
    Re 10-1000, FP32): device-timed steps of the whole batch, then a bounded
    run with the convergence check (residual 1e-8, every 100 steps), and (one
    GPU) the FP32 error at convergence on a subset run in FP64 too.  Under
    torchrun every rank takes a contiguous share of the cavities balanced by
    cells (lbm_gb300.shard) and steps it on its own GPU; the job time is the
    slowest rank's and the per-cavity results are gathered on every rank."""
    import torch

    from lbm_gb300 import cases, shard
    from lbm_gb300.solver import BatchSolver

    c = cases.cavities()
    sides, omegas = c["sides"], 1.0 / c["tau"]
    area_all = sides.astype(np.int64) ** 2
    world = dist.get_world_size() if dist is not None and dist.is_initialized() else 1
    info = {}

    def solve(lo, hi):
        b = BatchSolver(sides[lo:hi], omegas[lo:hi], c["lid"], "f32")
        b.initial_condition()
        b.step(args.warmup)
        if dist is not None and dist.is_initialized():
            dist.barrier()
        tot, ker, n = b.profile_steps(args.steps)
        info.update(tot=tot, ker=ker, n=n, cells=b.ncells, tuning=b.tuning())
        t0 = time.perf_counter()
        steps = b.run(args.cavity_steps, 100, 1e-8, raise_on_divergence=False)
        info["wall"] = time.perf_counter() - t0
        out = {"steps": steps, "status": b.status(), "residual": b.residuals().max(axis=1)}
        b.close()
        return out

    res_all = shard.run_sharded(area_all, solve, dist)
    t = torch.tensor([info["tot"], info["wall"], info["ker"] / max(info["n"], 1)], dtype=torch.float64,
                     device="cuda" if world > 1 else "cpu")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    tot, wall, kernel_avg_ms = (float(v) for v in t.tolist())
    cells = int(area_all.sum())
    hbm, peak_kind = peaks()
    bpc = 2 * 9 * 4 + 0  # no flag byte: the geometry follows from the side
    before = np.zeros(len(area_all), dtype=np.int64) + args.warmup + args.steps
    status, res, steps = res_all["status"], res_all["residual"], res_all["steps"]
    ok = np.isfinite(res) & (status != BatchSolver.DIVERGED)
    res_q = [float(x) for x in np.percentile(res[ok], [0, 50, 90, 100])] if ok.any() else None
    updates = float(np.sum((steps - before) * area_all))
    grid, tpb = info["tuning"]
    return {"metric": "MLUPS (2048 batched D2Q9 lid-driven cavities, FP32)", "value": cells * args.steps / (tot / 1e3) / 1e6,
            "unit": "MLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot / args.steps,
            "dtype": "f32", "scaling": "strong",
            "config": {"workload": "2048 D2Q9 lid-driven cavities, sides U{32..512}, Re logU[10,1000], lid 0.1, FP32",
                       "cells": cells, "bytes_per_cell": bpc, "grid": grid, "threads_per_block": tpb,
                       "parallelism": f"cavities sharded over {world} GPUs (contiguous shares balanced by cells)" if world > 1
                       else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": bpc * cells / world / (kernel_avg_ms / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": bpc * cells / world / (kernel_avg_ms / 1e3) / 1e9 / hbm, "peak_kind": peak_kind, "kernel": "k_batch",
                         "kernel_avg_ms": kernel_avg_ms},
            "run": {"max_steps": args.cavity_steps, "wall_s": wall, "mlups": updates / wall / 1e6,
                    "converged": int(np.sum(status == BatchSolver.CONVERGED)), "diverged": int(np.sum(status == BatchSolver.DIVERGED)),
                    "of": int(len(area_all)), "final_residual_min_median_p90_max": res_q},
            **({"f32_vs_f64_at_convergence": cavities_against_fp64(c)} if world == 1 and args.cavity_check else {})}


def cavities_against_fp64(c, max_steps: int = 100000, count: int = 48):
    """The FP32 batch's stated error at convergence: up to `count` of the
    cavities whose slowest viscous mode decays within the configuration's step
    bound (10 n Re <= 1e5, i.e. n^2 / nu <= 1e5 at lid speed 0.1), run to
    residual 1e-8 (every 100 steps, at most `max_steps`) in FP64 and in FP32
    storage; per cavity, the velocity relative L2 of the FP32 state against
    the converged FP64 one."""
    from lbm_gb300.solver import BatchSolver
    from lbm_gb300.warmstart import C_D2Q9

    sides, re = c["sides"], c["re"]
    pick = np.flatnonzero(10.0 * sides * re <= 1e5)
    pick = pick[np.linspace(0, len(pick) - 1, min(count, len(pick))).astype(int)] if len(pick) else pick
    out = {"cavities": int(len(pick)), "selection": "10 n Re <= 1e5, evenly spaced over the batch", "max_steps": max_steps}
    if not len(pick):
        return out
    res = {}
    for st in ("f64", "f32"):
        b = BatchSolver(sides[pick], 1.0 / c["tau"][pick], c["lid"], st)
        b.initial_condition()
        t0 = time.perf_counter()
        steps = b.run(max_steps, 100, 1e-8, raise_on_divergence=False)
        wall = time.perf_counter() - t0
        u = []
        for d in range(len(pick)):
            f = b.domain_populations(d)
            rho = f.sum(axis=0)
            u.append(np.stack([(C_D2Q9[:, k, None] * f).sum(axis=0) / rho for k in range(2)]))
        res[st] = dict(steps=steps, status=b.status(), u=u, wall=wall, resid=b.residuals().max(axis=1))
        b.close()
    conv64 = res["f64"]["status"] == BatchSolver.CONVERGED
    err = np.array([np.linalg.norm(a - b) / np.linalg.norm(b) for a, b in zip(res["f32"]["u"], res["f64"]["u"])])
    q = lambda v: [float(x) for x in np.percentile(v, [0, 50, 100])] if len(v) else None  # noqa: E731
    out.update({"f64_converged": int(conv64.sum()), "f64_steps_min_median_max": q(res["f64"]["steps"][conv64]),
                "f64_wall_s": res["f64"]["wall"], "f32_converged": int(np.sum(res["f32"]["status"] == BatchSolver.CONVERGED)),
                "f32_final_residual_min_median_max": q(res["f32"]["resid"]),
                "f32_vel_rel_l2_vs_f64_min_median_max": q(err[conv64]),
                "sides_min_max": [int(sides[pick].min()), int(sides[pick].max())],
                "re_min_max": [float(re[pick].min()), float(re[pick].max())]})
    return out


def poisson_run(args):
    """D3Q7 Poisson-Boltzmann on 256^3 (seeded charged spheres, Debye length
    and surface potentials by seed): device-timed steps in FP32 storage, the
    FP32 solve to residual 1e-10 (FP64 residual reductions), the FP32
    potential against an FP64 run after the same 5,000 steps, and the FP32
    end state against the FP64 solve to the same residual (at most 100,000
    steps)."""
    from lbm_gb300 import cases
    from lbm_gb300.solver import BoxSolver

    c = cases.pb_spheres(256, seed=7)
    kw = cases.box_kwargs(c)
    hbm, peak_kind = peaks()
    cells = 256 ** 3
    out = {"metric": "MLUPS (D3Q7 Poisson-Boltzmann 256^3, FP32 storage)", "unit": "MLUPS", "dtype": "f32",
           "config": {"workload": f"D3Q7 Poisson-Boltzmann 256^3, {len(c['spheres'])} spheres, Debye length {c['debye']:.2f}",
                      "cells": cells, "bytes_per_cell": 2 * 7 * 4 + 1}}
    g = BoxSolver(c["lattice"], c["shape"], c["omega"], "f32", pb_nonlinear=True, **kw)
    g.initial_condition()
    g.step(args.warmup)
    tot, ker, n = g.profile_steps(args.steps)
    out["value"] = cells * args.steps / (tot / 1e3) / 1e6
    ach = (2 * 7 * 4 + 1) * cells / (ker / n / 1e3) / 1e9
    out["roofline"] = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "peak_kind": peak_kind}
    g.initial_condition()
    g.step(5000)
    phi32, _ = g.moments()
    t0 = time.perf_counter()
    steps, res = g.run_to(1e-10, 1000, args.max_steps - 5000)
    wall = time.perf_counter() - t0
    out["solve_f32"] = {"steps": steps + 5000, "wall_s_after_5000": wall, "residual": float(np.max(res)), "converged": bool(np.max(res) < 1e-10)}
    phi32_end, _ = g.moments()
    g.close()
    h = BoxSolver(c["lattice"], c["shape"], c["omega"], "f64", pb_nonlinear=True, **kw)
    h.initial_condition()
    t0 = time.perf_counter()
    h.step(5000)
    out["f64_mlups"] = cells * 5000 / (time.perf_counter() - t0) / 1e6
    phi64, _ = h.moments()
    out["phi_rel_l2_f32_vs_f64_at_5000"] = float(np.linalg.norm(phi32 - phi64) / np.linalg.norm(phi64))
    # the FP64 solve to the configuration's residual, and the FP32 end state's
    # stated error against it
    t0 = time.perf_counter()
    steps64, res64 = h.run_to(1e-10, 1000, min(args.max_steps, 100000) - 5000)
    phi64_end, _ = h.moments()
    h.close()
    out["solve_f64"] = {"steps": steps64 + 5000, "wall_s_after_5000": time.perf_counter() - t0, "residual": float(np.max(res64)),
                        "converged": bool(np.max(res64) < 1e-10)}
    out["phi_rel_l2_f32_end_vs_f64_converged"] = float(np.linalg.norm(phi32_end - phi64_end) / np.linalg.norm(phi64_end))
    return out


def sweep_run(args):
    """A sweep over geometry and Reynolds number stepped by one launch per
    step: 256 inlet-driven D2Q9 channels 512x128 (1-8 cylinders each, Re
    20-200 by seed, inlet u = 0.05) as the z-slices of one box, each slice
    relaxing at its own rate, FP32 storage.  Device-timed steps and the HBM
    fraction; then three slices checked bit for bit against boxes of their
    own after 100 steps."""
    from lbm_gb300 import cases
    from lbm_gb300.solver import BoxSolver

    n_ch, nx, ny = 256, 512, 128
    chans = [cases.cylinder_channel(s, nx=nx, ny=ny) for s in range(n_ch)]
    st = cases.stacked_sweep(chans)
    g = BoxSolver(st["lattice"], st["shape"], st["omega"], "f32", **cases.box_kwargs(st))
    g.set_slice_omega(st["slice_omega"])
    g.initial_condition()
    g.step(args.warmup)
    tot, ker, n = g.profile_steps(args.steps)
    cells = nx * ny * n_ch
    bpc = 2 * 9 * 4 + 1
    hbm, peak_kind = peaks()
    ach = bpc * cells / (ker / n / 1e3) / 1e9
    g.initial_condition()
    g.step(100)
    f = g.populations()
    same = {}
    for k in (0, n_ch // 2, n_ch - 1):
        one = cases.stacked_sweep([chans[k]])
        s1 = BoxSolver(one["lattice"], one["shape"], 1.0 / chans[k]["tau"], "f32", **cases.box_kwargs(one))
        s1.initial_condition()
        s1.step(100)
        same[str(k)] = bool(np.array_equal(f[:, k * nx * ny:(k + 1) * nx * ny], s1.populations()))
        s1.close()
    kernel = g.kernel()
    g.close()
    re = [c["re"] for c in chans]
    return {"metric": "MLUPS (sweep: 256 D2Q9 cylinder channels 512x128, Re 20-200, FP32, one launch per step)",
            "value": cells * args.steps / (tot / 1e3) / 1e6, "unit": "MLUPS", "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": tot / args.steps, "dtype": "f32", "higher_is_better": True,
            "config": {"workload": "256 inlet-driven D2Q9 channels 512x128 with 1-8 cylinders, Re 20-200 by seed, one relaxation "
                                   "rate per slice", "cells": cells, "bytes_per_cell": bpc, "re_min_max": [min(re), max(re)],
                       "bulk_kernel": kernel},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "peak_kind": peak_kind,
                         "kernel_avg_ms": ker / n},
            "slices_bitwise_vs_own_boxes_after_100_steps": same}


def debye_run(args):
    """A Debye-length sweep stepped by one launch per step: 8 charged-sphere
    boxes 128^3 (Debye length 4-32 and 1-64 spheres by seed, potential 0 on
    each box's outer layer) stacked along z into one D3Q7 box 128x128x1024,
    each box at its own kappa^2, nonlinear sinh source, FP32 storage.
    Device-timed steps and the HBM fraction; then three boxes checked bit for
    bit against boxes of their own after 60 steps."""
    from lbm_gb300 import cases
    from lbm_gb300.solver import BoxSolver

    n_box, n = 8, 128
    units = [cases.pb_spheres(n, seed=s) for s in range(n_box)]
    st = cases.stacked_debye(units)
    g = BoxSolver(st["lattice"], st["shape"], st["omega"], "f32", pb_nonlinear=True, **cases.box_kwargs(st))
    g.set_slice_kappa(st["slice_kappa_sq"])
    g.initial_condition()
    g.step(args.warmup)
    tot, ker, nl = g.profile_steps(args.steps)
    cells = n * n * n * n_box
    bpc = 2 * 7 * 4 + 1
    hbm, peak_kind = peaks()
    ach = bpc * cells / (ker / nl / 1e3) / 1e9
    g.initial_condition()
    g.step(60)
    f = g.populations()
    same = {}
    for k in (0, n_box // 2, n_box - 1):
        u = units[k]
        s1 = BoxSolver(u["lattice"], u["shape"], u["omega"], "f32", pb_nonlinear=True, **cases.box_kwargs(u))
        s1.initial_condition()
        s1.step(60)
        same[str(k)] = bool(np.array_equal(f[:, k * n ** 3:(k + 1) * n ** 3], s1.populations()))
        s1.close()
    kernel = g.kernel()
    g.close()
    debye = [u["debye"] for u in units]
    return {"metric": "MLUPS (Debye-length sweep: 8 D3Q7 Poisson-Boltzmann boxes 128^3, FP32, one launch per step)",
            "value": cells * args.steps / (tot / 1e3) / 1e6, "unit": "MLUPS", "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": tot / args.steps, "dtype": "f32", "higher_is_better": True,
            "config": {"workload": "8 charged-sphere boxes 128^3 stacked along z, Debye length 4-32 and 1-64 spheres by seed, "
                                   "one kappa^2 per box", "cells": cells, "bytes_per_cell": bpc,
                       "debye_min_max": [min(debye), max(debye)], "spheres": [len(u["spheres"]) for u in units],
                       "bulk_kernel": kernel},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "peak_kind": peak_kind,
                         "kernel_avg_ms": ker / nl},
            "boxes_bitwise_vs_own_boxes_after_60_steps": same}


def poiseuille_run(args):
    """D2Q9 Guo-forced Poiseuille channel 256x64, plain FP64, 20,000 steps
    (the state fits in L2): device-timed MLUPS and the deviation from the
    analytic parabola."""
    from lbm_gb300 import cases
    from lbm_gb300.solver import BoxSolver

    c = cases.poiseuille_guo()
    g = BoxSolver(c["lattice"], c["shape"], c["omega"], "f64", **cases.box_kwargs(c))
    g.initial_condition()
    g.step(args.warmup)
    tot, ker, n = g.profile_steps(200)
    g.initial_condition()
    t0 = time.perf_counter()
    g.step(20000)
    wall = time.perf_counter() - t0
    _, u = g.moments()
    ux = u[0].reshape(64, 256).mean(axis=1)
    exact = cases.poiseuille_profile(64, c["tau"], c["g"])
    g.close()
    return {"metric": "MLUPS (D2Q9 Guo Poiseuille 256x64, FP64)", "unit": "MLUPS", "dtype": "f64",
            "value": 256 * 64 * 20000 / wall / 1e6, "device_timed_mlups": 256 * 64 * 200 / (tot / 1e3) / 1e6,
            "config": {"workload": "D2Q9 Guo Poiseuille 256x64, tau 0.8, g 1e-6, 20,000 steps", "cells": 256 * 64},
            "analytic_max_rel_dev_after_20000": float(np.abs(ux - exact).max() / exact.max())}


def warmstart_run(args):
    """Learned warm start, D2Q9 forced channel 511x128 with 1-8 cylinders, Re
    20-200: FP32 training fields, U-Net training with the project's BF16
    tensor-core kernels, then held-out channels by the plain FP64 LBM to
    residual 1e-8 (per channel) from rest, from rest with the period-2
    filters, the same with the flow-rate projection, from the prediction with
    the filters, and from the prediction with its flow rate balanced against
    the body force, the filters and the projection (the warm start;
    `value`)."""
    from lbm_gb300 import warmstart as ws

    out = ws.experiment(n_train=args.ws_train, per_batch=args.ws_per_batch, train_steps=args.ws_train_steps, epochs=args.ws_epochs,
                        n_eval=16, per_eval=8, tol=1e-8, max_steps=args.max_steps, lr=args.ws_lr,
                        log=lambda m: print(m, file=sys.stderr, flush=True))
    return {"metric": "learned warm start: wall time to residual 1e-8, warm / from rest", "value": out["wall_ratio"],
            "unit": "ratio", "higher_is_better": False, "dtype": "f64 (LBM), bf16 (network)",
            "arms_wall_ratio_vs_rest": {"rest_plus_filters": out["rest_filtered_wall_ratio"],
                                        "rest_plus_filters_plus_projection": out["rest_projected_wall_ratio"],
                                        "prediction_plus_filters": out["net_only_wall_ratio"],
                                        "prediction_balanced_plus_filters_plus_projection": out["wall_ratio"]},
            "config": {"workload": "D2Q9 forced channel 511x128, 1-8 cylinders r 6-20, Re 20-200, U-Net 4 levels width 32",
                       "n_train": out["n_train"], "train_steps": out["train_steps"], "epochs": out["epochs"],
                       "per_reynolds_number": args.ws_per_batch}, "detail": out}


def grid_run(args):
    """Grid and tables of the D3Q19 sphere channel (512 x 256 x 256 box with
    a subtracted sphere of radius 24, level 9) built from the JSON config:
    the host build and the device build (same tables, checked), wall time."""
    from lbm_gb300 import gridgen

    cfg = {"dim": 3, "partitionLevel": 9, "uniformLevel": 9, "maxRfnmtLvl": 9,
           "geometry": {"channel": {"type": "box", "A": [0, 0, 0], "B": [512, 256, 256], "body": "flow"},
                        "sphere": {"type": "sphere", "center": [128, 128, 128], "radius": 24, "body": "flow", "subtract": True}},
           "solver": {"boundary": {"channel": {"-x": {"type": "inlet", "velocity": [0.05, 0, 0]}, "+x": {"type": "outlet"},
                                               "-y": {"type": "freeslip"}, "+y": {"type": "freeslip"},
                                               "-z": {"type": "freeslip"}, "+z": {"type": "freeslip"}},
                                   "sphere": {"all": {"type": "wall"}}}}}
    gridgen.grid_tables(cfg, device=0)  # warm-up: context and module load
    t0 = time.perf_counter()
    dev = gridgen.grid_tables(cfg, device=0)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    host = gridgen.grid_tables(cfg)
    t_host = time.perf_counter() - t0
    same = bool(np.array_equal(dev.centers, host.centers) and np.array_equal(dev.nghbr, host.nghbr) and
                all(np.array_equal(dev.surfaces[k]["cells"], host.surfaces[k]["cells"]) for k in host.surfaces))
    # the multi-level generator (host): a 2D channel minus a cylinder,
    # partitioning level 4, uniform to level 10, boundary cells refined to 13
    tree_cfg = {"dim": 2, "partitionLevel": 4, "uniformLevel": 10, "maxRfnmtLvl": 13, "maxNoCells": 20_000_000,
                "geometry": {"cube": {"type": "box", "body": "flow", "A": [0.0, 0.0], "B": [10.0, 4.0]},
                             "cyl": {"type": "sphere", "body": "flow", "subtract": True, "center": [3.1, 2.05], "radius": 0.8}}}
    t0 = time.perf_counter()
    tree = gridgen.grid_tree(tree_cfg)
    t_tree = time.perf_counter() - t0
    return {"metric": "grid and table build, D3Q19 sphere channel 512x256x256 from its JSON config", "value": t_dev, "unit": "s",
            "higher_is_better": False, "config": {"workload": "uniform level 9, box minus sphere r=24", "cells": dev.ncells},
            "host_s": t_host, "device_s": t_dev, "identical": same,
            "tree": {"workload": "2D channel minus cylinder, partitioning level 4, uniform to 10, boundary-refined to 13 (host)",
                     "cells": int(len(tree.level)), "levels": [tree.partition_level, tree.highest_level], "s": t_tree}}


def lpt_run(args):
    """Particle step of the reference's falling1m case on the GPU: 10^6
    particles, 2D, the reference's default force model (gravity, buoyancy,
    Stokes drag) with forward Euler, dt 1e-7, 100 steps per call (one launch;
    the state stays in registers).  CPU baseline: the oracle's scalar
    restatement on a 1,000-particle sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import lpt_oracle as lo
    from lbm_gb300.lpt import ParticleSolver

    n, steps = 1_000_000, 100
    rng = np.random.default_rng(123456789)
    v = np.full((n, 11), np.nan)
    v[:, :2] = rng.uniform(0.0, 1.0, (n, 2))
    v[:, 2:4] = 0.0
    v[:, 6], v[:, 7], v[:, 9] = 0.01, 800.0, 4.0 / 3.0 * np.pi * 0.01 ** 3
    solver = {"dt": 1e-7, "gravity": [0, 10]}
    ps = ParticleSolver.from_config(solver, 2, capacity=n)
    ps.set_particles(v)
    ps.step(steps)  # warm-up
    times = []
    for _ in range(max(3, args.warmup)):
        t0 = time.perf_counter()
        ps.step(steps)
        times.append(time.perf_counter() - t0)
    sec = min(times)
    prm = lo.config_params(solver, 2)
    sample = v[:1000]
    t0 = time.perf_counter()
    lo.step(sample, 2, nsteps=steps, **prm)
    cpu = 1000 * steps / (time.perf_counter() - t0) / 1e6
    return {"metric": "particle steps per second (10^6 particles, 2D, gravity + buoyancy + Stokes drag, forward Euler)",
            "value": n * steps / sec / 1e6, "unit": "M particle-steps/s", "dtype": "f64",
            "config": {"workload": "falling1m: 1e6 particles, 100 steps per call", "particles": n, "steps_per_call": steps},
            "ms_per_call": sec * 1e3, "bytes_per_particle_call": 2 * 8 * 11,
            "cpu_baseline": {"value": cpu, "unit": "M particle-steps/s", "cores": 1, "kind": "port",
                             "sample": "1,000 particles x 100 steps, scalar Python restatement"}}


def profile_case(args):
    """A small case of one workload for ncu: set-up and autotuning first, then
    the measured launches inside the NVTX range "profile" (capture them with
    ncu --nvtx --nvtx-include "profile/")."""
    import torch

    rng = torch.cuda.nvtx
    if args.profile_case in B_PER_CELL:
        from lbm_gb300.solver import BoxSolver

        if args.profile_size == "slab":
            case = sphere_case(512, 256, 64, radius=24.0, center=(128.0, 128.0, 32.0))
        else:
            case = sphere_case(256, 128, 128, radius=12.0, center=(64.0, 64.0, 64.0))
        s = BoxSolver(D3Q19, case["shape"], 1.0 / case["tau"], args.profile_case, faces=case["faces"], flags=case["flags"],
                      inlet_velocity=case["inlet"], init_velocity=case["init"])
        s.initial_condition()
        if args.kernel:
            s.kernel(args.kernel)
        s.step(4)
        s.synchronize()
        rng.range_push("profile")
        s.step(4)
        s.synchronize()
        rng.range_pop()
        return {"profile_case": args.profile_case, "threads_per_block": s.threads_per_block(), "kernel": s.kernel(),
                "cells": int(np.prod(case["shape"]))}
    if args.profile_case == "cavities":
        from lbm_gb300 import cases
        from lbm_gb300.solver import BatchSolver

        c = cases.cavities()
        sides, om = c["sides"][:256], 1.0 / c["tau"][:256]
        b = BatchSolver(sides, om, c["lid"], "f32")
        b.initial_condition()
        b.step(4)
        torch.cuda.synchronize()
        rng.range_push("profile")
        b.step(4)
        torch.cuda.synchronize()
        rng.range_pop()
        return {"profile_case": "cavities", "domains": 256, "cells": b.ncells, "tuning": b.tuning()}
    if args.profile_case == "table":
        # the reference-table engine (the reference's phase sequence, FP64,
        # int32 pull table) on the own lid-driven cavity config at level 10:
        # 1024 x 1024 cells, state and tables larger than L2
        from lbm_gb300.solver import LBMSolver

        cfg = json.load(open(os.path.join(ROOT, "tests", "golden", "cases", "cavity_small.json")))
        cfg.update({"partitionLevel": 10, "uniformLevel": 10, "maxRfnmtLvl": 10})
        s = LBMSolver.from_config(cfg)
        g = s.gpu
        g.initial_condition()
        g.step(16)
        t0 = time.perf_counter()
        g.step(400)
        wall = time.perf_counter() - t0
        rng.range_push("profile")
        g.step(8)
        rng.range_pop()
        n = s.grid.ncells
        return {"profile_case": "table", "cells": n, "host_timed_mlups_400_steps": n * 400 / wall / 1e6,
                "ms_per_step": wall / 400 * 1e3}
    if args.profile_case == "poisson":
        from lbm_gb300 import cases
        from lbm_gb300.solver import BoxSolver

        c = cases.pb_spheres(256, seed=7)
        g = BoxSolver(c["lattice"], c["shape"], c["omega"], "f32", pb_nonlinear=True, **cases.box_kwargs(c))
        g.initial_condition()
        if args.kernel:
            g.kernel(args.kernel)
        g.step(4)
        g.synchronize()
        rng.range_push("profile")
        g.step(4)
        g.synchronize()
        rng.range_pop()
        return {"profile_case": "poisson", "cells": 256 ** 3, "kernel": g.kernel()}
    # the U-Net: one training step (forward, loss, backward) on a batch of 8
    from lbm_gb300.warmstart import UNet

    net = UNet(8, 128, 512, seed=1)
    r = np.random.default_rng(3)
    net.set_batch((r.normal(size=(8, 128, 512, 32)) * 0.5).astype(np.float32), r.normal(size=(8, 128, 512, 3)).astype(np.float32),
                  np.ones((8, 128, 512), dtype=bool))
    net.loss_and_grad()
    torch.cuda.synchronize()
    rng.range_push("profile")
    loss = net.loss_and_grad()
    torch.cuda.synchronize()
    rng.range_pop()
    return {"profile_case": "unet", "batch": 8, "shape": [128, 512], "loss": loss}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--storage", default="f16dev", choices=list(B_PER_CELL))
    ap.add_argument("--quick", action="store_true", help="skip the FP32/BF16 comparison runs")
    ap.add_argument("--workload", default="sphere",
                    choices=["sphere", "cavities", "poisson", "poiseuille", "warmstart", "grid", "lpt", "accuracy", "sweep", "debye"],
                    help="the headline sphere workload, or one of the other configurations (one JSON line each)")
    ap.add_argument("--max-steps", type=int, default=400000, help="step bound of the Poisson-Boltzmann and warm-start solves")
    ap.add_argument("--ws-train", type=int, default=1024, help="warm start: training channels")
    ap.add_argument("--ws-train-steps", type=int, default=250000, help="warm start: FP32 steps per training field")
    ap.add_argument("--ws-epochs", type=int, default=60, help="warm start: training epochs")
    ap.add_argument("--ws-per-batch", type=int, default=32, help="warm start: training channels per Reynolds number")
    ap.add_argument("--ws-lr", type=float, default=1e-3, help="warm start: peak learning rate")
    ap.add_argument("--cavity-steps", type=int, default=2000, help="step bound of the cavities' convergence run")
    ap.add_argument("--cavity-check", type=int, default=1, help="cavities: also run a subset to convergence in FP64 and FP32 (1) or not (0)")
    ap.add_argument("--acc-full-steps", type=int, default=0, help="accuracy: only the full 512x256x256 box, to this many steps")
    ap.add_argument("--profile-case", default=None, choices=list(B_PER_CELL) + ["cavities", "poisson", "unet", "table"],
                    help="a small case for ncu captures, its measured launches inside the NVTX range 'profile': 4 steps of "
                         "a 256x128x128 version of the sphere workload in this storage; or 4 steps of 256 of the cavities; "
                         "or 4 steps of the D3Q7 Poisson-Boltzmann 256^3 case (FP32); or one training step of the U-Net "
                         "(batch 8, 128x512)")
    ap.add_argument("--kernel", default=None, choices=["thread", "staged", "paired", "rows"],
                    help="--profile-case: force this bulk kernel")
    ap.add_argument("--profile-size", default="small", choices=["small", "slab"],
                    help="--profile-case of the sphere: 256x128x128 (r=12), or a 512x256x64 slab of the full box (r=24): "
                         "full-length rows, state well above L2")
    args = ap.parse_args()
    if args.profile_case:
        print(json.dumps(profile_case(args)))
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "cavities" and int(os.environ.get("WORLD_SIZE", "1")) > 1:
        # independent cavities sharded over the ranks (no device collective)
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        line = cavities_run(args, dist)
        if dist.get_rank() == 0:
            print(json.dumps(line))
        dist.destroy_process_group()
        return
    if args.workload != "sphere":
        if int(os.environ.get("RANK", "0")) == 0:
            fn = {"cavities": cavities_run, "poisson": poisson_run, "poiseuille": poiseuille_run, "warmstart": warmstart_run,
                  "grid": grid_run, "lpt": lpt_run, "accuracy": accuracy_run, "sweep": sweep_run,
                  "debye": debye_run}[args.workload]
            # clocks sampled over the whole workload run (set-up included)
            with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
                line = fn(args)
            line["clocks"] = clk.summary()
            print(json.dumps(line))
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        cb = cpu_baseline(threads)
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "MLUPS", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "D3Q19 flow past a sphere (CPU sample)", "sample": cb["sample"]},
                "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "vs_baseline": None}
        print(json.dumps(line))
        return

    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    device = local
    case = sphere_case()
    cells = int(np.prod(case["shape"]))
    hbm, peak_kind = peaks()

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    # headline storage, resident in HBM
    barrier()
    with ClockSampler(device) as clk:
        s, tot_ms, ker_ms, launches = run_variant(args.storage, case, args.warmup, args.steps, device)
    barrier()
    tot_ms, mlups = job_throughput(tot_ms, cells, args.steps, dist, "cuda")
    kernel_avg_ms = ker_ms / launches
    achieved = B_PER_CELL[args.storage] * cells / (kernel_avg_ms / 1e3) / 1e9
    # kernels of the timed steps: the bulk step kernel each step, the outlet
    # ghost fill each step (open outlet), the boundary kernel on odd steps
    odd_steps = sum((args.warmup + k) & 1 for k in range(args.steps))
    timed_launches = args.steps * (2 if case["faces"][1] == "open" else 1) + odd_steps
    _, u_head = s.moments()
    tpb = s.threads_per_block()
    bulk_kernel = s.kernel()
    s.close()

    # the plain FP64 method and the other storages, same steps from the same start
    variants = {}
    ref64, t64, k64, n64 = run_variant("f64", case, args.warmup, args.steps, device)
    _, u64 = ref64.moments()
    ref64.close()
    variants["f64"] = {"mlups": cells * args.steps / (t64 / 1e3) / 1e6, "kernel_ms": k64 / n64}
    err_head = float(np.linalg.norm(u_head - u64) / np.linalg.norm(u64))
    del u_head
    if not args.quick:
        for st in ("f16dev", "f32", "bf16dev", "e3m12dev"):
            if st == args.storage:
                continue
            v, tt, kk, nn = run_variant(st, case, args.warmup, args.steps, device)
            _, uu = v.moments()
            v.close()
            variants[st] = {"mlups": cells * args.steps / (tt / 1e3) / 1e6, "kernel_ms": kk / nn,
                            "vel_rel_l2_vs_f64": float(np.linalg.norm(uu - u64) / np.linalg.norm(u64))}
            del uu
    del u64

    # mass conservation per storage and the error after a long run (reported;
    # a failure here never costs the line)
    try:
        drift = mass_drift(case["tau"], device)
    except Exception as exc:
        drift = {"error": str(exc)[:200]}
    try:
        long_acc = long_horizon_accuracy(device)
    except Exception as exc:
        long_acc = {"error": str(exc)[:200]}

    # end to end through the C ABI with host buffers
    from lbm_gb300.solver import BoxSolver

    e = BoxSolver(D3Q19, case["shape"], 1.0 / case["tau"], args.storage, faces=case["faces"], flags=case["flags"],
                  inlet_velocity=case["inlet"], init_velocity=case["init"], device=device)
    host = torch.empty((19, cells), dtype=torch.float64, pin_memory=True).numpy()
    w = np.array([1 / 18] * 6 + [1 / 36] * 12 + [1 / 3])
    host[:] = w[:, None]
    e.set_populations(host)
    e.step(args.warmup)
    barrier()
    t0 = time.perf_counter()
    e.set_populations(host)  # H2D of the job's input state
    t_up = time.perf_counter()
    e.step(2)  # the residual needs two steps of history after a state upload
    e.residual()
    for _ in range(args.steps - 2):
        e.step(1)
        e.residual()  # D2H of the step's result
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    wall = t1 - t0
    e.close()
    e2e = {"value": cells * args.steps * world / wall / 1e6, "unit": "MLUPS",
           "h2d_bytes_per_step": int(host.nbytes // args.steps), "d2h_bytes_per_step": 8 * 4,
           "steps": args.steps, "upload_ms": (t_up - t0) * 1e3, "upload_gbs": host.nbytes / (t_up - t0) / 1e9,
           "step_and_residual_ms": (t1 - t_up) * 1e3 / args.steps}
    del host

    line = {
        # the headline metric names the FP16 storage; another --storage names its own
        "metric": METRIC if args.storage == "f16dev" else METRIC.replace("FP16-deviation storage", f"{args.storage} storage"),
        "value": mlups,
        "unit": "MLUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": tot_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "D3Q19 flow past a sphere 512x256x256, r=24 at (128,128,128), eq. inlet u=0.05, zero-gradient outlet, "
                               "free-slip sides", "tau": case["tau"], "storage": args.storage, "cells": cells,
                   "bytes_per_cell": B_PER_CELL[args.storage], "l2": "state larger than L2 (no flush needed)",
                   "parallelism": "replicas" if world > 1 else "single GPU", "threads_per_block": tpb,
                   "bulk_kernel": bulk_kernel},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": PROFILED_TRAFFIC_PER_STEP.get(args.storage),
                     "traffic_source": "ncu capture of the bulk step kernel (dram__bytes_read.sum + dram__bytes_write.sum) on the "
                                       "512x256x64 slab of this workload, scaled by cells to the full box; recorded with the source, "
                                       "not measured in this run", "algorithmic_bytes": B_PER_CELL[args.storage] * cells,
                     "peak_kind": peak_kind, "kernel": "AA step (the bulk kernel the autotuner picked: k_box_rows, k_box_bulk_lean or k_box_tma; + k_box_bnd, "
                               "k_box_outlet)",
                     "kernel_avg_ms": kernel_avg_ms},
        "accuracy": {"vel_rel_l2_vs_f64": err_head, "after_steps": args.warmup + 2 * args.steps,
                     "start": "free stream (equilibrium at the inlet velocity)",
                     "vel_rel_l2_vs_f64_long": long_acc,
                     "mass_drift_per_1e5_steps": drift,
                     "mass_drift_case": "closed D3Q19 sphere channel 96x64x64, periodic x, free-slip sides, u0 = 0.05"},
        "variants": variants,
        "gpu_launches": timed_launches,
        "e2e": e2e,
        "clocks": clk.summary(),
    }
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(threads)
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
