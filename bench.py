#!/usr/bin/env python
"""Benchmark of the GB300 HPS solver: prints ONE JSON line.

Workload (default): uniform quadtree of level 7 with 16x16-cell patches (2048^2 = 4.19 M dofs),
Poisson on [-1,1]^2; each step is one request -- a seeded load f (sum of 8 Gaussian bumps) and
Dirichlet data (6 Fourier modes per side) -- solved on the factored tree: upwards stage (leaf
particular Neumann data + merges of h), root Dirichlet data, downwards stage (u_Gamma = S g + w)
and leaf solves.  The build stage (leaf DtN + all merges) is timed once and reported as build_s.

  value  -- solves/s with the inputs resident in HBM (device-to-device staging of each request)
  e2e    -- solves/s through the reference-facing C ABI with pinned host buffers: upwards(f_host),
            solve(a, b, r host), get_leaf_u(u_host) per step
  --impl reference -- the FP64 CPU oracle (a restatement of the reference's HPS path, same LAPACK
            calls) on the same workload, rank 0 only, on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "build s + solves/s, Mdof/s, p50/p99 vs plain FP64 GPU HPS at ≤1e-10 rel err"
DOM = (-1.0, 1.0, -1.0, 1.0)


# ------------------------------------------------------------------------------------------------
# synthetic requests (config-4 style): f = 8 Gaussian bumps, g = 6 Fourier modes per side
# ------------------------------------------------------------------------------------------------
def make_request(seed, X, Y, bpts):
    rng = np.random.default_rng(seed)
    amp = rng.uniform(-1, 1, 8)
    cx = rng.uniform(-1, 1, 8)
    cy = rng.uniform(-1, 1, 8)
    wd = rng.uniform(0.05, 0.3, 8)
    co = rng.standard_normal((4, 6))
    f = np.zeros_like(X)
    for k in range(8):
        f += amp[k] * np.exp(-((X - cx[k]) ** 2 + (Y - cy[k]) ** 2) / wd[k] ** 2)
    r = []
    for side, (x, y) in enumerate(bpts):
        t = y if side < 2 else x
        r.append(sum(co[side, m] * np.sin((m + 1) * np.pi * (t + 1) / 2) for m in range(6)))
    r = np.concatenate(r)
    return f, np.ones_like(r), np.zeros_like(r), r


def workload_desc(level, n):
    N = n * 2 ** level
    return (f"uniform quadtree level {level}, {n}x{n} cells per patch ({N}^2 = {N * N / 1e6:.2f} M dofs), "
            f"Poisson on [-1,1]^2, one right-hand side per step (Gaussian-bump load, Fourier Dirichlet data)")


# ------------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ------------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id=None):
        self.proc = None
        self.lines = []
        self.gpu_id = gpu_id

    def start(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.gpu_id:
            cmd += ["-i", self.gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------------
# CPU oracle runs (cpu_baseline leg and --impl reference)
# ------------------------------------------------------------------------------------------------
def cpu_sample(level, n, leaf_sample=256, seed=0, build=False):
    """Seconds of one literal solve (upwards + solve stages) -- and optionally of the build -- of
    the FP64 CPU oracle on the uniform level-`level` tree, measured on a sample and scaled by node
    counts: per tree level the oracle's own upwards4to1 + split1to4 (merge4to1 for the build) on
    a few nodes (after one untimed warm-up node) with synthetic operators of the exact sizes, the
    leaf particular-Neumann
    and leaf solves (buildD2N for the build) on `leaf_sample` leaves, and the full dense root
    solve of HPSAlgorithm.hpp:402-420 once."""
    from oracle import hps_oracle as O
    rng = np.random.default_rng(seed)
    h0 = 2.0 / 2 ** level
    grid = O.FiniteVolumeGrid(n, -1.0, -1.0 + h0, n, -1.0, -1.0 + h0)
    solver = O.FiniteVolumeSolver(solver_type=O.FISHPACK90)
    nleaf = 4 ** level
    kl = min(leaf_sample, nleaf)
    F = rng.standard_normal((kl, n * n))
    G = rng.standard_normal((kl, 4 * n))
    solver.solve(grid, G[0], F[0])  # LU of the leaf operator (part of the build)
    t0 = time.perf_counter()
    for k in range(kl):
        solver.particularNeumannData(grid, F[k])
        solver.solve(grid, G[k], F[k])
    t_solve = (time.perf_counter() - t0) * nleaf / kl
    t_build = 0.0
    if build:
        t0 = time.perf_counter()
        for k in range(min(kl, 16)):
            solver.buildD2N(grid)
        t_build += (time.perf_counter() - t0) * nleaf / min(kl, 16)
    hps = O.HPSAlgorithm(None, solver)
    for lvl in range(level - 1, -1, -1):
        s = n * 2 ** (level - 1 - lvl)
        cnt = 4 ** lvl
        kn = min(cnt, 32 if s <= 64 else (4 if s <= 256 else 1))
        for k in range(-1, kn):  # k = -1: untimed warm-up node
            w = 0.0 if k < 0 else 1.0
            kids = []
            for c in range(4):
                p = O.FiniteVolumePatch(O.FiniteVolumeGrid(s, 0, 1, s, 0, 1))
                p.T = rng.standard_normal((4 * s, 4 * s)) + 8.0 * np.eye(4 * s)
                p.h = rng.standard_normal(4 * s)
                kids.append(p)
            tau = O.FiniteVolumePatch(O.FiniteVolumeGrid(2 * s, 0, 1, 2 * s, 0, 1))
            if build:
                t0 = time.perf_counter()
                hps.merge4to1(tau, *kids)
                t_build += w * (time.perf_counter() - t0) * cnt / kn
            else:
                tau.S = rng.standard_normal((4 * s, 8 * s))
                tau.H = rng.standard_normal((8 * s, 4 * s))
            tau.g = rng.standard_normal(8 * s)
            t0 = time.perf_counter()
            hps.upwards4to1(tau, *kids)
            hps.split1to4(tau, *kids)
            t_solve += w * (time.perf_counter() - t0) * cnt / kn
    M = n * 2 ** level
    root = O.FiniteVolumePatch(O.FiniteVolumeGrid(M, -1, 1, M, -1, 1))
    root.T = rng.standard_normal((4 * M, 4 * M)) + 8.0 * np.eye(4 * M)
    root.h = rng.standard_normal(4 * M)
    ones, zeros = np.ones(4 * M), np.zeros(4 * M)
    t0 = time.perf_counter()
    hps.root_dirichlet(root, ones, zeros, rng.standard_normal(4 * M))
    t_solve += time.perf_counter() - t0
    return t_solve, t_build


CPU_SAMPLE_DESC = ("literal FP64 oracle (numpy/LAPACK restatement of the reference's HPS path, BLAS threads "
                   "= host cores) timed per step on a sample: per tree level upwards4to1 + split1to4 on 1-32 "
                   "nodes (after a warm-up node) with operators of the exact sizes, 256 leaves of particular-Neumann + leaf solves, "
                   "and the full dense root solve; scaled to the whole tree by node counts")


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    level, n = args.level, args.n
    _, tb = cpu_sample(level, n, build=True)
    for i in range(args.warmup):
        cpu_sample(level, n, seed=i)
    per = []
    t0 = time.perf_counter()
    for i in range(args.steps):
        ts, _ = cpu_sample(level, n, seed=100 + i)
        per.append(ts)
    wall = time.perf_counter() - t0
    v = args.steps / sum(per)
    dofs = (n * 2 ** level) ** 2
    out = {
        "metric": METRIC, "value": v, "unit": "solves/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sum(per) / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_desc(level, n), "leaves": 4 ** level, "dofs": dofs},
        "build_s": tb, "mdof_per_s": v * dofs / 1e6,
        "latency_ms": {"p50": float(np.percentile(per, 50) * 1e3), "p99": float(np.percentile(per, 99) * 1e3)},
        "cpu_baseline": {"value": v, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": CPU_SAMPLE_DESC, "build_s_extrapolated": tb, "wall_s": wall},
        "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------------------------------------
# GB300 arm
# ------------------------------------------------------------------------------------------------
def measure_fp64_peak(torch):
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2 * 4096 ** 3 / best / 1e12


# DRAM bytes per launch / algorithmic bytes per launch of the solve kernels, from one ncu capture
# of the same kernels on the uniform L6 tree (profiles/k_gemv_down_uniform_L6.md); L7 launches
# stream 4x the bytes of L6 launches with the same access pattern.
TRAFFIC_RATIO = {"downward": 1.005}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def run_gb300(args):
    import torch
    import torch.distributed as dist
    import ellipticforest_gb300 as ef
    from ellipticforest_gb300 import build as efbuild
    from ellipticforest_gb300.hps import kernel_launches

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    efbuild.build()
    stream = torch.cuda.current_stream()

    level, n = args.level, args.n
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, DOM[0], DOM[1], n, DOM[2], DOM[3]))
    mesh = ef.Mesh().uniform(level, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.set_stream(stream.cuda_stream)
    hps.setupStage()

    # build stage (timed once, sections profiled with CUDA events)
    hps.profile_enable(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hps.buildStage()
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    build_prof = hps.profile()
    hps.profile_reset()
    hps.profile_enable(False)
    build_flops = sum(v["flops"] for v in build_prof.values())

    # requests
    X, Y = mesh.cell_centres()
    bpts = hps.boundary_points()
    P = 4
    reqs = [make_request(1000 + i + 97 * rank, X, Y, bpts) for i in range(P)]
    dev = [tuple(torch.from_numpy(x).cuda() for x in rq) for rq in reqs]
    host = []
    for rq in reqs:
        hs = tuple(torch.from_numpy(x).pin_memory() for x in rq)
        host.append(tuple(h.numpy() for h in hs))
    u_host = torch.empty(X.size, dtype=torch.float64).pin_memory().numpy()
    dofs = X.size

    def device_step(i):
        f, a, b, r = dev[i % P]
        hps.load_device_async(f.data_ptr(), a.data_ptr(), b.data_ptr(), r.data_ptr())
        hps.solve_device_async(True)

    # warm-up
    for i in range(args.warmup):
        device_step(i)
    torch.cuda.synchronize()

    gpu_uuid = None
    try:
        gpu_uuid = str(torch.cuda.get_device_properties(local).uuid)
        if not gpu_uuid.startswith("GPU-"):
            gpu_uuid = "GPU-" + gpu_uuid
    except Exception:
        gpu_uuid = None
    clocks = ClockSampler(gpu_uuid)
    clocks.start()
    time.sleep(0.3)

    # timed region: exactly K device-resident steps
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    l0 = kernel_launches()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev[0].record(stream)
    for i in range(args.steps):
        device_step(i)
        ev[i + 1].record(stream)
    torch.cuda.synchronize()
    launches = kernel_launches() - l0
    lat = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    elapsed = ev[0].elapsed_time(ev[-1]) / 1e3
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
        dist.barrier()
    value = world * args.steps / elapsed

    # e2e through the reference-facing C ABI with pinned host buffers
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    from ellipticforest_gb300._lib import check, dptr, load
    lib = load()
    t0 = time.perf_counter()
    e0.record(stream)
    for i in range(args.steps):
        f, a, b, r = host[i % P]
        hps.upwards_array(f)
        hps.solve_arrays(a, b, r)
        check(lib.ef_hps_get_leaf_u(hps.handle, dptr(u_host)))
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_wall = time.perf_counter() - t0
    e2e_value = world * args.steps / max(e2e_wall, e0.elapsed_time(e1) / 1e3)
    clk = clocks.stop()

    # per-section kernel timing (CUDA events on the library's stream) over K profiled steps
    hps.profile_enable(True)
    hps.profile_reset()
    for i in range(args.steps):
        device_step(i)
    prof = hps.profile()
    hps.profile_enable(False)
    solve_secs = {k: v for k, v in prof.items()}
    tot_ms = sum(v["ms"] for v in solve_secs.values())
    dom_name = max(solve_secs, key=lambda k: solve_secs[k]["ms"])
    d = solve_secs[dom_name]
    hbm_peak, peak_kind = load_peaks()
    achieved = d["bytes"] / (d["ms"] / 1e3) / 1e9
    fp64_peak = measure_fp64_peak(torch)
    fp64_solve = sum(v["flops"] for v in solve_secs.values()) / (tot_ms / 1e3) / 1e12

    # correctness spot check on the manufactured solution u = sin x + sin y
    hps.upwards_array(-(np.sin(X) + np.sin(Y)))
    bx = np.concatenate([np.sin(x) + np.sin(y) for x, y in bpts])
    hps.solve_arrays(np.ones_like(bx), np.zeros_like(bx), bx)
    err = float(np.abs(hps.leaf_solution() - (np.sin(X) + np.sin(Y))).max())

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        _, cb = cpu_sample(level, n, build=True)
        cs = [cpu_sample(level, n, seed=7 + k)[0] for k in range(2)]
        cpu = {"value": len(cs) / sum(cs), "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
               "sample": CPU_SAMPLE_DESC + " (2 samples)", "build_s_extrapolated": cb}

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian-bump loads, Fourier Dirichlet data)",
            "config": {"workload": workload_desc(level, n), "leaves": 4 ** level, "dofs": dofs,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "operators (3.5 GiB) far exceed L2; every solve streams them from HBM"},
            "build_s": build_s, "mdof_per_s": value * dofs / 1e6,
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
            "e2e": {"value": e2e_value, "unit": "solves/s",
                    "h2d_bytes_per_step": int(8 * (dofs + 3 * 4 * hps.M)),
                    "d2h_bytes_per_step": int(8 * dofs)},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak,
                         "traffic": (TRAFFIC_RATIO[dom_name] * d["bytes"] / max(d["launches"], 1)
                                     if dom_name in TRAFFIC_RATIO else None),
                         "algorithmic_bytes_per_launch": d["bytes"] / max(d["launches"], 1),
                         "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                         "share_of_solve": d["ms"] / tot_ms},
            "fp64": {"solve_tflops": fp64_solve, "build_tflops": build_flops / build_s / 1e12,
                     "build_flops": build_flops, "dgemm_peak_tflops_measured": fp64_peak,
                     "build_frac_of_dgemm": build_flops / build_s / 1e12 / fp64_peak},
            "build_sections_ms": {k: v["ms"] for k, v in sorted(build_prof.items())},
            "kernels_ms_per_solve": {k: v["ms"] / args.steps for k, v in sorted(solve_secs.items())},
            "check_max_err_vs_exact": err,
            "clocks": clk,
        }
        if cpu:
            out["cpu_baseline"] = cpu
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--level", type=int, default=7)
    ap.add_argument("--n", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
