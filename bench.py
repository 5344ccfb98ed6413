#!/usr/bin/env python
"""Benchmark of the GB300 HPS solver: prints ONE JSON line.

Workload (default): uniform quadtree of level 7 with 16x16-cell patches (2048^2 = 4.19 M dofs),
Poisson on [-1,1]^2, requests = seeded loads f (sum of 8 Gaussian bumps) and Dirichlet data (6
Fourier modes per side).  The build stage (leaf DtN + all merges, FP64) is timed once (build_s).

  value  -- solves/s of the batched mixed-precision form: each step is one block of --batch
            requests solved on the factored tree by FP32 HPS passes (batched node GEMMs, FP32 leaf
            eigen-solves) with --sweeps refinement sweeps (exact fixed-point leaf residual + FP64
            interface flux mismatch), to <= 1e-10 relative of the FP64 HPS solution (rel_err_vs_fp64,
            measured); inputs resident in HBM; one lane by default (--lanes 2 or 3 alternate the
            steps over lanes sharing the operators, several blocks in flight: slower since the
            kernels fill the GPU on their own)
  e2e    -- the same form through the C ABI call ef_hps_mixed_solve_blocks on pinned host buffers
            (K blocks in one call, three lanes rotating so two blocks' copies overlap a third's
            solve), the host<->device copies of every block inside the timed region; the one-block
            ef_hps_mixed_solve rate is reported beside it
  plain_fp64 -- the plain FP64 form one request at a time (device-resident solves/s, p50/p99, and
            e2e through the reference-facing upwards/solve/get_leaf_u calls)
  many_rhs_L6 -- 512 right-hand sides on a uniform level-6 tree: one mixed block vs 512 plain solves
  adaptive_L7 -- config 2 (refineByFunction tree, 7 750 leaves): build, plain FP64 solves/s, error
            against the exact solution, and the mixed block form
  variable_coefficient_L5 -- config 3 (FivePointStencil leaves, variable beta): build, plain FP64
            solves/s, discretisation error, and the mixed block form against the FP64 HPS
  incremental_rebuild -- a localised mesh change re-merged from the config-2 tree vs a fresh build
  mixed_build -- FP32 merges with the interface LU of the top 3 levels in FP64 (uniform L7, config
            2): build seconds, the FP64 sweeps needed for 1e-10 and the block rate
  serving -- 2000 Poisson-arrival requests over three resident trees (uniform L4, adaptive max level
            7, uniform L7) through the serving loop (continuous same-tree batching, p50/p99 latency)
            against the same requests one at a time through the plain FP64 path
  --impl reference -- the FP64 CPU oracle (a restatement of the reference's HPS path, same LAPACK
            calls) on the same workload, rank 0 only, on the host cores.
"""
from __future__ import annotations

import argparse
import gc
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


def workload_desc(level, n, batch=1, sweeps=0):
    N = n * 2 ** level
    w = (f"uniform quadtree level {level}, {n}x{n} cells per patch ({N}^2 = {N * N / 1e6:.2f} M dofs), "
         f"Poisson on [-1,1]^2")
    if batch > 1 or sweeps:
        return w + (f"; each step one block of {batch} requests (Gaussian-bump loads, Fourier Dirichlet data) "
                    f"solved by FP32 HPS passes with {sweeps} refinement sweep(s) to <=1e-10 of the FP64 HPS")
    return w + ", one right-hand side per step (Gaussian-bump load, Fourier Dirichlet data)"


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


# DRAM bytes per launch / algorithmic bytes per launch of the solve kernels, from ncu captures of
# the same kernels on the uniform L6 tree (launches of 33.5 M cell-requests, far above L2); L7
# launches stream 4x the bytes of L6 launches with the same access pattern.
# Below 1 where part of a launch's inputs are still in L2 from the launch before it.
TRAFFIC_RATIO = {"downward": 1.005, "mx_leaf_residual": 0.934, "mx_leaf_solve": 0.90, "mx_leaf_first": 0.88}
# sections that launch one kernel (with at most a small reduction): the roofline's candidates
SINGLE_KERNEL = ("mx_leaf_first", "mx_leaf_residual", "mx_leaf_neumann", "mx_leaf_solve")


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _events(torch, k):
    return [torch.cuda.Event(enable_timing=True) for _ in range(k)]


def run_gb300(args):
    import torch
    import torch.distributed as dist
    import ellipticforest_gb300 as ef
    from ellipticforest_gb300 import build as efbuild
    from ellipticforest_gb300._lib import check, dptr, load
    from ellipticforest_gb300.hps import kernel_launches

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    efbuild.build()
    lib = load()
    stream = torch.cuda.current_stream()

    level, n, B, sweeps = args.level, args.n, args.batch, args.sweeps
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, DOM[0], DOM[1], n, DOM[2], DOM[3]))
    mesh = ef.Mesh().uniform(level, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.set_stream(stream.cuda_stream)
    hps.setupStage()

    # ---- build stage (timed once, sections profiled with CUDA events) ----
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

    X, Y = mesh.cell_centres()
    bpts = hps.boundary_points()
    dofs = X.size
    P = 4
    reqs = [make_request(1000 + i + 97 * rank, X, Y, bpts) for i in range(P)]  # (f, a, b, r)

    # ---- plain FP64 form, one request at a time, inputs resident in HBM ----
    dev = [tuple(torch.from_numpy(x).cuda() for x in rq) for rq in reqs]

    def plain_step(i):
        f, a, b, r = dev[i % P]
        hps.load_device_async(f.data_ptr(), a.data_ptr(), b.data_ptr(), r.data_ptr())
        hps.solve_device_async(True)

    for i in range(args.warmup):
        plain_step(i)
    torch.cuda.synchronize()
    Kp = args.plain_steps
    ev = _events(torch, Kp + 1)
    ev[0].record(stream)
    for i in range(Kp):
        plain_step(i)
        ev[i + 1].record(stream)
    torch.cuda.synchronize()
    plain_lat = [ev[i].elapsed_time(ev[i + 1]) for i in range(Kp)]
    plain_value = Kp / (ev[0].elapsed_time(ev[-1]) / 1e3)
    # FP64 reference solutions of the P distinct requests (also the plain form's e2e, through the
    # reference-facing upwards/solve/get_leaf_u calls with pinned host buffers)
    host = []
    for rq in reqs:
        hs = tuple(torch.from_numpy(x).pin_memory() for x in rq)
        host.append(tuple(h.numpy() for h in hs))
    u_host = torch.empty(dofs, dtype=torch.float64).pin_memory().numpy()
    ref_u = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(P):
        f, a, b, r = host[i]
        hps.upwards_array(f)
        hps.solve_arrays(a, b, r)
        check(lib.ef_hps_get_leaf_u(hps.handle, dptr(u_host)))
        ref_u.append(u_host.copy())
    plain_e2e = P / (time.perf_counter() - t0)
    # plain-form roofline: its dominant section over the plain steps
    hps.profile_enable(True)
    hps.profile_reset()
    for i in range(Kp):
        plain_step(i)
    plain_prof = hps.profile()
    hps.profile_reset()
    hps.profile_enable(False)
    p_tot = sum(v["ms"] for v in plain_prof.values())
    # the plain form's roofline: its largest operator-streaming section (the FP64 leaf passes are
    # bound by the FP64 pipe, not by HBM, and are reported in kernels_ms_per_solve)
    streaming = [k for k in ("downward", "upward_h", "upward_w") if k in plain_prof] or list(plain_prof)
    p_dom = max(streaming, key=lambda k: plain_prof[k]["ms"])
    p_ach = plain_prof[p_dom]["bytes"] / (plain_prof[p_dom]["ms"] / 1e3) / 1e9

    # ---- batched mixed-precision form: the headline ----
    check(lib.ef_hps_set_option(hps.handle, b"tensor-cores", args.tensor_cores))
    hps.mixed_init(B)
    F = np.stack([reqs[i % P][0] for i in range(B)])
    A = np.stack([reqs[i % P][1] for i in range(B)])
    R = np.stack([reqs[i % P][3] for i in range(B)])
    u_mixed = hps.mixed_solve(F, A, R, sweeps)  # also leaves the block's inputs resident in HBM
    rel_err = max(float(np.abs(u_mixed[i] - ref_u[i]).max() / np.abs(ref_u[i]).max()) for i in range(P))
    # with two lanes (the second shares the FP32 operators, own stream) two blocks are in flight: the
    # residual's integer work overlaps the other block's FP32 GEMM and leaf work.  Both lanes' inputs
    # are made resident by one two-block call, and lane 1 must give the same bits as lane 0.
    lanes = max(1, min(3, args.lanes))
    if lanes > 1:
        # the pipelined call leaves block k's inputs resident in lane k mod 3
        u2 = hps.mixed_solve_blocks([(F, A, R)] * lanes, sweeps)
        assert all(np.array_equal(x, u_mixed) for x in u2)
        lane_streams = [stream] + [torch.cuda.ExternalStream(hps.mixed_lane(k)[4]) for k in range(1, lanes)]
    else:
        lane_streams = [stream]
    for i in range(args.warmup):
        hps.mixed_solve_async(B, sweeps, lane=i % lanes)
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

    # timed region: exactly K device-resident steps, each one block of B requests, alternating over
    # the lanes; a block's latency is the time from the end of the previous block on its lane to its
    # own end
    K = args.steps
    ev = _events(torch, K + 1)
    ev_end = torch.cuda.Event(enable_timing=True)
    l0 = kernel_launches()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev[0].record(stream)
    for ls in lane_streams[1:]:
        ls.wait_event(ev[0])
    for i in range(K):
        hps.mixed_solve_async(B, sweeps, lane=i % lanes)
        ev[i + 1].record(lane_streams[i % lanes])
    for e in ev[max(1, K + 1 - lanes):]:
        stream.wait_event(e)
    ev_end.record(stream)
    torch.cuda.synchronize()
    launches = kernel_launches() - l0
    lat = [ev[max(0, i + 1 - lanes)].elapsed_time(ev[i + 1]) for i in range(K)]
    elapsed = ev[0].elapsed_time(ev_end) / 1e3
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
        dist.barrier()
    value = world * K * B / elapsed

    # e2e: the C ABI call a user makes (ef_hps_mixed_solve) on pinned host buffers, with the
    # host<->device copies of every block inside the timed region
    Fh = torch.from_numpy(F).pin_memory()
    Ah = torch.from_numpy(A).pin_memory()
    Rh = torch.from_numpy(R).pin_memory()
    Uh = [torch.empty_like(Fh).pin_memory() for _ in range(3)]
    Fn, An, Rn, Un = Fh.numpy(), Ah.numpy(), Rh.numpy(), [x.numpy() for x in Uh]
    # (1) one block per call (ef_hps_mixed_solve: copy in, solve, copy out, synchronise)
    Ke = max(2, K // 4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(Ke):
        check(lib.ef_hps_mixed_solve(hps.handle, B, sweeps, dptr(Fn), dptr(An), dptr(Rn), dptr(Un[0])))
    e2e_single = world * Ke * B / (time.perf_counter() - t0)
    assert np.array_equal(Un[0][0], u_mixed[0])
    # (2) the headline e2e: K blocks through one pipelined call (ef_hps_mixed_solve_blocks), every
    # block's inputs copied in and its results copied out inside the call; three lanes rotate so
    # that two blocks' copies overlap a third block's solve
    import ctypes as C
    nbk = K
    batch_arr = (C.c_int * nbk)(*([B] * nbk))
    f_arr = (C.c_void_p * nbk)(*([Fn.ctypes.data] * nbk))
    a_arr = (C.c_void_p * nbk)(*([An.ctypes.data] * nbk))
    r_arr = (C.c_void_p * nbk)(*([Rn.ctypes.data] * nbk))
    u_arr = (C.c_void_p * nbk)(*[Un[k % 3].ctypes.data for k in range(nbk)])  # one host output per lane
    # set-up and graph capture of the pipelined call's three lanes (two calls per lane)
    check(lib.ef_hps_mixed_solve_blocks(hps.handle, min(nbk, 6), batch_arr, sweeps, f_arr, a_arr, r_arr, u_arr))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    check(lib.ef_hps_mixed_solve_blocks(hps.handle, nbk, batch_arr, sweeps, f_arr, a_arr, r_arr, u_arr))
    e2e_wall = time.perf_counter() - t0
    e2e_value = world * nbk * B / e2e_wall
    clk = clocks.stop()
    assert all(np.array_equal(x[0], u_mixed[0]) for x in Un)

    # per-section kernel timing of the mixed form (CUDA events on the library's stream)
    hps.profile_enable(True)
    hps.profile_reset()
    for i in range(max(2, K // 4)):
        hps.mixed_solve_async(B, sweeps)
    prof = hps.profile()
    hps.profile_enable(False)
    ksteps = max(2, K // 4)
    tot_ms = sum(v["ms"] for v in prof.values())
    # the dominant kernel: the node-GEMM sections run several kernels (CUDA-core and tensor-core,
    # one launch per level); they are reported apart below
    dom_name = max((k for k in prof if k in SINGLE_KERNEL), key=lambda k: prof[k]["ms"])
    d = prof[dom_name]
    hbm_peak, peak_kind = load_peaks()
    achieved = d["bytes"] / (d["ms"] / 1e3) / 1e9
    fp64_peak = measure_fp64_peak(torch)

    # correctness spot check of the plain form on the manufactured solution u = sin x + sin y
    hps.upwards_array(-(np.sin(X) + np.sin(Y)))
    bx = np.concatenate([np.sin(x) + np.sin(y) for x, y in bpts])
    hps.solve_arrays(np.ones_like(bx), np.zeros_like(bx), bx)
    err = float(np.abs(hps.leaf_solution() - (np.sin(X) + np.sin(Y))).max())

    extras = {}
    if not args.no_extras:
        extras["many_rhs_L6"] = many_rhs(ef, torch, stream, args)
        c2 = build_config2(ef, torch, stream)
        extras["adaptive_L7"] = adaptive(ef, torch, stream, args, c2)
        extras["incremental_rebuild"] = incremental(ef, torch, stream, c2)
        extras["serving"] = serving(ef, torch, stream, (mesh, hps), args, c2)
        extras["mixed_build"] = mixed_build(ef, torch, stream, args, (mesh, hps, DOM, build_s),
                                            (c2[0], c2[1], (-10.0, 10.0, -10.0, 10.0), c2[2]))
        extras["variable_coefficient_L5"] = variable_coefficient(ef, torch, stream, args)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        _, cb = cpu_sample(level, n, build=True)
        cs = [cpu_sample(level, n, seed=7 + k)[0] for k in range(2)]
        cpu = {"value": len(cs) / sum(cs), "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
               "sample": CPU_SAMPLE_DESC + " (2 samples)", "build_s_extrapolated": cb}

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": K, "warmup": args.warmup, "ms_per_step": elapsed / K * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded Gaussian-bump loads, Fourier Dirichlet data)",
            "config": {"workload": workload_desc(level, n, B, sweeps), "leaves": 4 ** level, "dofs": dofs,
                       "batch": B, "sweeps": sweeps, "lanes_in_flight": lanes,
                       "rel_err_vs_fp64": rel_err, "tolerance": 1e-10,
                       "plain_fp64_solves_per_s": plain_value,
                       "speedup_vs_plain_fp64": value / plain_value,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "FP32 operators (1.75 GiB) and the block's leaf arrays far exceed L2"},
            "build_s": build_s, "mdof_per_s": value * dofs / 1e6,
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "note": "every request of a block completes with its block; with several lanes "
                                   "a block shares the GPU with the other lanes' blocks"},
            "rel_err_vs_fp64": rel_err,
            "speedup_vs_plain_fp64": value / plain_value,
            "plain_fp64": {
                "solves_per_s": plain_value, "mdof_per_s": plain_value * dofs / 1e6,
                "latency_ms": {"p50": float(np.percentile(plain_lat, 50)),
                               "p99": float(np.percentile(plain_lat, 99))},
                "e2e_solves_per_s": plain_e2e,
                "roofline": {"bound": "hbm", "kernel": p_dom, "achieved": p_ach, "peak": hbm_peak,
                             "unit": "GB/s", "frac": p_ach / hbm_peak,
                             "traffic": (TRAFFIC_RATIO[p_dom] * plain_prof[p_dom]["bytes"] /
                                         max(plain_prof[p_dom]["launches"], 1) if p_dom in TRAFFIC_RATIO else None),
                             "share_of_solve": plain_prof[p_dom]["ms"] / p_tot},
                "kernels_ms_per_solve": {k: v["ms"] / Kp for k, v in sorted(plain_prof.items())},
            },
            "e2e": {"value": e2e_value, "unit": "solves/s",
                    "h2d_bytes_per_step": int(B * 8 * (dofs + 2 * 4 * hps.M)),
                    "d2h_bytes_per_step": int(B * 8 * dofs),
                    "api": "ef_hps_mixed_solve_blocks (K blocks per call, three lanes, pinned host arrays)",
                    "one_block_per_call_solves_per_s": e2e_single},
            "gpu_launches": int(launches),
            "mixed_gemm_plan": {"columns": ["level", "s", "W", "H", "DOWN"],
                                "codes": "> 0: FP32 CUDA-core GEMM with that K split; < 0: tcgen05 GEMM, K split -code",
                                "groups": [list(r) for r in hps.mixed_gemm_plan()]},
            "build_merge_launches": hps.build_info()[0],
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak,
                         "traffic": (TRAFFIC_RATIO[dom_name] * d["bytes"] / max(d["calls"], 1)
                                     if TRAFFIC_RATIO.get(dom_name) else None),
                         "traffic_unit": "DRAM bytes per section call (its kernel launches of one step), "
                                         "the L6 ncu ratio of DRAM to algorithmic bytes applied to the L7 bytes",
                         "algorithmic_bytes_per_call": d["bytes"] / max(d["calls"], 1),
                         "launches_per_call": d["launches"] / max(d["calls"], 1),
                         "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                         "share_of_step": d["ms"] / tot_ms},
            "node_gemm_sections": {k: {"ms_per_step": prof[k]["ms"] / ksteps,
                                       "achieved_gbs": prof[k]["bytes"] / (prof[k]["ms"] / 1e3) / 1e9,
                                       "frac_of_hbm": prof[k]["bytes"] / (prof[k]["ms"] / 1e3) / 1e9 / hbm_peak,
                                       "launches_per_step": prof[k]["launches"] / ksteps}
                                   for k in ("mx_gemm_w", "mx_gemm_h", "mx_gemm_down") if k in prof},
            "fp64": {"build_tflops": build_flops / build_s / 1e12, "build_flops": build_flops,
                     "dgemm_peak_tflops_measured": fp64_peak,
                     "build_frac_of_dgemm": build_flops / build_s / 1e12 / fp64_peak},
            "build_sections_ms": {k: v["ms"] for k, v in sorted(build_prof.items())},
            "kernels_ms_per_step": {k: v["ms"] / ksteps for k, v in sorted(prof.items())},
            "kernels_tflops": {k: v["flops"] / (v["ms"] / 1e3) / 1e12 for k, v in sorted(prof.items()) if v["ms"]},
            "check_max_err_vs_exact": err,
            "clocks": clk,
        }
        out.update(extras)
        if cpu:
            out["cpu_baseline"] = cpu
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def make_request_box(seed, X, Y, bpts, box):
    """make_request on a tree over `box`: the bumps and modes live on the box mapped to [-1,1]^2."""
    x0, x1, y0, y1 = box
    sx = lambda x: 2 * (x - x0) / (x1 - x0) - 1
    sy = lambda y: 2 * (y - y0) / (y1 - y0) - 1
    return make_request(seed, sx(X), sy(Y), [(sx(x), sy(y)) for x, y in bpts])


def build_config2(ef, torch, stream):
    """Config-2 tree: refineByFunction(|sin x + sin y| > 1.2, min 0, max 7) on [-10,10]^2, 16x16
    patches, FISHPACK90 leaves; returns (mesh, hps, build seconds)."""
    rc = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, -10.0, 10.0, 16, -10.0, 10.0))
    mesh = ef.Mesh().refineByFunction(lambda x, y: abs(np.sin(x) + np.sin(y)) > 1.2, 1.2, 0, 7, rc)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.set_stream(stream.cuda_stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hps.buildStage()
    torch.cuda.synchronize()
    return mesh, hps, time.perf_counter() - t0


def adaptive(ef, torch, stream, args, c2):
    """Config 2: the adaptive tree with f = -(sin x + sin y), g = sin x + sin y: build, plain FP64
    solves/s and error against the exact solution, and the mixed block form against FP64."""
    mesh, hps, build_s = c2
    X, Y = mesh.cell_centres()
    bp = hps.boundary_points()
    f = -(np.sin(X) + np.sin(Y))
    r = np.concatenate([np.sin(x) + np.sin(y) for x, y in bp])
    a = np.ones_like(r)
    hps.upwards_array(f)
    hps.solve_arrays(a, np.zeros_like(a), r)
    u64 = hps.leaf_solution()
    err = float(np.abs(u64 - (np.sin(X) + np.sin(Y))).max())
    dev = tuple(torch.from_numpy(v).cuda() for v in (f, a, np.zeros_like(a), r))
    for _ in range(3):
        hps.load_device_async(*[t.data_ptr() for t in dev])
        hps.solve_device_async(True)
    torch.cuda.synchronize()
    K = 20
    e0, e1 = _events(torch, 2)
    e0.record(stream)
    for _ in range(K):
        hps.load_device_async(*[t.data_ptr() for t in dev])
        hps.solve_device_async(True)
    e1.record(stream)
    torch.cuda.synchronize()
    plain = K / (e0.elapsed_time(e1) / 1e3)
    B = 32
    reqs = [(f, a, r)]
    for i in range(3):
        fq, aq, _, rq = make_request_box(8000 + i, X, Y, bp, (-10.0, 10.0, -10.0, 10.0))
        reqs.append((fq, aq, rq))
    refs = []
    for q in reqs:
        hps.upwards_array(q[0])
        hps.solve_arrays(q[1], np.zeros_like(q[1]), q[2])
        refs.append(hps.leaf_solution())
    F = np.stack([reqs[i % 4][0] for i in range(B)])
    A = np.stack([reqs[i % 4][1] for i in range(B)])
    R = np.stack([reqs[i % 4][2] for i in range(B)])
    hps.mixed_init(B)
    U = hps.mixed_solve(F, A, R, args.adaptive_sweeps)
    errs = [float(np.abs(U[i] - refs[i]).max() / np.abs(refs[i]).max()) for i in range(4)]
    hps.mixed_solve_async(B, args.adaptive_sweeps)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(3):
        hps.mixed_solve_async(B, args.adaptive_sweeps)
    e1.record(stream)
    torch.cuda.synchronize()
    mixed = 3 * B / (e0.elapsed_time(e1) / 1e3)
    hps.mixed_init(1)  # release the block's memory
    return {"workload": "config 2: refineByFunction(|sin x + sin y| > 1.2, 0, 7) on [-10,10]^2, 16x16 patches, "
                        "f = -(sin x + sin y), g = sin x + sin y",
            "leaves": hps.num_leaves, "dofs": int(X.size), "build_s": build_s,
            "plain_fp64_solves_per_s": plain, "max_err_vs_exact": err,
            "mixed_block": {"batch": B, "sweeps": args.adaptive_sweeps, "solves_per_s": mixed,
                            "speedup_vs_plain": mixed / plain, "rel_err_vs_fp64_per_request": errs}}


def mixed_build(ef, torch, stream, args, main, c2):
    """Mixed-precision build (FP32 merges, interface LU of the top 3 levels in FP64) of the uniform
    L7 tree and of the config-2 tree: build seconds and TFLOP/s, the fewest FP64 sweeps that keep
    every result within 1e-10 of the FP64-built tree's solution, and the block rate at that count."""
    out = {}
    for name, (mesh64, hps64, box, build64_s) in (("uniform_L7", main), ("adaptive_L7", c2)):
        root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, box[0], box[1], 16, box[2], box[3]))
        mesh = (ef.Mesh().uniform(7, root) if name == "uniform_L7" else
                ef.Mesh().refineByFunction(lambda x, y: abs(np.sin(x) + np.sin(y)) > 1.2, 1.2, 0, 7, root))
        hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
        hps.set_stream(stream.cuda_stream)
        hps.profile_enable(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hps.buildStageMixed(3)
        torch.cuda.synchronize()
        tb = time.perf_counter() - t0
        prof = hps.profile()
        hps.profile_enable(False)
        flops = sum(v["flops"] for v in prof.values())
        X, Y = mesh.cell_centres()
        bp = hps.boundary_points()
        reqs = [make_request_box(6000 + i, X, Y, bp, box) for i in range(4)]
        refs = []
        for f, a, b, r in reqs:
            hps64.upwards_array(f)
            hps64.solve_arrays(a, b, r)
            refs.append(hps64.leaf_solution())
        B = 32
        F = np.stack([reqs[i % 4][0] for i in range(B)])
        A = np.stack([reqs[i % 4][1] for i in range(B)])
        R = np.stack([reqs[i % 4][3] for i in range(B)])
        hps.mixed_init(B)
        sweeps, err = None, None
        for sw in (2, 3, 4):
            U = hps.mixed_solve(F, A, R, sw)
            err = max(float(np.abs(U[i] - refs[i]).max() / np.abs(refs[i]).max()) for i in range(4))
            if err <= 1e-10:
                sweeps = sw
                break
        rate = None
        if sweeps is not None:
            hps.mixed_solve_async(B, sweeps)
            torch.cuda.synchronize()
            e0, e1 = _events(torch, 2)
            e0.record(stream)
            for _ in range(3):
                hps.mixed_solve_async(B, sweeps)
            e1.record(stream)
            torch.cuda.synchronize()
            rate = 3 * B / (e0.elapsed_time(e1) / 1e3)
        out[name] = {"build_s": tb, "fp64_build_s": build64_s, "build_speedup": build64_s / tb,
                     "build_tflops": flops / tb / 1e12, "fp64_levels": 3,
                     "sections_ms": {k: v["ms"] for k, v in sorted(prof.items())},
                     "sweeps_for_1e-10": sweeps, "rel_err_vs_fp64": err, "block_solves_per_s": rate}
        del hps
    return out


def incremental(ef, torch, stream, c2):
    """Local re-factorisation: the config-2 tree after an extra refined disk (a localised mesh change)
    built fresh and incrementally from the config-2 tree (operators of unchanged subtrees reused)."""
    _, old, _ = c2
    pred = lambda x, y: abs(np.sin(x) + np.sin(y)) > 1.2 or (x - 3.0) ** 2 + (y - 3.0) ** 2 < 0.5

    def tree():
        rc = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, -10.0, 10.0, 16, -10.0, 10.0))
        mesh = ef.Mesh().refineByFunction(pred, 1.2, 0, 7, rc)
        h = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
        h.set_stream(stream.cuda_stream)
        return mesh, h
    mesh, fresh = tree()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fresh.buildStage()
    torch.cuda.synchronize()
    t_fresh = time.perf_counter() - t0
    _, inc = tree()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reused = inc.buildStageFrom(old)
    torch.cuda.synchronize()
    t_inc = time.perf_counter() - t0
    same = bool(np.array_equal(fresh.root_T(), inc.root_T()))
    return {"workload": "config-2 tree plus a refined disk (x-3)^2+(y-3)^2 < 0.5 at level 7",
            "leaves": fresh.num_leaves, "merges": mesh.num_nodes() - mesh.num_leaves(), "reused_merges": reused,
            "fresh_build_s": t_fresh, "incremental_build_s": t_inc, "speedup": t_fresh / t_inc,
            "root_T_bit_identical": same}


def serving(ef, torch, stream, main_tree, args, c2):
    """Poisson-arrival stream of 2000 requests (seeded) over three resident trees -- uniform L4,
    the adaptive tree of refineByFunction(|sin x + sin y| > 1.2, 0, 7) on [-10,10]^2, uniform L7 --
    answered by the serving loop (continuous same-tree batching, two lanes per tree, HBM budget), against
    the same requests one at a time through the plain FP64 path's C ABI calls."""
    import threading
    from ellipticforest_gb300._lib import check, dptr, load
    lib = load()
    trees = []
    r4 = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, -1.0, 1.0, 16, -1.0, 1.0))
    m4 = ef.Mesh().uniform(4, r4)
    h4 = ef.HPSAlgorithm(m4, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    h4.set_stream(stream.cuda_stream)
    h4.buildStage()
    trees.append(("uniform L4", m4, h4, (-1.0, 1.0, -1.0, 1.0)))
    mc, hc, _ = c2
    trees.append((f"adaptive max_level 7 ({hc.num_leaves} leaves)", mc, hc, (-10.0, 10.0, -10.0, 10.0)))
    mesh7, h7 = main_tree
    trees.append(("uniform L7", mesh7, h7, DOM))
    T = len(trees)
    P = 6
    pool, outs = [], []
    RING = 64
    for t, (_, mesh, hps, box) in enumerate(trees):
        X, Y = mesh.cell_centres()
        bp = hps.boundary_points()
        reqs = []
        for i in range(P):
            f, a, b, r = make_request_box(7000 + 31 * t + i, X, Y, bp, box)
            reqs.append(tuple(torch.from_numpy(v).pin_memory().numpy() for v in (f, a, r)))
        pool.append(reqs)
        outs.append([torch.empty(X.size, dtype=torch.float64).pin_memory().numpy() for _ in range(RING)])
    rng = np.random.default_rng(2024)
    NREQ = 2000
    plan = [(int(rng.integers(0, T)), int(rng.integers(0, P))) for _ in range(NREQ)]
    budget = 64 << 30
    tree_sweeps = [args.sweeps, args.adaptive_sweeps, args.sweeps]
    srv = ef.Server([h for _, _, h, _ in trees], bmax=[32, 32, 32], lanes=2, hbm_budget_bytes=budget,
                    sweeps=tree_sweeps)
    lanes = [srv.lanes(t) for t in range(T)]

    def run_stream(rate):
        """Submit the plan at Poisson times of the given rate (inf: all at once); ring slots are
        reused once their previous request has completed."""
        ids = [None] * NREQ
        lat = [None] * NREQ
        slot_owner = [[None] * RING for _ in range(T)]
        counts = [0] * T
        gaps = rng.exponential(1.0 / rate, NREQ) if np.isfinite(rate) else np.zeros(NREQ)
        t0 = time.perf_counter()
        due = t0
        for k, (t, i) in enumerate(plan):
            due += gaps[k]
            while time.perf_counter() < due:
                pass
            s = counts[t] % RING
            counts[t] += 1
            prev = slot_owner[t][s]
            if prev is not None and lat[prev] is None:
                _, lat[prev] = srv.wait(ids[prev])
            f, a, r = pool[t][i]
            ids[k] = srv.submit(t, f, a, r, outs[t][s])
            slot_owner[t][s] = k
        for k in range(NREQ):
            if lat[k] is None:
                _, lat[k] = srv.wait(ids[k])
        wall = time.perf_counter() - t0
        return wall, np.array(lat)

    # warm-up (graphs captured for the block sizes that occur), then saturation, then the stream
    run_stream(float("inf"))
    wall_sat, _ = run_stream(float("inf"))
    sat = NREQ / wall_sat
    st0 = srv.stats()
    rate = 0.7 * sat
    wall, lat = run_stream(rate)
    st1 = srv.stats()
    # correctness: the last result of every tree against its plain FP64 solution
    errs = []
    for t, (_, mesh, hps, _) in enumerate(trees):
        k = max(j for j, (tt, _) in enumerate(plan) if tt == t)
        i = plan[k][1]
        s = (sum(1 for tt, _ in plan[:k] if tt == t)) % RING
        f, a, r = pool[t][i]
        hps.upwards_array(f)
        hps.solve_arrays(a, np.zeros_like(a), r)
        ref = hps.leaf_solution()
        errs.append(float(np.abs(outs[t][s] - ref).max() / np.abs(ref).max()))
    srv.close()
    # plain FP64 serial GPU path: the same requests one at a time through the C ABI
    u = [torch.empty(m.cell_centres()[0].size, dtype=torch.float64).pin_memory().numpy() for _, m, _, _ in trees]
    for t, (_, _, hps, _) in enumerate(trees):  # warm
        f, a, r = pool[t][0]
        hps.upwards_array(f)
        hps.solve_arrays(a, np.zeros_like(a), r)
    zeros = [np.zeros_like(pool[t][0][1]) for t in range(T)]
    plain_lat = []
    t0 = time.perf_counter()
    for t, i in plan:
        hps = trees[t][2]
        f, a, r = pool[t][i]
        ts = time.perf_counter()
        hps.upwards_array(f)
        hps.solve_arrays(a, zeros[t], r)
        check(lib.ef_hps_get_leaf_u(hps.handle, dptr(u[t])))
        plain_lat.append(time.perf_counter() - ts)
    plain_wall = time.perf_counter() - t0
    return {
        "workload": ("2000 requests, seeded Poisson arrivals at 0.7x the saturated rate, uniformly over 3 resident "
                     "trees: " + "; ".join(f"{nm} ({m.cell_centres()[0].size} dofs)" for nm, m, _, _ in trees)),
        "lanes_per_tree": lanes, "bmax": 32, "hbm_budget_bytes": budget, "sweeps_per_tree": tree_sweeps,
        "arrival_rate_per_s": rate, "solves_per_s": NREQ / wall,
        "latency_ms": {"p50": float(np.percentile(lat, 50) * 1e3), "p99": float(np.percentile(lat, 99) * 1e3)},
        "saturated_solves_per_s": sat,
        "blocks": st1["blocks"] - st0["blocks"], "max_block": st1["max_block"],
        "plain_fp64_serial": {"solves_per_s": NREQ / plain_wall,
                              "latency_ms": {"p50": float(np.percentile(plain_lat, 50) * 1e3),
                                             "p99": float(np.percentile(plain_lat, 99) * 1e3)}},
        "speedup_saturated_vs_plain_serial": sat / (NREQ / plain_wall),
        "rel_err_vs_fp64_last_per_tree": errs,
    }


def variable_coefficient(ef, torch, stream, args):
    """Config 3: alpha div(beta grad u) + lambda u = f on [-1,1]^2 with alpha = 1,
    beta = 1 + 0.5 sin(pi x) cos(pi y), lambda = -1, uniform level 5 of 32x32 FivePointStencil leaves
    (1024^2 dofs), manufactured u = sin(2 pi x) sin(pi y): build, plain FP64 solves and the mixed
    block form against the FP64 HPS per result."""
    PI = np.pi
    beta = lambda x, y: 1.0 + 0.5 * np.sin(PI * x) * np.cos(PI * y)
    solver = ef.FiniteVolumeSolver(alpha_function=lambda x, y: 1.0 + 0.0 * x, beta_function=beta,
                                   lambda_function=lambda x, y: -1.0 + 0.0 * x, solver_type=ef.FivePointStencil)
    uex = lambda x, y: np.sin(2 * PI * x) * np.sin(PI * y)

    def fex(x, y):
        bx = 0.5 * PI * np.cos(PI * x) * np.cos(PI * y)
        by = -0.5 * PI * np.sin(PI * x) * np.sin(PI * y)
        ux = 2 * PI * np.cos(2 * PI * x) * np.sin(PI * y)
        uy = PI * np.sin(2 * PI * x) * np.cos(PI * y)
        return beta(x, y) * (-5 * PI ** 2) * uex(x, y) + bx * ux + by * uy - uex(x, y)

    level, n = 5, 32
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, -1.0, 1.0, n, -1.0, 1.0))
    mesh = ef.Mesh().uniform(level, root)
    hps = ef.HPSAlgorithm(mesh, solver)
    hps.set_stream(stream.cuda_stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hps.buildStage()
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    X, Y = mesh.cell_centres()
    bp = hps.boundary_points()
    f = fex(X, Y)
    r = np.concatenate([uex(x, y) for x, y in bp])
    a = np.ones_like(r)
    hps.upwards_array(f)
    hps.solve_arrays(a, np.zeros_like(a), r)
    u64 = hps.leaf_solution()
    disc_err = float(np.abs(u64 - uex(X, Y)).max())
    dev = tuple(torch.from_numpy(v).cuda() for v in (f, a, np.zeros_like(a), r))
    for _ in range(3):
        hps.load_device_async(*[t.data_ptr() for t in dev])
        hps.solve_device_async(True)
    torch.cuda.synchronize()
    K = 10
    e0, e1 = _events(torch, 2)
    e0.record(stream)
    for _ in range(K):
        hps.load_device_async(*[t.data_ptr() for t in dev])
        hps.solve_device_async(True)
    e1.record(stream)
    torch.cuda.synchronize()
    plain = K / (e0.elapsed_time(e1) / 1e3)
    # mixed block: the manufactured request plus seeded bump/Fourier requests
    B = 16
    reqs = [(f, a, r)]
    for i in range(3):
        fq, aq, _, rq = make_request(9000 + i, X, Y, bp)
        reqs.append((fq, aq, rq))
    F = np.stack([reqs[i % 4][0] for i in range(B)])
    A = np.stack([reqs[i % 4][1] for i in range(B)])
    R = np.stack([reqs[i % 4][2] for i in range(B)])
    refs = []
    for q in reqs:
        hps.upwards_array(q[0])
        hps.solve_arrays(q[1], np.zeros_like(q[1]), q[2])
        refs.append(hps.leaf_solution())
    hps.mixed_init(B)
    U = hps.mixed_solve(F, A, R, args.sweeps)
    errs = [float(np.abs(U[i] - refs[i]).max() / np.abs(refs[i]).max()) for i in range(4)]
    hps.mixed_solve_async(B, args.sweeps)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(3):
        hps.mixed_solve_async(B, args.sweeps)
    e1.record(stream)
    torch.cuda.synchronize()
    mixed = 3 * B / (e0.elapsed_time(e1) / 1e3)
    return {"workload": "config 3: variable beta, lambda = -1, uniform level 5 of 32x32 FivePointStencil leaves "
                        "(1024^2 dofs), manufactured u = sin(2 pi x) sin(pi y)",
            "build_s": build_s, "plain_fp64_solves_per_s": plain, "max_err_vs_manufactured": disc_err,
            "mixed_block": {"batch": B, "sweeps": args.sweeps, "solves_per_s": mixed,
                            "speedup_vs_plain": mixed / plain, "rel_err_vs_fp64_per_request": errs}}


def many_rhs(ef, torch, stream, args):
    """512 right-hand sides on one factored uniform level-6 tree of 16x16 patches (1024^2 dofs):
    one mixed block of 512 against 512 plain FP64 solves one at a time."""
    level, n, nrhs = 6, 16, 512
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, DOM[0], DOM[1], n, DOM[2], DOM[3]))
    mesh = ef.Mesh().uniform(level, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.set_stream(stream.cuda_stream)
    hps.buildStage()
    X, Y = mesh.cell_centres()
    bpts = hps.boundary_points()
    P = 8
    reqs = [make_request(5000 + i, X, Y, bpts) for i in range(P)]
    F = np.stack([reqs[i % P][0] for i in range(nrhs)])
    A = np.stack([reqs[i % P][1] for i in range(nrhs)])
    R = np.stack([reqs[i % P][3] for i in range(nrhs)])
    ref = []
    for i in range(P):
        hps.upwards_array(reqs[i][0])
        hps.solve_arrays(reqs[i][1], reqs[i][2], reqs[i][3])
        ref.append(hps.leaf_solution())
    dev = [tuple(torch.from_numpy(x).cuda() for x in rq) for rq in reqs]
    for i in range(3):
        f, a, b, r = dev[i % P]
        hps.load_device_async(f.data_ptr(), a.data_ptr(), b.data_ptr(), r.data_ptr())
        hps.solve_device_async(True)
    torch.cuda.synchronize()
    e0, e1 = _events(torch, 2)
    e0.record(stream)
    for i in range(nrhs):
        f, a, b, r = dev[i % P]
        hps.load_device_async(f.data_ptr(), a.data_ptr(), b.data_ptr(), r.data_ptr())
        hps.solve_device_async(True)
    e1.record(stream)
    torch.cuda.synchronize()
    plain = nrhs / (e0.elapsed_time(e1) / 1e3)
    hps.mixed_init(nrhs)
    U = hps.mixed_solve(F, A, R, args.sweeps)
    err = max(float(np.abs(U[i] - ref[i]).max() / np.abs(ref[i]).max()) for i in range(P))
    hps.mixed_solve_async(nrhs, args.sweeps)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(3):
        hps.mixed_solve_async(nrhs, args.sweeps)
    e1.record(stream)
    torch.cuda.synchronize()
    mixed = 3 * nrhs / (e0.elapsed_time(e1) / 1e3)
    return {"workload": f"uniform level 6, 16x16 patches (1024^2 dofs), 512 right-hand sides, {args.sweeps} sweeps",
            "mixed_block_solves_per_s": mixed, "plain_fp64_serial_solves_per_s": plain,
            "speedup": mixed / plain, "rel_err_vs_fp64": err, "mdof_per_s": mixed * mesh.cell_centres()[0].size / 1e6}


def run_profile_only(args):
    """The build (or the mixed blocks) of the headline tree alone, for an ncu launch list."""
    import torch
    import ellipticforest_gb300 as ef
    from ellipticforest_gb300 import build as efbuild
    efbuild.build()
    stream = torch.cuda.current_stream()
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(args.n, DOM[0], DOM[1], args.n, DOM[2], DOM[3]))
    mesh = ef.Mesh().uniform(args.level, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.set_stream(stream.cuda_stream)
    hps.setupStage()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("build")  # ncu --nvtx --nvtx-include "build/"
    if args.profile_only == "mbuild":
        hps.buildStageMixed(3)
    else:
        hps.buildStage()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    out = {"profile_only": args.profile_only, "level": args.level, "build_merge_launches": hps.build_info()[0]}
    if args.profile_only == "mixed":
        X, Y = mesh.cell_centres()
        bpts = hps.boundary_points()
        reqs = [make_request(1000 + i, X, Y, bpts) for i in range(4)]
        B = args.batch
        F = np.stack([reqs[i % 4][0] for i in range(B)])
        A = np.stack([reqs[i % 4][1] for i in range(B)])
        R = np.stack([reqs[i % 4][3] for i in range(B)])
        from ellipticforest_gb300._lib import check as _check, load as _load
        _check(_load().ef_hps_set_option(hps.handle, b"tensor-cores", args.tensor_cores))
        if args.gemm_plan:
            # a plan timed in an earlier run without the profiler (under ncu the candidates' times
            # are those of serialised replays)
            hps.mixed_set_gemm_plan(json.loads(args.gemm_plan))
        hps.mixed_init(B)
        hps.mixed_solve(F, A, R, args.sweeps)
        torch.cuda.synchronize()
        # the steady-state blocks alone, for ncu --nvtx --nvtx-include "steady/"
        torch.cuda.nvtx.range_push("steady")
        for _ in range(args.steps):
            hps.mixed_solve_async(B, args.sweeps)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        out["gemm_plan"] = hps.mixed_gemm_plan()
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--level", type=int, default=7)
    ap.add_argument("--n", type=int, default=16)
    ap.add_argument("--batch", type=int, default=32, help="requests per block of the mixed form")
    ap.add_argument("--sweeps", type=int, default=1,
                    help="refinement sweeps of the mixed form on uniform trees (one keeps the L7 results "
                         "within 1e-10 of the FP64 HPS, and within 3e-11 of a sparse direct solve)")
    ap.add_argument("--lanes", type=int, default=1,
                    help="device-resident lanes of the headline, 1-3 (2: two blocks in flight on two streams)")
    ap.add_argument("--adaptive-sweeps", type=int, default=2,
                    help="refinement sweeps on the adaptive config-2 tree (one sweep leaves up to 2e-10 there)")
    ap.add_argument("--plain-steps", type=int, default=30, help="timed steps of the plain FP64 form")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the 512-RHS level-6 case")
    ap.add_argument("--tensor-cores", type=int, default=1, choices=[0, 1, 2],
                    help="node GEMMs of the mixed form: 0 CUDA cores, 1 the faster per level (tuned), 2 tcgen05 wherever supported")
    ap.add_argument("--gemm-plan", default=None,
                    help="--profile-only mixed: JSON node-GEMM plan (rows level, s, W, H, DOWN) instead of timing one")
    ap.add_argument("--profile-only", choices=["build", "mbuild", "mixed"], default=None,
                    help="short run for a profiler's launch list: 'build' = set-up and one FP64 build of the "
                         "tree; 'mbuild' = the mixed build (FP64 LU on the top 3 levels); 'mixed' = build, "
                         "block-solver set-up and --steps mixed blocks (no timing line)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    gc.disable()  # no collector pauses inside the timed loops (nothing here builds reference cycles)
    if args.impl == "reference":
        run_reference(args)
    elif args.profile_only:
        run_profile_only(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
