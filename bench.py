#!/usr/bin/env python
"""Benchmark of the PFEM per-time-step solve on one GB300.

Default workload (the largest configuration that fits one GPU): the 3D incompressible dam break
- 0.5 x 0.5 x 1.0 m water column in a 2.0 x 0.5 x 1.5 m tank, nodes on an h = 0.01 m lattice
jittered +-0.1h (seeded), Delaunay + alpha shape (alpha = 1.2): ~330k nodes, ~1.74M tetrahedra,
~1.3M unknowns; rho = 1000, mu = 1e-3, dt = 5e-4, PSPG P1-P1 Picard (residual Ax_f, minRes 1e-6,
maxIter 10).  One "step" is one Picard time step (MomContEqIncompNewton::solve without the host
remesh).  By default the mixed form runs: FP32 node-pair assembly and FP32 BiCGSTAB correction
solves (multigrid preconditioned) under FP64 iterative refinement of a matrix-free double-float
residual; --precision fp64 runs the plain FP64 form (FP64 assembly, block-Jacobi BiCGSTAB).
Every timed step starts from the state after the warm-up steps (no remesh inside the bench).
The line reports the error of the mixed form against the plain FP64 form with its linear solves
taken to relative residual 1e-14, the roofline of the Krylov SpMV and of the assembly, an e2e
figure through the C ABI with host buffers, and a time-bounded CPU sample of the oracle.

Other workloads (--workload): wc-c2 (2D weakly compressible dam break, h = 0.005, ~82k nodes:
explicit CDS_dpdt steps), wc-c2-batch (independent C2-sized WC meshes in one batched step),
incomp-c1 (2D incompressible, h = 0.05), batch-c4 (256 independent 2D instances in one batched
Picard step, sharded over ranks with --gpus N), serve-c5 (a Poisson request stream through the
server), heat-c3 (heat-equation steps on the C3 mesh).

Timing: W warm-up steps, then K steps, each timed with CUDA events on the library's own
stream, with a 256 MB write between steps to flush L2 (or inputs larger than L2).  --impl
reference times the CPU restatement of the reference's path (the FP64 C++/OpenMP oracle with
SciPy SuperLU/COLAMD, all host threads) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time-steps/s (2D WC dam break, CDS_dpdt explicit step)"
UNIT = "steps/s"
H = 0.005


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--cpu-sample-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=150.0,
                    help="incomp-c3: seconds the one-step CPU oracle sample may run before it is stopped")
    ap.add_argument("--workload", choices=["incomp-c3", "wc-c2", "wc-c2-batch", "incomp-c1", "batch-c4", "serve-c5",
                                           "heat-c3"],
                    default="incomp-c3",
                    help="incomp-c3 (default): PSPG Picard steps on the 3D dam break (~1.3M unknowns, the "
                         "largest single-GPU configuration); wc-c2: the 2D weakly compressible dam break; "
                         "wc-c2-batch: independent C2-sized WC meshes in one batched step; incomp-c1: PSPG "
                         "Picard steps on the small 2D dam break; batch-c4: 256 independent 2D instances; "
                         "serve-c5: a Poisson stream of requests served under an HBM budget; heat-c3: "
                         "heat-equation steps (problem Conduction) on the 3D dam-break mesh")
    ap.add_argument("--instances", type=int, default=256, help="batch-c4: number of instances")
    ap.add_argument("--wc-instances", type=int, default=32, help="wc-c2-batch: number of C2-sized meshes")
    ap.add_argument("--h", type=float, default=None,
                    help="incomp-c1 / incomp-c3: node spacing (default 0.05 / 0.01); smaller cases for profiling")
    ap.add_argument("--requests", type=int, default=24, help="serve-c5: number of requests")
    ap.add_argument("--rate", type=float, default=1.5, help="serve-c5: mean arrivals per second")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload_config(mesh, precision):
    return {
        "workload": "2D weakly compressible dam break (C2)",
        "h_m": H, "nodes": int(mesh.n_nodes), "elements": int(mesh.n_elems),
        "dof_per_step": int(3 * mesh.n_nodes), "state": "fp64",
        "element_arithmetic": precision, "dt": "adaptive CFL 0.3",
        "l2": "flushed between timed steps (256 MB write)", "remesh": "excluded (host side)",
        "parallelism": "replicas only",
    }


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(rows), "reasons": sorted(reasons)}


def wc_phase_bytes(d, N, E, r):
    """Algorithmic bytes per launch of each WC kernel.  Node state (x, v, p, rho, a) is FP64;
    element partials are r bytes (4 mixed, 8 plain) plus d(d+1) FP64 area gradients; int32
    connectivity and incidence lists, uint8 local indices and flags.  Each datum counted once."""
    inc = E * (d + 1)
    npe = d + 1
    el_cont = 2 * npe * r
    el_mom = (npe + d * npe) * r + d * npe * 8
    return {
        "WC predict": N * (3 * d * 8 + 16 * d + 1),
        "WC continuity element": E * npe * 4 + N * (8 * d + 8 * d + 8) + E * el_cont,
        "WC continuity node": E * el_cont + inc * 5 + (N + 1) * 4 + N + N * 24,
        "WC momentum element": E * npe * 4 + N * (8 * d + 8 * d + 16) + E * el_mom,
        "WC momentum node": E * el_mom + inc * 5 + (N + 1) * 4 + N + N * (8 * d + 16 + 8 * d) + N * 16 * d
                            + 2 * N * r,
        "WC time step": E * npe * 4 + N * 8 * d + 2 * N * r,
    }


def step_bytes(d, N, E, precision="fp64"):
    """Algorithmic bytes of one whole step: connectivity once, x, v, a, p, rho read and written
    once at their stored precision, flags once.  Plain form: all FP64.  Mixed form: x, v, p as
    double-float pairs (8 bytes a component), a and rho - rho* in FP32."""
    if precision == "fp64":
        per_node = (3 * d + 2) * 8
    else:
        per_node = 8 * d + 8 * d + 4 * d + 8 + 4
    return E * (d + 1) * 4 + 2 * N * per_node + N


def wc_phase_bytes_mixed(d, N, E):
    """Algorithmic bytes per launch of each of the four kernels of the mixed form: double-float
    x, v, p (8 bytes a component), FP32 rho - rho* and a; element->node records (2 floats for
    continuity, 2+3d useful floats for momentum) written once by the element kernels (int32
    slot map) and read once by the node kernels; int32 connectivity and incidence offsets, one
    flag byte per node.  The prediction (x, v, a read; x, v written) is counted in the
    continuity kernels, the CFL reduction in the momentum node kernel."""
    inc = E * (d + 1)
    npe = d + 1
    state_in = N * (8 * d + 8 * d + 4 * d + 8)          # x, v, a, p
    return {
        "WC continuity element": E * npe * 4 + N + state_in + inc * 4 + 2 * inc * 4,
        "WC continuity node": 2 * inc * 4 + (N + 1) * 4 + N + state_in + N * (16 * d + 8 + 4),
        "WC momentum element": E * npe * 4 + N * (8 * d + 4 * d + 8 + 4) + inc * 4 + (2 + 3 * d) * inc * 4,
        "WC momentum node": (2 + 3 * d) * inc * 4 + (N + 1) * 4 + N + N * (4 + 4 + 8 * d) + N * (4 * d + 8 * d),
    }


def time_oracle(mesh, s0, seconds, max_steps, threads=None):
    """Oracle WC steps (with the CFL dt update) for up to `seconds`; returns (steps, elapsed, threads)."""
    from oracle import oracle as O

    if threads:
        O.set_threads(threads)
    om = O.OracleMesh(mesh)
    p = O.wc_params()
    s = s0.copy()
    dt = O.wc_next_dt(om, p, s)
    O.wc_step(om, p, dt, s)  # warm caches / thread pool
    dt = O.wc_next_dt(om, p, s)
    n = 0
    t0 = time.perf_counter()
    while n < max_steps:
        O.wc_step(om, p, dt, s)
        dt = O.wc_next_dt(om, p, s)
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    return n, time.perf_counter() - t0, O.num_threads()


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from pfem_gb300 import mesh as M

    mesh = M.dam_break_2d(H)
    s0 = M.wc_initial_states(mesh)
    from oracle import oracle as O

    O.build()
    # warm-up steps untimed, then a bounded sample of K steps (at most ~120 s)
    time_oracle(mesh, s0, 1e9, max(0, min(args.warmup, 3)))
    n, el, thr = time_oracle(mesh, s0, 120.0, args.steps)
    v = n / el
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": n,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / n, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered lattice)",
        "config": workload_config(mesh, "fp64"),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": thr, "kind": "port",
                         "sample": f"{n} full C2 steps (the {args.steps} asked, capped at 120 s of CPU time)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(out))
    return 0


def run_gpu(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from pfem_gb300 import api, build
    from pfem_gb300 import mesh as M

    build.build()
    mesh = M.dam_break_2d(H)
    s0 = M.wc_initial_states(mesh)
    d, N, E = mesh.dim, mesh.n_nodes, mesh.n_elems
    prec = api.PREC_MIXED if args.precision == "fp32" else api.PREC_FP64
    rbytes = 4 if args.precision == "fp32" else 8

    def make(precision):
        p = api.default_params(api.KIND_WC_CDS_DPDT, 2)
        p.precision = precision
        ctx = api.Context(p)
        ctx.upload_mesh(mesh)
        ctx.set_states(s0)
        ctx.set_time(0.0, ctx.next_dt())
        return ctx

    ctx = make(prec)
    ext = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")  # 256 MB > 129 MB L2

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    # warm-up
    ctx.wc_step_async(0.0, args.warmup)
    ctx.synchronize()
    # timed region: K steps, L2 flushed between steps, events on the library stream
    K = args.steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    barrier()
    torch.cuda.synchronize()
    with torch.cuda.stream(ext):
        for k in range(K):
            flush.fill_(k & 0xFF)
            ev[k][0].record(ext)
            ctx.wc_step_async(0.0, 1)   # one CUDA-graph launch of the step's kernels
            ev[k][1].record(ext)
    st = ctx.synchronize()
    torch.cuda.synchronize()
    barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)

    # per-kernel durations: same steps launched without the graph, with the library's phase
    # timers (CUDA events on its stream) between kernels, L2 flushed between steps
    Kp = min(K, 500)
    ctx.set_profiling(True)
    ctx.reset_phase_times()
    with torch.cuda.stream(ext):
        for k in range(Kp):
            flush.fill_(k & 0xFF)
            ctx.wc_step_async(0.0, 1)
    ctx.synchronize()
    phases = ctx.phase_times()
    ctx.set_profiling(False)
    launches_per_step = sum(v[1] for v in phases.values()) / Kp
    if world > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * K / (total_ms / 1e3)

    # L2-resident throughput (steps back to back, no flush) for context
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(ext):
        e0.record(ext)
        ctx.wc_step_async(0.0, K)
        e1.record(ext)
    ctx.synchronize()
    warm_value = K / (e0.elapsed_time(e1) / 1e3)

    # end to end through the C ABI with host buffers
    nst = ctx.nstates * N
    h_in = torch.empty(nst, dtype=torch.float64, pin_memory=True).numpy()
    h_out = torch.empty(nst, dtype=torch.float64, pin_memory=True).numpy()
    h_in[:] = ctx.get_states()
    Ke = min(K, 300)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(Ke):
        ctx.set_states(h_in)
        ctx.wc_step(0.0, 1)
        ctx.get_states(out=h_out)
        h_in, h_out = h_out, h_in
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    clk = clocks.stop()

    # accuracy of the timed form against the FP64 plain form (fixed dt, same steps)
    acc = None
    if rank == 0:
        ref = make(api.PREC_FP64)
        tst = make(prec)
        dt0 = ref.next_dt()
        S = min(K, 2000)
        ref.wc_step(dt0, S)
        tst.wc_step(dt0, S)
        a, b = ref.get_states(), tst.get_states()
        names = ["vx", "vy", "p", "rho", "ax", "ay"]
        acc = {nm: float(np.linalg.norm(b[i * N:(i + 1) * N] - a[i * N:(i + 1) * N]) /
                         max(np.linalg.norm(a[i * N:(i + 1) * N]), 1e-300)) for i, nm in enumerate(names)}
        xa, xb = ref.get_positions(), tst.get_positions()
        acc["x"] = float(np.abs(xb - xa).max() / np.abs(xa).max())
        acc["mass_rel"] = abs(tst.mass() - ref.mass()) / ref.mass()
        acc["steps"] = S
        ref.close()
        tst.close()

    peak, peak_kind = hbm_peak()
    sb = step_bytes(d, N, E, args.precision)
    step_gbs = sb / (total_ms / K / 1e3) / 1e9
    # per kernel (one CUDA graph per step): the dominant one from the phase timers, with the
    # bytes it moves including its element->node records (implementation traffic)
    pb = wc_phase_bytes_mixed(d, N, E) if args.precision == "fp32" else wc_phase_bytes(d, N, E, rbytes)
    dom_name, (dom_ms, dom_n) = max(phases.items(), key=lambda kv: kv[1][0])
    dom_bytes = pb[dom_name]
    dom_us = 1e3 * dom_ms / dom_n
    gpu_launches = int(round(launches_per_step * K))
    achieved = dom_bytes / (dom_us / 1e6) / 1e9

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        n, el, thr = time_oracle(mesh, s0, args.cpu_sample_seconds, 100000)
        cpu = {"value": n / el, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{n} full C2 steps of the FP64 C++/OpenMP oracle ({el:.1f} s)"}

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": args.warmup,
            "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32" if args.precision == "fp32" else "f64",
            "data": "synthetic (seeded jittered lattice, no .msh shipped by the reference)",
            "config": workload_config(mesh, args.precision),
            "dof_per_s": value * 3 * N,
            "value_l2_resident": warm_value,
            "step_hbm_gbs": step_gbs,
            "e2e": {"value": Ke / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h_in.nbytes),
                    "d2h_bytes_per_step": int(h_out.nbytes)},
            "roofline": {"bound": "hbm", "kernel": "whole WC step (one CUDA graph of four kernels)",
                         "achieved": step_gbs, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": step_gbs / peak, "traffic": None, "algorithmic_bytes": sb,
                         "avg_launch_us": 1e3 * total_ms / K,
                         "dominant_kernel": {"kernel": dom_name, "achieved": achieved, "frac": achieved / peak,
                                             "bytes_with_records": dom_bytes, "avg_launch_us": dom_us,
                                             "traffic": NCU_TRAFFIC.get(("wc-c2", args.precision, dom_name))}},
            "phases_ms_per_step": {k: v[0] / max(v[1], 1) for k, v in phases.items()},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": gpu_launches,
            "err_vs_fp64": acc,
            "last_dt": st.dt,
        }
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_gpu_wc_batch(args):
    """Independent C2-sized weakly compressible dam breaks (per-instance seeds) in one mixed
    context: one launch sequence per step over all of them, each with its own CFL time step."""
    import numpy as np
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    from pfem_gb300 import api, build
    from pfem_gb300 import mesh as M

    build.build()
    n = args.wc_instances
    t0 = time.perf_counter()
    meshes = [M.dam_break_2d(H, seed=20261203 + i) for i in range(n)]
    mesh_s = time.perf_counter() - t0
    U, off = M.concat_meshes(meshes)
    s0 = M.concat_states([M.wc_initial_states(m) for m in meshes], meshes)
    N, E = U.n_nodes, U.n_elems
    p = api.default_params(api.KIND_WC_CDS_DPDT, 2)
    p.precision = api.PREC_MIXED
    ctx = api.Context(p)
    ctx.upload_mesh(U)
    ctx.set_instances(off, p.rho_star, p.mu)
    ctx.set_states(s0)
    ctx.next_dt()
    ext = torch.cuda.ExternalStream(ctx.stream)
    ctx.wc_step_batch(0.0, max(3, args.warmup))
    K = args.steps
    clocks = ClockSampler(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    torch.cuda.synchronize()
    clocks.start()
    with torch.cuda.stream(ext):  # the union's state (> L2) is streamed every step: no flush needed
        for k in range(K):
            ev[k][0].record(ext)
            ctx.wc_step_async(0.0, 1)
            ev[k][1].record(ext)
    sts = ctx.wc_step_batch(0.0, 0)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    ctx.set_profiling(True)
    ctx.reset_phase_times()
    ctx.wc_step_async(0.0, 5)
    ctx.synchronize()
    phases = ctx.phase_times()
    ctx.set_profiling(False)

    # end to end through the C ABI with host buffers (all instances' states in and out)
    h_in = torch.empty(ctx.nstates * N, dtype=torch.float64, pin_memory=True).numpy()
    h_out = torch.empty(ctx.nstates * N, dtype=torch.float64, pin_memory=True).numpy()
    h_in[:] = ctx.get_states()
    Ke = min(K, 20)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(Ke):
        ctx.set_states(h_in)
        ctx.wc_step_batch(0.0, 1)
        ctx.get_states(out=h_out)
    e2e_s = time.perf_counter() - t1

    # the batch against one instance run alone (same steps): bitwise
    solo_equal = None
    if rank == 0:
        pp = api.default_params(api.KIND_WC_CDS_DPDT, 2)
        pp.precision = api.PREC_MIXED
        solo = api.Context(pp)
        solo.upload_mesh(meshes[0])
        solo.set_states(M.wc_initial_states(meshes[0]))
        solo.next_dt()
        bt = api.Context(p)
        bt.upload_mesh(U)
        bt.set_instances(off, p.rho_star, p.mu)
        bt.set_states(s0)
        bt.next_dt()
        solo.wc_step(0.0, 20)
        bt.wc_step_batch(0.0, 20)
        solo_equal = bool(np.array_equal(solo.get_states(), M.split_states(bt.get_states(), meshes)[0]))
        solo.close()
        bt.close()

    peak, peak_kind = hbm_peak()
    sb = sum(step_bytes(2, m.n_nodes, m.n_elems, "fp32") for m in meshes)
    step_us = 1e3 * total_ms / K
    achieved = sb / (step_us / 1e6) / 1e9
    value = n * K / (total_ms / 1e3)
    if rank == 0:
        out = {
            "metric": f"instance-steps/s ({n} independent 2D WC dam breaks of C2 size, batched explicit step)",
            "value": value, "unit": "instance-steps/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
            "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32", "data": "synthetic (seeded jittered lattices, per-instance seeds)",
            "config": {"workload": f"{n} x 2D weakly compressible dam break (C2 size, h = {H})", "instances": n,
                       "nodes": int(N), "elements": int(E), "host_meshing_s": mesh_s,
                       "dt": "adaptive CFL 0.3 per instance", "l2": "working set > L2 (129 MB), no flush",
                       "parallelism": "one batched launch sequence"},
            "dof_per_s": value * 3 * N / n,
            "e2e": {"value": n * Ke / e2e_s, "unit": "instance-steps/s", "h2d_bytes_per_step": int(h_in.nbytes),
                    "d2h_bytes_per_step": int(h_out.nbytes)},
            "roofline": {"bound": "hbm", "kernel": "whole batched WC step (one CUDA graph)", "achieved": achieved,
                         "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "algorithmic_bytes": sb, "avg_launch_us": step_us},
            "phases_ms_per_step": {k: v[0] / 5 for k, v in phases.items()},
            "clocks": clk, "cpu_baseline": None,
            "gpu_launches": int(round(sum(v[1] for v in phases.values()) / 5 * K)),
            "instance0_bitwise_equal_to_solo_run": solo_equal,
            "dt_range": [min(st.dt for st in sts), max(st.dt for st in sts)],
        }
        print(json.dumps(out))
    return 0


# ------------------------------------------------------------------------------------------------
# Incompressible PSPG workloads: C1 (2D), C3 (3D) single meshes and C4 (batched 2D instances)
# ------------------------------------------------------------------------------------------------

INCOMP = {
    "incomp-c1": dict(dt=1e-3, column=(1.0, 2.0), max_steps=200, max_warmup=5,
                      metric="time-steps/s (2D incompressible dam break, PSPG Picard step)", unit="steps/s",
                      name="2D incompressible dam break (C1), h = 0.05"),
    "incomp-c3": dict(dt=5e-4, column=(0.5, 0.5, 1.0), max_steps=100, max_warmup=3,
                      metric="time-steps/s (3D incompressible dam break, PSPG Picard step)", unit="steps/s",
                      name="3D incompressible dam break (C3), h = 0.01"),
    "batch-c4": dict(dt=1e-3, max_steps=20, max_warmup=3,
                     metric="instance-steps/s (independent 2D incompressible dam breaks, batched Picard step)",
                     unit="instance-steps/s", name="batched 2D incompressible dam breaks (C4)"),
}


def incomp_params(api, dim, precision, workload, mu=1e-3):
    """C3's linear solves stop at relative residual 1e-8 (the configuration); the mixed form's
    FP64 refinement is taken to workloads.C3_MIXED_TOL so that its fields stay within 1e-6 of
    the FP64 reference (its inner FP32 solves are unchanged)."""
    from pfem_gb300 import workloads as WL

    p = api.default_params(api.KIND_INCOMP_PSPG, dim)
    p.precision = precision
    p.mu = mu
    if workload == "incomp-c3":
        p.krylov_rel_tol = WL.C3_MIXED_TOL if precision == api.PREC_MIXED else WL.C3_TOL
        p.krylov_abs_tol = 0.0
    elif workload == "batch-c4":
        p.krylov_rel_tol, p.krylov_abs_tol = WL.C4_TOL, 0.0
        p.krylov_max_iter = max(p.krylov_max_iter, 20000)
    return p


def linear_tolerance_text(workload, prec):
    from pfem_gb300 import api
    from pfem_gb300 import workloads as WL

    if workload == "incomp-c1":
        return "||r|| <= max(1e-14 ||b||, 1e-10)"
    tol = WL.C3_MIXED_TOL if prec == api.PREC_MIXED else WL.C3_TOL
    return f"||r|| <= {tol:g} ||b|| (FP64 residual)"


def pattern_nnz(mesh):
    from pfem_gb300 import mesh as M

    return M.pspg_nnz(mesh)


def node_pairs(mesh):
    """Node pairs sharing an element, each node with itself included: the scalar pattern."""
    import numpy as np
    import scipy.sparse as sp

    d, N, E = mesh.dim, mesh.n_nodes, mesh.n_elems
    inc = sp.csr_matrix((np.ones(E * (d + 1)), (np.repeat(np.arange(E), d + 1), mesh.conn.T.ravel())), shape=(E, N))
    return int((inc.T @ inc).tocsr().nnz)


def spmv_bytes(nnz, R, s):
    """One SpMV: values + column indices, row pointers, input and output vectors."""
    return nnz * (s + 4) + (R + 1) * 4 + 2 * R * s


def asm_bytes(d, N, E, R, nnz, s):
    """One assembly: connectivity, FP64 positions, current and previous velocities, flags, the
    CSR structure, the values and the right-hand side written once."""
    return E * (d + 1) * 4 + N * (d * 8 + 2 * d * s + 1) + (R + 1) * 4 + nnz * 4 + nnz * s + R * s


def field_errors(a, b, nf, N):
    import numpy as np

    return [float(np.linalg.norm(a[f * N:(f + 1) * N] - b[f * N:(f + 1) * N]) /
                  max(np.linalg.norm(b[f * N:(f + 1) * N]), 1e-300)) for f in range(nf)]


# DRAM bytes (read + write) of one launch of a kernel, from one ncu capture of the same
# workload (dram__bytes_read.sum + dram__bytes_write.sum; cold caches).
NCU_TRAFFIC = {
    ("wc-c2", "fp32", "WC momentum node"): 17.7664e6,
    ("wc-c2", "fp32", "WC momentum element"): 6.7676e6,
    ("wc-c2", "fp32", "WC continuity element"): 7.8026e6,
    ("wc-c2", "fp32", "WC continuity node"): 8.1851e6,
    # scaled from the h = 0.012 capture by nnz (189.4 MB x 66.96 / 39.16): node-pair blocks
    ("incomp-c3", "fp32", "Krylov SpMV"): 323.9e6,
    # one cold launch on the C3 heat system: 56.66 MB read + 0.24 MB written
    ("heat-c3", "fp64", "Heat CG SpMV"): 56.9e6,
}


def _spmv_work(ctx, phases, nnz, d):
    """Share of the full system one timed SpMV launch reads on average: converged instances of a
    batch drop out of the products, so launches late in a batched solve cover fewer rows."""
    n = phases.get("Krylov SpMV", (0.0, 0))[1]
    pairs = ctx.spmv_pairs()
    total = nnz // (d + 1) ** 2
    return pairs / (n * total) if n and pairs else 1.0


def _phase_roofline(phases, pb_spmv, pb_asm, peak):
    """Krylov SpMV (the dominant product) and the whole assembly: element prep, node kernel
    (diagonal blocks, right-hand side, scales, block inverses) and the pair kernel."""
    spmv_ms, spmv_n = phases.get("Krylov SpMV", (0.0, 0))
    asm_ms = sum(phases.get(k, (0.0, 0))[0] for k in ("PSPG element prep", "PSPG right-hand side", "PSPG matrix"))
    asm_n = max(phases.get("PSPG element prep", (0.0, 0))[1], 1)
    spmv_us = 1e3 * spmv_ms / max(spmv_n, 1)
    asm_us = 1e3 * asm_ms / asm_n
    out = {
        "bound": "hbm", "kernel": "Krylov SpMV", "achieved": pb_spmv / (spmv_us / 1e6) / 1e9 if spmv_n else None,
        "peak": peak, "unit": "GB/s", "algorithmic_bytes": pb_spmv, "avg_launch_us": spmv_us, "traffic": None,
    }
    out["frac"] = out["achieved"] / peak if out["achieved"] else None
    out["assembly"] = {"achieved": pb_asm / (asm_us / 1e6) / 1e9 if asm_us else None, "avg_us": asm_us,
                       "algorithmic_bytes": pb_asm,
                       "kernels_us": {k: 1e3 * phases[k][0] / max(phases[k][1], 1)
                                      for k in ("PSPG element prep", "PSPG right-hand side", "PSPG matrix")
                                      if k in phases}}
    if out["assembly"]["achieved"]:
        out["assembly"]["frac"] = out["assembly"]["achieved"] / peak
    return out


class _MarkTimes(dict):
    """Phase-time dict of the oracle's Picard step that also appends each update, with a
    timestamp, to a file: the parent of a time-bounded sample reads how far the step got."""

    def __init__(self, path):
        super().__init__()
        self.path = path

    def __setitem__(self, key, value):
        super().__setitem__(key, value)
        with open(self.path, "a") as f:
            f.write(f"{time.perf_counter():.6f}\t{key}\t{value:.6f}\n")


def _c3_cpu_child(h, path):
    """One oracle Picard step (FP64 C++/OpenMP assembly, SciPy SuperLU/COLAMD solve) on the C3
    mesh, in a child process so that the parent can stop it at its time budget."""
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    from pfem_gb300 import mesh as M
    from pfem_gb300 import workloads as WL

    mesh = WL.c3(h)
    q = M.incomp_initial_states(mesh, column=WL.C3_COLUMN)
    om = O.OracleMesh(mesh)
    with open(path, "a") as f:
        f.write(f"{time.perf_counter():.6f}\tstart\t{O.num_threads()}\n")
        f.write(f"{time.perf_counter():.6f}\tunknowns\t{(mesh.dim + 1) * mesh.n_nodes}\n")
    times = _MarkTimes(path)
    _, res = O.pspg_picard_step(om, q, WL.C3_DT, g=(0.0, 0.0, -9.81), times=times)
    with open(path, "a") as f:
        f.write(f"{time.perf_counter():.6f}\tdone\t{int(res.converged)}\n")


def c3_cpu_sample(h, budget_s):
    """Time one C3 Picard step of the oracle for at most budget_s seconds (mesh generation and
    oracle set-up excluded).  Returns (steps/s, cores, sample text, upper_bound): when the step
    does not finish in the budget, steps/s is 1 / (time spent so far), an upper bound."""
    import multiprocessing as mp

    fd, path = tempfile.mkstemp(suffix=".log")
    os.close(fd)
    proc = mp.get_context("spawn").Process(target=_c3_cpu_child, args=(h, path))
    t_launch = time.perf_counter()
    proc.start()
    t_start = None
    deadline = None
    while True:
        proc.join(timeout=1.0)
        lines = [ln.split("\t") for ln in open(path).read().splitlines() if ln.count("\t") == 2]
        if t_start is None and lines and lines[0][1] == "start":
            t_start = float(lines[0][0])
            deadline = time.perf_counter() + budget_s
        if not proc.is_alive():
            break
        if deadline is not None and time.perf_counter() > deadline:
            proc.terminate()
            proc.join(timeout=10)
            if proc.is_alive():
                proc.kill()
                proc.join()
            break
        if deadline is None and time.perf_counter() - t_launch > 600:  # set-up never finished
            proc.terminate()
            proc.join()
            break
    lines = [ln.split("\t") for ln in open(path).read().splitlines() if ln.count("\t") == 2]
    os.unlink(path)
    if not lines or lines[0][1] != "start":
        return None, 0, "C3 oracle set-up did not finish", True
    cores = int(float(lines[0][2]))
    t0 = float(lines[0][0])
    phases = {k: float(v) for _, k, v in lines[1:] if k not in ("done", "unknowns")}
    R = int(float(next((v for _, k, v in lines if k == "unknowns"), "0")))
    if any(k == "done" for _, k, _ in lines):
        el = float([t for t, k, _ in lines if k == "done"][0]) - t0
        return 1.0 / el, cores, f"one full C3 Picard step of the FP64 oracle ({el:.1f} s)", False
    el = max(budget_s, float(lines[-1][0]) - t0)
    got = ", ".join(f"{k} {v:.1f} s" for k, v in phases.items())
    return (1.0 / el, cores,
            f"one C3 Picard step of the FP64 C++/OpenMP oracle with SciPy SuperLU/COLAMD, stopped after {el:.0f} s "
            f"before it finished (phases completed: {got or 'none'}; SuperLU had not finished factorising the "
            f"{R}-unknown system), so the value is an upper bound on the CPU's steps/s", True)


def incomp_cfg(args):
    cfg = INCOMP[args.workload]
    if args.h is not None and args.workload in ("incomp-c1", "incomp-c3"):
        cfg = dict(cfg, name=cfg["name"].rsplit("h = ", 1)[0] + f"h = {args.h:g}")
    return cfg


def incomp_mesh(args):
    from pfem_gb300 import mesh as M
    from pfem_gb300 import workloads as WL

    if args.h is not None:
        return M.dam_break_2d(args.h) if args.workload == "incomp-c1" else M.dam_break_3d(args.h)
    return WL.c1() if args.workload == "incomp-c1" else WL.c3()


def run_gpu_incomp(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    from pfem_gb300 import api, build
    from pfem_gb300 import mesh as M
    from pfem_gb300 import workloads as WL

    build.build()
    if args.workload == "heat-c3":
        return run_gpu_heat(args)
    if args.workload == "batch-c4":
        return run_gpu_batch(args)
    if args.workload == "serve-c5":
        return run_gpu_serve(args)
    cfg = incomp_cfg(args)
    mesh = incomp_mesh(args)
    d, N, E = mesh.dim, mesh.n_nodes, mesh.n_elems
    R = (d + 1) * N
    nnz = pattern_nnz(mesh)
    q0 = M.incomp_initial_states(mesh, column=cfg["column"])
    dt = cfg["dt"]
    K = max(1, min(args.steps, cfg["max_steps"]))
    Wm = max(3, min(args.warmup, cfg["max_warmup"]))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")

    def make(precision):
        ctx = api.Context(incomp_params(api, d, precision, args.workload))
        ctx.upload_mesh(mesh)
        ctx.set_states(q0)
        return ctx

    # The bench does not remesh (the remesh is host work outside the path), and without it the
    # thinnest 3D elements invert after a few steps (the Picard step then fails, as the
    # reference's would): every timed step starts from the state after the warm-up steps.
    tuning = {}

    def run(precision, clocks=None):
        ctx = make(precision)
        ext = torch.cuda.ExternalStream(ctx.stream)
        for _ in range(Wm):
            ctx.picard_step(dt)
        x_w, q_w = ctx.get_positions(), ctx.get_states()
        if precision == api.PREC_MIXED:  # launch shapes for this device and mesh size
            from pfem_gb300 import tune

            def restore():
                ctx.set_positions(x_w)
                ctx.set_states(q_w)

            choice, src = tune.autotune(ctx, d, N, torch.cuda.get_device_name(local), lambda: ctx.picard_step(dt),
                                        restore)
            tuning.update(choice)
            tuning["source"] = src
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        stats = {"converged": 0, "picard_iterations": 0, "krylov_iterations": 0}
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        with torch.cuda.stream(ext):
            for k in range(K):
                ctx.set_positions(x_w)
                ctx.set_states(q_w)
                flush.fill_(k & 0xFF)
                ev[k][0].record(ext)
                st = ctx.picard_step(dt)
                ev[k][1].record(ext)
                stats["converged"] += st.converged
                stats["picard_iterations"] += st.picard_iterations
                stats["krylov_iterations"] += st.krylov_iterations
        torch.cuda.synchronize()
        clk = clocks.stop() if clocks else None
        ms = sum(a.elapsed_time(b) for a, b in ev)
        if stats["converged"] != K:
            raise RuntimeError(f"{K - stats['converged']} of {K} timed steps did not converge")
        return ctx, ms, stats, clk, (x_w, q_w)  # ctx holds the state one step after the warm-up

    prec = api.PREC_MIXED if args.precision == "fp32" else api.PREC_FP64
    clocks = ClockSampler(local)
    ctx, total_ms, stats, clk, (x_w, q_w) = run(prec, clocks)
    q_fast, x_fast = ctx.get_states(), ctx.get_positions()
    other = api.PREC_FP64 if prec == api.PREC_MIXED else api.PREC_MIXED
    ctx_o, ms_o, stats_o, _, _ = run(other)
    q_o, x_o = ctx_o.get_states(), ctx_o.get_positions()
    acc_vs_fp64 = acc_vs_other = None
    if prec == api.PREC_MIXED:
        acc_vs_other = dict(zip(["v" + "xyz"[i] for i in range(d)] + ["p"], field_errors(q_fast, q_o, d + 1, N)))
        acc_vs_other["x"] = float(np.abs(x_fast - x_o).max() / np.abs(x_o).max())
        acc_vs_other["steps"] = Wm + 1
        # the FP64 reference: the plain FP64 form with its linear solves taken to 1e-14 relative
        # residual (BiCGSTAB to the direct solver's accuracy), the same Wm + 1 steps from rest
        p_ref = incomp_params(api, d, api.PREC_FP64, args.workload)
        p_ref.krylov_rel_tol, p_ref.krylov_abs_tol, p_ref.krylov_max_iter = 1e-14, 0.0, 50000
        ctx_r = api.Context(p_ref)
        ctx_r.upload_mesh(mesh)
        ctx_r.set_states(q0)
        for _ in range(Wm + 1):
            if not ctx_r.picard_step(dt).converged:
                raise RuntimeError("FP64 reference step did not converge")
        q_r, x_r = ctx_r.get_states(), ctx_r.get_positions()
        ctx_r.close()
        acc_vs_fp64 = dict(zip(["v" + "xyz"[i] for i in range(d)] + ["p"], field_errors(q_fast, q_r, d + 1, N)))
        acc_vs_fp64["x"] = float(np.abs(x_fast - x_r).max() / np.abs(x_r).max())
        acc_vs_fp64["steps"] = Wm + 1
        acc_vs_fp64["reference"] = "plain FP64 form, linear solves to relative residual 1e-14"
    ctx_o.close()

    # per-phase times (library event timers, direct launches) on a few more steps from the warm
    # state, as the timed steps
    Kp = min(K, 3)
    x_s, q_s = x_w, q_w
    ctx.set_profiling(True)
    ctx.reset_phase_times()
    for _ in range(Kp):  # from the same state every time, as the timed steps
        ctx.set_positions(x_s)
        ctx.set_states(q_s)
        ctx.picard_step(dt)
    phases = ctx.phase_times()
    work = _spmv_work(ctx, phases, nnz, d)
    ctx.set_profiling(False)
    ctx.set_positions(x_s)
    ctx.set_states(q_s)
    s = 4 if prec == api.PREC_MIXED else 8
    peak, peak_kind = hbm_peak()
    roof = _phase_roofline(phases, spmv_bytes(nnz, R, s) * work, asm_bytes(d, N, E, R, nnz, s), peak)
    roof["peak_kind"] = peak_kind
    roof["spmv_work_fraction"] = work
    roof["traffic"] = NCU_TRAFFIC.get((args.workload, args.precision, "Krylov SpMV"))

    # end to end through the C ABI with host buffers: positions and states in, states out
    h_in = torch.empty(R, dtype=torch.float64, pin_memory=True).numpy()
    h_out = torch.empty(R, dtype=torch.float64, pin_memory=True).numpy()
    h_x = torch.empty(d * N, dtype=torch.float64, pin_memory=True).numpy()
    h_in[:] = ctx.get_states()
    h_x[:] = ctx.get_positions().ravel()
    Ke = min(K, 20)
    t0 = time.perf_counter()
    for _ in range(Ke):
        ctx.set_positions(h_x)
        ctx.set_states(h_in)
        ctx.picard_step(dt)
        ctx.get_states(out=h_out)
    e2e_s = time.perf_counter() - t0

    # the plain form with the device sparse LU (the reference's solver choice), same timed steps
    plain_lu = None
    if args.workload == "incomp-c1":
        p_lu = incomp_params(api, d, api.PREC_FP64, args.workload)
        p_lu.linear_solver = api.LINSOLVE_LU
        c_lu = api.Context(p_lu)
        c_lu.upload_mesh(mesh)
        c_lu.set_states(q0)
        for _ in range(Wm):
            c_lu.picard_step(dt)
        x_l, q_l = c_lu.get_positions(), c_lu.get_states()
        lu_ms = 0.0
        ext_l = torch.cuda.ExternalStream(c_lu.stream)
        for _ in range(K):
            c_lu.set_positions(x_l)
            c_lu.set_states(q_l)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(ext_l):
                e0.record(ext_l)
                c_lu.picard_step(dt)
                e1.record(ext_l)
            torch.cuda.synchronize()
            lu_ms += e0.elapsed_time(e1)
        plain_lu = {"solver": "device sparse LU (nested dissection, multifrontal, FP64)", "value": K / (lu_ms / 1e3),
                    "mixed_speedup": (K / (total_ms / 1e3)) / (K / (lu_ms / 1e3))}
        c_lu.close()

    cpu = None
    acc_vs_oracle = None
    if rank == 0 and not args.no_cpu_baseline and args.workload == "incomp-c3":
        v_cpu, cores, sample, upper = c3_cpu_sample(args.h or 0.01, args.cpu_budget)
        cpu = {"value": v_cpu, "unit": cfg["unit"], "cores": cores, "kind": "port", "sample": sample,
               "upper_bound": upper}
    if rank == 0 and not args.no_cpu_baseline and args.workload == "incomp-c1":
        from oracle import oracle as O

        O.build()
        om = O.OracleMesh(mesh)
        qo = q0.copy()
        g = (0.0, -9.81)
        t0 = time.perf_counter()
        n_cpu = 0
        q_cmp = x_cmp = None
        for k in range(Wm + K):
            qo, res = O.pspg_picard_step(om, qo, dt, g=g)
            n_cpu += 1
            if n_cpu == Wm + 1:  # the GPU's q_fast: one step after the warm-up steps
                q_cmp, x_cmp = qo.copy(), om.positions
        el = time.perf_counter() - t0
        cpu = {"value": n_cpu / el, "unit": cfg["unit"], "cores": O.num_threads(), "kind": "port",
               "sample": f"{n_cpu} C1 Picard steps of the FP64 C++/OpenMP oracle with SciPy SuperLU/COLAMD "
                         f"({el:.1f} s)"}
        acc_vs_oracle = dict(zip(["vx", "vy", "p"], field_errors(q_fast, q_cmp, 3, N)))
        acc_vs_oracle["x"] = float(np.abs(x_fast - x_cmp).max() / np.abs(x_cmp).max())
        acc_vs_oracle["steps"] = Wm + 1

    value = K / (total_ms / 1e3)
    if rank == 0:
        out = {
            "metric": cfg["metric"], "value": value, "unit": cfg["unit"], "n_gpus": world, "steps": K, "warmup": Wm,
            "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32" if prec == api.PREC_MIXED else "f64",
            "data": "synthetic (seeded jittered lattice, no .msh shipped by the reference)",
            "config": {"workload": cfg["name"], "nodes": N, "elements": E, "unknowns": R, "nnz": nnz, "dt": dt,
                       "precision": "mixed (FP32 assembly + FP32 BiCGSTAB, double-float refinement residual)"
                       if prec == api.PREC_MIXED else "plain FP64",
                       "linear_tolerance": linear_tolerance_text(args.workload, prec),
                       "l2": "flushed between timed steps (256 MB write)", "remesh": "excluded (host side)",
                       "timed_steps": "each from the state after the warm-up steps (positions and states "
                                      "restored outside the timed region; all converged)",
                       "parallelism": "replicas only"},
            "dof_per_s": value * R,
            "step_stats": stats,
            "other_precision": {"precision": "fp64" if prec == api.PREC_MIXED else "mixed",
                                "solver": "block-Jacobi BiCGSTAB" if prec == api.PREC_MIXED else "multigrid BiCGSTAB",
                                "value": K / (ms_o / 1e3), "step_stats": stats_o},
            "plain_lu": plain_lu,
            "e2e": {"value": Ke / e2e_s, "unit": cfg["unit"], "h2d_bytes_per_step": int(h_in.nbytes + h_x.nbytes),
                    "d2h_bytes_per_step": int(h_out.nbytes)},
            "roofline": roof,
            "phases_ms_per_step": {k: v[0] / Kp for k, v in phases.items()},
            "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": int(round(sum(v[1] for k, v in phases.items() if k != "Krylov SpMV") / Kp * K)),
            "err_vs_fp64": acc_vs_fp64, "err_vs_other_form": acc_vs_other, "err_vs_oracle": acc_vs_oracle,
            "tuning": tuning or None,
        }
        print(json.dumps(out))
    return 0


# Heat equation (problem "Conduction", HeatEqIncompNewton) on the C3 mesh with the material,
# time step and wall temperature of the reference's conduction example (conductionIncomp.lua:
# rho 1, k 237, cv 1000, initialDT 0.025, walls at T = 10) and a Gaussian initial temperature.
HEAT = dict(metric="heat steps/s (3D conduction on the dam-break mesh, HeatEqIncompNewton step)", unit="steps/s",
            name="3D conduction on the C3 mesh (h = 0.01)", dt=0.025, max_steps=100, max_warmup=3,
            rho=1.0, k=237.0, cv=1000.0, t_wall=10.0, cpu_h=0.03)


def heat_setup(mesh):
    import numpy as np
    from pfem_gb300 import mesh as M

    bound = (mesh.flags & M.BOUND) != 0
    flags = np.where(bound, 1, 0).astype(np.uint8)   # PFG_HEAT_T on the walls
    tbc = np.where(bound, HEAT["t_wall"], 0.0)
    x = mesh.pos
    t0 = 10.0 * np.exp(-((x[0] - 0.3) ** 2 + (x[1] - 0.3) ** 2 + (x[2] - 0.2) ** 2) / 0.05)
    return flags, tbc, t0


def heat_oracle_sample(seconds):
    """Oracle heat steps (C++ assembly, SuperLU) on a coarser mesh of the same domain: the
    C3 mesh's one LU step does not fit a bounded sample.  Returns (node-steps/s, sample)."""
    from oracle import oracle as O
    from pfem_gb300 import mesh as M

    O.build()
    m = M.dam_break_3d(HEAT["cpu_h"])
    flags, tbc, t = heat_setup(m)
    om = O.OracleMesh(m)
    p = O.heat_params(HEAT["rho"], HEAT["cv"], HEAT["k"])
    t0 = time.perf_counter()
    n = 0
    while n < 1 or (time.perf_counter() - t0 < seconds and n < 50):
        t = O.heat_step(om, p, HEAT["dt"], t, flags, tbc)
        n += 1
    el = time.perf_counter() - t0
    return m.n_nodes * n / el, (f"{n} oracle heat steps on the same domain at h = {HEAT['cpu_h']} ({m.n_nodes} nodes, "
                                f"{el:.1f} s), scaled to the C3 mesh by node count (LU cost grows faster: "
                                f"favours the CPU)"), O.num_threads()


def run_gpu_heat(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    from pfem_gb300 import api, build
    from pfem_gb300 import mesh as M
    from pfem_gb300 import workloads as WL

    build.build()
    mesh = WL.c3() if args.h is None else M.dam_break_3d(args.h)
    N = mesh.n_nodes
    flags, tbc, t0 = heat_setup(mesh)
    p = api.default_params(api.KIND_INCOMP_PSPG, 3)
    p.rho, p.heat_k, p.heat_cv = HEAT["rho"], HEAT["k"], HEAT["cv"]
    mixed = args.precision == "fp32"  # FP32 CG corrections under FP64 refinement; fp64: FP64 CG
    p.precision = api.PREC_MIXED if mixed else api.PREC_FP64
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    ctx.set_temperature(t0)
    ctx.heat_set_bc(flags, tbc)
    dt = HEAT["dt"]
    K = max(1, min(args.steps, HEAT["max_steps"]))
    Wm = max(3, min(args.warmup, HEAT["max_warmup"]))
    ext = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")  # 256 MB > 129 MB L2
    for _ in range(Wm):
        ctx.heat_step(dt)
    # every timed step starts from the state after the warm-up: consecutive steps would relax
    # to the steady state, where the CG needs a single iteration
    t_w = ctx.get_temperature()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    clocks = ClockSampler(local)
    conv, iters = 0, 0
    torch.cuda.synchronize()
    clocks.start()
    with torch.cuda.stream(ext):
        for k in range(K):
            ctx.set_temperature(t_w)
            flush.fill_(k & 0xFF)
            ev[k][0].record(ext)
            st = ctx.heat_step(dt)
            ev[k][1].record(ext)
            conv += st.converged
            iters += st.krylov_iterations
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    if conv != K:
        raise RuntimeError(f"{K - conv} of {K} timed heat steps did not converge")

    # phases on a few more steps: assembly and the CG products
    Kp = min(K, 5)
    ctx.set_profiling(True)
    ctx.reset_phase_times()
    it_p = 0
    for _ in range(Kp):
        ctx.set_temperature(t_w)
        it_p += ctx.heat_step(dt).krylov_iterations
    phases = ctx.phase_times()
    ctx.set_profiling(False)
    P = node_pairs(mesh)                            # node pairs (diagonal included)
    s_b = 4 if mixed else 8                          # the CG's value and vector width
    spmv_b = P * (s_b + 4) + (N + 1) * 4 + 2 * N * s_b  # values + columns, row pointers, p in, Ap out
    spmv_ms, spmv_n = phases.get("Heat CG SpMV", (0.0, 0))
    peak, peak_kind = hbm_peak()
    achieved = spmv_b * it_p / (spmv_ms / 1e3) / 1e9 if spmv_ms else None
    roof = {"bound": "hbm", "kernel": "Heat CG SpMV", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None,
            "traffic": None if mixed else NCU_TRAFFIC.get(("heat-c3", "fp64", "Heat CG SpMV")),
            "algorithmic_bytes": spmv_b,
            "avg_launch_us": 1e3 * spmv_ms / max(it_p, 1), "peak_kind": peak_kind,
            "note": "time of all SpMV launches (including the no-op tail of the last 8-iteration chunk) "
                    "over the iterations run"}

    # end to end through the C ABI: temperatures in from pinned host memory, out after the step
    h_t = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    h_o = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    h_t[:] = t_w
    Ke = min(K, 20)
    t1 = time.perf_counter()
    for _ in range(Ke):
        ctx.set_temperature(h_t)
        ctx.heat_step(dt)
        ctx.get_temperature(out=h_o)
    e2e_s = time.perf_counter() - t1

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        nps, sample, cores = heat_oracle_sample(args.cpu_sample_seconds)
        cpu = {"value": nps / N, "unit": HEAT["unit"], "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        out = {
            "metric": HEAT["metric"], "value": K / (total_ms / 1e3), "unit": HEAT["unit"], "n_gpus": world,
            "steps": K, "warmup": Wm, "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32" if mixed else "f64", "data": "synthetic (seeded jittered lattice)",
            "config": {"workload": HEAT["name"], "nodes": N, "elements": int(mesh.n_elems), "node_pairs": P,
                       "dt": dt, "material": "rho 1, k 237, cv 1000 (conduction example)",
                       "linear_solver": ("FP32 Jacobi CG corrections under FP64 refinement of b - A x"
                                         if mixed else "FP64 Jacobi CG") + ", ||r|| <= max(1e-14 ||b||, 1e-10)",
                       "l2": "flushed between timed steps (256 MB write)", "parallelism": "replicas only"},
            "step_stats": {"converged": conv, "cg_iterations": iters},
            "roofline": roof, "phases_ms_per_step": {k: v[0] / Kp for k, v in phases.items()},
            "cpu_baseline": cpu, "clocks": clk,
            "e2e": {"value": Ke / e2e_s, "unit": HEAT["unit"], "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * N},
            "gpu_launches": int(round(sum(v[1] for v in phases.values()) / Kp * K)),
        }
        print(json.dumps(out))
    return 0


def run_gpu_batch(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    from pfem_gb300 import api
    from pfem_gb300 import mesh as M
    from pfem_gb300 import shard
    from pfem_gb300 import workloads as WL

    cfg = INCOMP["batch-c4"]
    # instance sharding: with N ranks each meshes and runs only its share of the instances
    # (partitioned by fluid-node target and device-memory estimate; no collective on the data
    # path, host-side aggregation of the metrics only)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    n_all = args.instances
    targets = [WL.c4_params(i)[0] for i in range(n_all)]
    budget = 0.9 * torch.cuda.get_device_properties(local).total_memory
    mine = shard.my_share(targets, world, rank, [shard.instance_bytes(t, 2) for t in targets], budget)
    t0 = time.perf_counter()
    insts = WL.c4(n_all, only=mine)
    mesh_s = time.perf_counter() - t0
    meshes = [i.mesh for i in insts]
    U, off = M.concat_meshes(meshes)
    mus = np.array([i.mu for i in insts])
    q0 = M.concat_states([i.q0 for i in insts], meshes)
    Ntot = U.n_nodes
    R = 3 * Ntot
    nnz = sum(pattern_nnz(m) for m in meshes)
    dt = cfg["dt"]
    K = max(1, min(args.steps, cfg["max_steps"]))
    Wm = max(3, min(args.warmup, cfg["max_warmup"]))
    n = len(insts)

    ctx = api.Context(incomp_params(api, 2, api.PREC_MIXED, "batch-c4"))
    ctx.upload_mesh(U)
    ctx.set_instances(off, 1000.0, mus)
    ctx.set_states(q0)
    ext = torch.cuda.ExternalStream(ctx.stream)
    for _ in range(Wm):
        ctx.picard_step_batch(dt)
    from pfem_gb300 import tune

    x_t, q_t = ctx.get_positions(), ctx.get_states()

    def restore():
        ctx.set_positions(x_t)
        ctx.set_states(q_t)

    tuning, tsrc = tune.autotune(ctx, 2, Ntot, torch.cuda.get_device_name(local), lambda: ctx.picard_step_batch(dt),
                                 restore)
    tuning = dict(tuning, source=tsrc)
    # one batched step from the warm state: the plain form repeats it per sampled instance
    ctx.picard_step_batch(dt)
    q1 = M.split_states(ctx.get_states(), meshes)
    restore()
    clocks = ClockSampler(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    conv = 0
    pic = 0
    kry = 0
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks.start()
    with torch.cuda.stream(ext):
        for k in range(K):
            ev[k][0].record(ext)
            sts = ctx.picard_step_batch(dt)
            ev[k][1].record(ext)
            conv += sum(s.converged for s in sts)
            pic += sum(s.picard_iterations for s in sts)
            kry = max(kry, max(s.krylov_iterations for s in sts))
            fp64_inst = sum(s.fp64_solves for s in sts)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    if world > 1:  # the slowest rank's time; every rank's instance steps
        t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
        counts = shard.gather_results({rank: (n, R, conv, pic, kry)}, world)
        n_job = sum(v[0] for v in counts.values())
        R_job = sum(v[1] for v in counts.values())
        conv = sum(v[2] for v in counts.values())
        pic = sum(v[3] for v in counts.values())
        kry = max(v[4] for v in counts.values())
    else:
        n_job, R_job = n, R
    qb = M.split_states(ctx.get_states(), meshes)

    # end to end through the C ABI with host buffers: every instance's positions and states in,
    # states out, each step from the same state
    h_in = torch.empty(R, dtype=torch.float64, pin_memory=True).numpy()
    h_out = torch.empty(R, dtype=torch.float64, pin_memory=True).numpy()
    h_x = torch.empty(2 * Ntot, dtype=torch.float64, pin_memory=True).numpy()
    h_in[:] = ctx.get_states()
    h_x[:] = ctx.get_positions().ravel()
    Ke = min(K, 5)
    e2e_conv = 0
    t0 = time.perf_counter()
    for _ in range(Ke):
        ctx.set_positions(h_x)
        ctx.set_states(h_in)
        e2e_conv += sum(s.converged for s in ctx.picard_step_batch(dt))
        ctx.get_states(out=h_out)
    e2e_s = time.perf_counter() - t0
    if e2e_conv != n * Ke:
        raise RuntimeError(f"end-to-end batch steps: {e2e_conv} of {n * Ke} instance steps converged")

    # plain FP64 drop-in, one context per instance, on a sample spread over the size range
    order = np.argsort([m.n_nodes for m in meshes])
    sample = sorted(set(order[np.linspace(0, n - 1, min(n, 16)).astype(int)].tolist()))
    plain_ms, plain_dof_steps = 0.0, 0
    errs, errs_traj = [], []
    for i in sample:
        m = meshes[i]
        c = api.Context(incomp_params(api, 2, api.PREC_FP64, "batch-c4", mu=float(mus[i])))
        c.upload_mesh(m)
        c.set_states(insts[i].q0)
        for _ in range(Wm):
            c.picard_step(dt)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        cext = torch.cuda.ExternalStream(c.stream)
        torch.cuda.synchronize()
        with torch.cuda.stream(cext):
            e0.record(cext)
            for _ in range(K):
                c.picard_step(dt)
            e1.record(cext)
        torch.cuda.synchronize()
        plain_ms += e0.elapsed_time(e1)
        plain_dof_steps += 3 * m.n_nodes * K
        errs_traj.append(max(field_errors(qb[i], c.get_states(), 3, m.n_nodes)))
        c.close()
        # one step from the same warm state as the batched step above, the plain form's linear
        # solves taken to relative residual 1e-14 (BiCGSTAB at 1e-12 leaves up to ~3e-8 in the
        # fields of the stiffest instances; the mixed form's refinement lands below that)
        p_ref = incomp_params(api, 2, api.PREC_FP64, "batch-c4", mu=float(mus[i]))
        p_ref.krylov_rel_tol, p_ref.krylov_max_iter = 1e-14, 50000
        c = api.Context(p_ref)
        c.upload_mesh(m)
        c.set_positions(x_t[:, off[i]:off[i + 1]])
        c.set_states(M.split_states(q_t, meshes)[i])
        c.picard_step(dt)
        errs.append(max(field_errors(q1[i], c.get_states(), 3, m.n_nodes)))
        c.close()
    sample_dof = sum(3 * meshes[i].n_nodes for i in sample)
    plain_dof_per_s = plain_dof_steps / (plain_ms / 1e3)

    # the plain form with the device sparse LU on four instances of the sample (one timed step
    # each, after the warm-up steps)
    lu_ms, lu_dof = 0.0, 0
    for i in sample[::max(1, len(sample) // 4)][:4]:
        m = meshes[i]
        p_lu = incomp_params(api, 2, api.PREC_FP64, "batch-c4", mu=float(mus[i]))
        p_lu.linear_solver = api.LINSOLVE_LU
        c = api.Context(p_lu)
        c.upload_mesh(m)
        c.set_states(insts[i].q0)
        for _ in range(Wm):
            c.picard_step(dt)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        cext = torch.cuda.ExternalStream(c.stream)
        torch.cuda.synchronize()
        with torch.cuda.stream(cext):
            e0.record(cext)
            c.picard_step(dt)
            e1.record(cext)
        torch.cuda.synchronize()
        lu_ms += e0.elapsed_time(e1)
        lu_dof += 3 * m.n_nodes
        c.close()
    lu_dof_per_s = lu_dof / (lu_ms / 1e3) if lu_ms else None

    # phase times of one batched step
    ctx.set_profiling(True)
    ctx.reset_phase_times()
    ctx.picard_step_batch(dt)
    phases = ctx.phase_times()
    work = _spmv_work(ctx, phases, nnz, 2)
    ctx.set_profiling(False)
    peak, peak_kind = hbm_peak()
    roof = _phase_roofline(phases, spmv_bytes(nnz, R, 4) * work, asm_bytes(2, Ntot, U.n_elems, R, nnz, 4), peak)
    roof["peak_kind"] = peak_kind
    roof["spmv_work_fraction"] = work

    value = n_job * K / (total_ms / 1e3)
    dof_per_s = R_job * K / (total_ms / 1e3)
    if rank == 0:
        out = {
            "metric": cfg["metric"], "value": value, "unit": cfg["unit"], "n_gpus": world, "steps": K, "warmup": Wm,
            "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32", "data": "synthetic (seeded jittered lattices, per-instance seeds)",
            "config": {"workload": cfg["name"], "instances": n_job, "instances_rank0": n, "nodes_rank0": Ntot,
                       "elements_rank0": int(U.n_elems),
                       "unknowns": R, "nnz": nnz, "dt": dt, "host_meshing_s": mesh_s,
                       "precision": "mixed (FP32 assembly + FP32 BiCGSTAB, double-float refinement residual)",
                       "linear_tolerance": f"||r|| <= {WL.C4_TOL:g} ||b|| (FP64 residual), both forms",
                       "l2": "working set > L2 (129 MB)",
                       "parallelism": "one batched launch sequence" if world == 1 else
                       f"instances sharded over {world} ranks by node count and memory (no collective)"},
            "dof_per_s": dof_per_s,
            "step_stats": {"converged_instance_steps": conv, "of": n_job * K, "picard_iterations": pic,
                           "max_krylov_iterations_per_instance_step": kry,
                           "instances_with_fp64_correction_solves": fp64_inst},
            "plain_fp64_sample": {"instances": len(sample), "dof": sample_dof, "dof_per_s": plain_dof_per_s,
                                  "speedup_dof_per_s": dof_per_s / world / plain_dof_per_s,
                                  "max_rel_err_vs_plain": max(errs) if errs else None,
                                  "err_definition": "one Picard step from the same warm state against the plain "
                                                    "form solved to relative residual 1e-14",
                                  "max_rel_err_after_all_steps": max(errs_traj) if errs_traj else None},
            "plain_lu_sample": {"instances": 4, "dof_per_s": lu_dof_per_s,
                                "speedup_dof_per_s": dof_per_s / world / lu_dof_per_s if lu_dof_per_s else None},
            "roofline": roof, "phases_ms_per_step": {k: v[0] for k, v in phases.items()},
            "cpu_baseline": None, "clocks": clk,
            "e2e": {"value": n * Ke / e2e_s, "unit": cfg["unit"], "h2d_bytes_per_step": (R + 2 * Ntot) * 8,
                    "d2h_bytes_per_step": R * 8},
            "gpu_launches": int(round(sum(v[1] for k, v in phases.items() if k != "Krylov SpMV") * K)),
            "tuning": tuning,
        }
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def c5_requests(n, rate, seed=20261203):
    """The served mix: Poisson arrivals at `rate`; 80% 2D (half dam breaks with 1k-20k fluid
    nodes and column aspect 0.5-2, half sloshing tanks of `examples/2D/sloshing` with
    h = 0.01-0.03 and its material: rho = 1, mu = 0.01, K0 = 2.2e5, K0' = 7.6), 20% 3D dam
    breaks with 10k-200k fluid nodes; weakly compressible or incompressible at even odds; dam
    break mu log-uniform in [1e-3, 1e-1]; WC requests 50-500 explicit steps, incompressible
    ones 10-50 Picard steps in 2D and 5-20 in 3D."""
    import math

    import numpy as np
    from pfem_gb300 import api
    from pfem_gb300 import mesh as M
    from pfem_gb300 import serve as SV

    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        is3d = rng.random() < 0.2
        wc = rng.random() < 0.5
        mu = math.exp(rng.uniform(math.log(1e-3), math.log(1e-1)))
        sloshing = (not is3d) and rng.random() < 0.5
        params, case = None, "dam break"
        if is3d:
            nf = math.exp(rng.uniform(math.log(1e4), math.log(2e5)))
            col = (0.5, 0.5, 1.0)
            h = (0.25 / nf) ** (1 / 3)
            m = M.dam_break_3d(h, seed=seed + i)
            steps = int(rng.integers(50, 501)) if wc else int(rng.integers(5, 21))
        elif sloshing:
            h = math.exp(rng.uniform(math.log(0.01), math.log(0.03)))
            m = M.sloshing_2d(h, seed=seed + i)
            steps = int(rng.integers(50, 501)) if wc else int(rng.integers(10, 51))
            kind = api.KIND_WC_CDS_DPDT if wc else api.KIND_INCOMP_PSPG
            if wc:
                st = M.sloshing_wc_initial_states(m)
                params = dict(rho_star=1.0, K0=2.2e5, K0p=7.6, security_coeff=0.1, max_dt=0.1)
            else:
                st = np.zeros(3 * m.n_nodes)
                params = dict(rho=1.0)
            out.append(SV.Request(kind, m, st, steps, dt=1e-2, mu=0.01, arrival=t, rid=i, params=params,
                                  case="sloshing"))
            continue
        else:
            nf = math.exp(rng.uniform(math.log(1e3), math.log(2e4)))
            a = rng.uniform(0.5, 2.0)
            col = (math.sqrt(2 / a), math.sqrt(2 * a))
            h = math.sqrt(2.0 / nf)
            m = M.dam_break_2d(h, column=col, seed=seed + i)
            steps = int(rng.integers(50, 501)) if wc else int(rng.integers(10, 51))
        kind = api.KIND_WC_CDS_DPDT if wc else api.KIND_INCOMP_PSPG
        st = M.wc_initial_states(m, column=col) if wc else M.incomp_initial_states(m, column=col)
        out.append(SV.Request(kind, m, st, steps, dt=5e-4 if is3d else 1e-3, mu=mu, arrival=t, rid=i))
    return out


def run_gpu_serve(args):
    import numpy as np
    import torch
    from pfem_gb300 import serve as SV

    world, rank, local = dist_env()
    t0 = time.perf_counter()
    reqs = c5_requests(args.requests, args.rate)
    mesh_s = time.perf_counter() - t0
    free, total = torch.cuda.mem_get_info()
    budget = int(0.5 * free)
    srv = SV.Server(hbm_budget_bytes=budget, max_active=8)
    clocks = ClockSampler(local)
    clocks.start()
    out = srv.run(reqs, realtime=True)
    clk = clocks.stop()
    m = SV.metrics(out, srv.makespan)
    # the same two requests alone: results must not depend on the mix
    same = True
    for r in [x for x in out if x.error is None][:2]:
        alone = SV.Server(hbm_budget_bytes=budget, max_active=1).run(
            [c5_requests(args.requests, args.rate)[r.rid]], realtime=False)[0]
        same &= bool(np.array_equal(alone.result, r.result))
    h2d = sum(r.states.nbytes + r.mesh.pos.nbytes + r.mesh.conn.nbytes + r.mesh.flags.nbytes for r in out)
    d2h = sum(r.states.nbytes + r.mesh.pos.nbytes for r in out)
    steps = sum(r.steps for r in out if r.error is None)
    if rank == 0:
        res = {
            "metric": "aggregate time-steps/s of a served request mix (C5), with p50/p99 request latency",
            "value": m["steps_per_s"], "unit": "steps/s", "n_gpus": world, "steps": steps, "warmup": 0,
            "ms_per_step": 1e3 * srv.makespan / max(steps, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "mixed",
            "data": "synthetic (seeded dam breaks and sloshing tanks, Poisson arrivals)",
            "config": {"workload": "served mix (C5)", "requests": args.requests, "rate_per_s": args.rate,
                       "hbm_budget_bytes": budget, "slots": 8, "host_meshing_s": mesh_s,
                       "kinds": {"wc": sum(r.kind == 1 for r in out), "incomp": sum(r.kind == 0 for r in out)},
                       "dims": {"2d": sum(r.mesh.dim == 2 for r in out), "3d": sum(r.mesh.dim == 3 for r in out)},
                       "cases": {"sloshing": sum(r.case == "sloshing" for r in out),
                                 "dam break": sum(r.case == "dam break" for r in out)},
                       "nodes_max": max(r.mesh.n_nodes for r in out),
                       "remesh": "C++ host remesh (libpfemremesh.so) after every accepted incompressible step"},
            "latency_p50_s": m["latency_p50_s"], "latency_p99_s": m["latency_p99_s"],
            "queue_wait_p50_s": m["queue_wait_p50_s"], "queue_wait_p99_s": m["queue_wait_p99_s"],
            "dof_per_s": m["dof_per_s"], "completed": m["completed"], "failed": m["failed"],
            "errors": [r.error for r in out if r.error][:3],
            "peak_active": srv.peak_active, "peak_estimated_bytes": srv.peak_bytes,
            "mean_active": m["mean_active"], "slowest_requests": m["slowest"],
            "alone_equals_mix": same,
            "e2e": {"value": m["steps_per_s"], "unit": "steps/s", "h2d_bytes_per_step": int(h2d / max(steps, 1)),
                    "d2h_bytes_per_step": int(d2h / max(steps, 1))},
            "roofline": None, "cpu_baseline": None, "clocks": clk, "gpu_launches": None,
        }
        print(json.dumps(res))
    return 0


def run_reference_incomp(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    from pfem_gb300 import mesh as M
    from pfem_gb300 import workloads as WL

    O.build()
    upper = False
    if args.workload == "heat-c3":
        from pfem_gb300 import workloads as WL2

        nps, sample, cores = heat_oracle_sample(args.cpu_sample_seconds)
        n_c3 = WL2.c3().n_nodes
        v = nps / n_c3
        out = {"impl": "reference", "metric": HEAT["metric"], "value": v, "unit": HEAT["unit"], "n_gpus": args.gpus,
               "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered lattice)",
               "config": {"workload": HEAT["name"]},
               "cpu_baseline": {"value": v, "unit": HEAT["unit"], "cores": cores, "kind": "port", "sample": sample},
               "e2e": {"value": v, "unit": HEAT["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
               "gpu_launches": 0}
        print(json.dumps(out))
        return 0
    if args.workload == "serve-c5":
        cfg = {"metric": "aggregate time-steps/s of a served request mix (C5), with p50/p99 request latency",
               "unit": "steps/s", "name": "served mix (C5)"}
        t0 = time.perf_counter()
        n_steps, n_req = 0, 0
        for r in c5_requests(args.requests, args.rate):
            om = O.OracleMesh(r.mesh)
            s = r.states.copy()
            if r.kind == 1:
                p = O.wc_params(mu=r.mu, g=(0.0, -9.81) if r.mesh.dim == 2 else (0.0, 0.0, -9.81))
                dt = O.wc_next_dt(om, p, s)
                for _ in range(r.steps):
                    O.wc_step(om, p, dt, s)
                    dt = O.wc_next_dt(om, p, s)
                    n_steps += 1
            else:
                g = (0.0, -9.81) if r.mesh.dim == 2 else (0.0, 0.0, -9.81)
                for _ in range(r.steps):
                    s, _ = O.pspg_picard_step(om, s, r.dt, mu=r.mu, g=g)
                    n_steps += 1
            n_req += 1
            if time.perf_counter() - t0 > 120:
                break
        el = time.perf_counter() - t0
        v = n_steps / el
        sample = f"the first {n_req} requests run one after another ({n_steps} steps, {el:.1f} s)"
    else:
        cfg = incomp_cfg(args)
    if args.workload == "serve-c5":
        pass
    elif args.workload == "batch-c4":
        insts = WL.c4(args.instances)
        t0 = time.perf_counter()
        dof, inst_steps = 0, 0
        for inst in insts:
            om = O.OracleMesh(inst.mesh)
            O.pspg_picard_step(om, inst.q0, cfg["dt"], mu=inst.mu)
            dof += 3 * inst.mesh.n_nodes
            inst_steps += 1
            if time.perf_counter() - t0 > 120:
                break
        el = time.perf_counter() - t0
        v = inst_steps / el
        sample = f"one Picard step of each of the first {inst_steps} instances ({el:.1f} s), {dof / el:.3g} DOF/s"
    elif args.workload == "incomp-c3":
        v, _, sample, upper = c3_cpu_sample(args.h or 0.01, args.cpu_budget)
        if v is None:
            print(json.dumps({"impl": "reference", "unavailable": sample}))
            return 0
    else:
        mesh = incomp_mesh(args)
        q = M.incomp_initial_states(mesh, column=cfg["column"])
        om = O.OracleMesh(mesh)
        g = (0.0, -9.81) if mesh.dim == 2 else (0.0, 0.0, -9.81)
        t0 = time.perf_counter()
        n_done = 0
        while n_done < min(args.steps, cfg["max_steps"]):
            q, _ = O.pspg_picard_step(om, q, cfg["dt"], g=g)
            n_done += 1
            if time.perf_counter() - t0 > 120:
                break
        el = time.perf_counter() - t0
        v = n_done / el
        sample = f"{n_done} Picard steps ({el:.1f} s)"
    out = {"impl": "reference", "metric": cfg["metric"], "value": v, "unit": cfg["unit"], "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered lattice)",
           "config": {"workload": cfg["name"]},
           "cpu_baseline": {"value": v, "unit": cfg["unit"], "cores": O.num_threads(), "kind": "port",
                            "sample": sample, "upper_bound": bool(upper)},
           "upper_bound": bool(upper),
           "e2e": {"value": v, "unit": cfg["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "gpu_launches": 0}
    print(json.dumps(out))
    return 0


def main():
    args = parse_args()
    if args.workload == "wc-c2-batch":
        if args.impl == "reference":
            return run_reference(args)
        return run_gpu_wc_batch(args)
    if args.workload != "wc-c2":
        if args.impl == "reference":
            return run_reference_incomp(args)
        return run_gpu_incomp(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
