"""Serving many simulations on one GPU: continuous admission under an HBM budget.

Each admitted request gets its own library context: its mesh and fields stay resident on the
device for its whole life, its kernels run on the context's own CUDA stream, and a worker
thread drives its time loop.  Incompressible requests run the reference's loop: the host
remeshes after every accepted step (in the request's thread, while the other requests keep
the GPU busy) and a failed step is retried with half the time step.  Every library call runs without the Python interpreter lock, so
the device interleaves the work of all admitted requests.  Admission is first come, first
served under two limits, a number of slots and an HBM budget: a request's device footprint is
estimated from its mesh before admission, and when a request finishes its context (and
memory) is released and the next waiting requests are admitted at once.  Contexts never share
device data, so a request's result is the same alone and in any mix.

No reference counterpart: the reference runs one Problem per process.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import api
from . import mesh as M
from . import remesh as RM
from . import solver as SO


@dataclass
class Request:
    kind: int                       # api.KIND_INCOMP_PSPG or api.KIND_WC_CDS_DPDT
    mesh: M.HostMesh
    states: np.ndarray
    steps: int
    dt: float = 1e-3                # incompressible time step (WC steps use their CFL step)
    precision: int = api.PREC_MIXED
    mu: float = 1e-3
    remesh: bool = True             # incompressible: remesh after every accepted step
    arrival: float = 0.0            # seconds after the start of the run
    rid: int = -1
    params: dict | None = None      # further pfg_params fields (e.g. rho, K0, rho_star)
    case: str = "dam break"
    t_device: float = 0.0           # incompressible with remesh: seconds in the device steps
    t_remesh: float = 0.0           # ... and in the host remesh
    # filled in by the server
    t_admit: float | None = None
    t_done: float | None = None
    result: np.ndarray | None = None
    positions: np.ndarray | None = None
    converged_steps: int = 0
    device_bytes: int = 0
    estimate_bytes: int = 0
    error: str | None = None

    @property
    def dof(self):
        return (self.mesh.dim + 1) * self.mesh.n_nodes

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


def estimate_device_bytes(kind, precision, mesh) -> int:
    """Upper estimate of a context's device memory for `mesh`, from the library's buffers:
    mesh and topology (positions, flags, connectivity, incidence lists, adjacency, CSR
    structure), then the incompressible system (FP64 values, right-hand side, element data,
    three state vectors, FP64 Krylov vectors and block inverses; FP32 copies in mixed form) or
    the WC state and element->node planes."""
    d, N, E = mesh.dim, mesh.n_nodes, mesh.n_elems
    R = (d + 1) * N
    npe = d + 1
    nnz = M.pspg_nnz(mesh)
    P = nnz // (npe * npe) + N
    b = 3 * d * N * 8 + N + npe * E * (4 + 4 + 1 + 4) + (N + 1) * 8 + 2 * P * 4 + (R + 1) * 4 + nnz * 4 + R * 4
    if kind == api.KIND_INCOMP_PSPG:
        b += nnz * 8 + R * 8 + (2 + d * npe) * E * 8 + 3 * R * 8 + 12 * R * 8 + npe * npe * N * 8
        if precision == api.PREC_MIXED:
            b += nnz * 4 + 8 * R * 4 + npe * npe * N * 4 + R * 8 + N * 4
            # multigrid: bfloat16 blocks, coarse levels (< half the FP32 blocks), cycle vectors
            b += nnz * 3 + nnz * 2 + 3 * R * 4
    else:
        b += (2 * d + 2) * N * 8 * 3 + (7 * d + 5) * N * 4 + (1 + 3 * d) * npe * E * 4 + npe * E * 8 * (2 + d) \
             + 4 * N * 8
    return int(1.25 * b) + (4 << 20)


def admission_bytes(req: Request) -> int:
    """What admission reserves for a request: its estimate, with half again for an
    incompressible request that remeshes (the remesh may add nodes)."""
    b = estimate_device_bytes(req.kind, req.precision, req.mesh)
    return int(1.5 * b) if req.kind == api.KIND_INCOMP_PSPG and req.remesh else b


class Server:
    """Runs requests with at most `max_active` at a time and their estimated device memory
    summed below `hbm_budget_bytes`."""

    def __init__(self, hbm_budget_bytes: int, max_active: int = 8, native_remesh: bool = True):
        self.budget = int(hbm_budget_bytes)
        self.max_active = int(max_active)
        self.native_remesh = bool(native_remesh)   # the C++ host remesh (else the Python one)
        self._lock = threading.Condition()
        self._active = 0
        self._used = 0
        self.peak_active = 0
        self.peak_bytes = 0

    # -- one request ----------------------------------------------------------------------
    def _run_one(self, req: Request, t0: float):
        try:
            p = api.default_params(req.kind, req.mesh.dim)
            p.precision = req.precision
            p.mu = req.mu
            for k, v in (req.params or {}).items():
                setattr(p, k, v)
            # the context's own cap: twice the admission reserve for a request that remeshes (the
            # remesh may add nodes; admission reserves 1.5x the initial mesh's estimate)
            p.hbm_budget_bytes = 2 * req.estimate_bytes if req.kind == api.KIND_INCOMP_PSPG and req.remesh \
                else req.estimate_bytes
            if req.kind == api.KIND_INCOMP_PSPG and req.remesh:
                self._run_incomp(req, p, self.native_remesh)
            else:
                ctx = api.Context(p)
                try:
                    ctx.upload_mesh(req.mesh)
                    ctx.set_states(req.states)
                    if req.kind == api.KIND_WC_CDS_DPDT:
                        ctx.set_time(0.0, ctx.next_dt())
                        ctx.wc_step(0.0, req.steps)
                        req.converged_steps = req.steps
                    else:
                        for _ in range(req.steps):
                            st = ctx.picard_step(req.dt)
                            req.converged_steps += st.converged
                    req.result = ctx.get_states()
                    req.positions = ctx.get_positions()
                    req.device_bytes = ctx.device_bytes()
                finally:
                    ctx.close()
        except Exception as e:  # reported with the request; the server keeps serving
            req.error = str(e)
        req.t_done = time.perf_counter() - t0
        with self._lock:
            self._active -= 1
            self._used -= req.estimate_bytes
            self._lock.notify_all()

    @staticmethod
    def _run_incomp(req: Request, p, native_remesh=True):
        """`steps` accepted steps of the reference's loop (`IncompNewton/Solver.cpp:216-247`):
        remesh after each accepted step, dt halved after a failed one (at most 4 x steps tries)."""
        m = req.mesh
        lo, hi = m.pos.min(axis=1), m.pos.max(axis=1)
        pad = 0.1 * (hi - lo)
        box = tuple(lo - pad) + tuple(hi + pad)
        box = box[:2 * m.dim - 1] + (1e30,)  # open at the top: nodes leave only sideways or below
        prm = RM.RemeshParams(hchar=m.hchar, alpha=m.alpha, bounding_box=box, native=native_remesh)
        sol = SO.SolverIncompNewtonGPU(m, req.states, params=p, remesh_params=prm, precision=req.precision,
                                       initial_dt=req.dt, max_dt=req.dt)
        try:
            tries = 0
            while sol.steps < req.steps and tries < 4 * req.steps:
                sol.solve_one_time_step()
                sol.compute_next_dt()
                tries += 1
            req.converged_steps = sol.steps
            req.t_device, req.t_remesh = sol.t_device, sol.t_remesh
            req.result = sol.states()
            req.positions = sol.positions()
            req.device_bytes = sol.ctx.device_bytes()
            if sol.steps < req.steps:
                req.error = f"{sol.steps} of {req.steps} steps converged in {tries} tries"
        finally:
            sol.close()

    # -- the request loop -----------------------------------------------------------------
    def run(self, requests, realtime=True):
        """Serve `requests` (arrival times in seconds from now when `realtime`, else all at
        once, in list order).  Returns the requests with their timings and results."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        for i, r in enumerate(reqs):
            if r.rid < 0:
                r.rid = i
            r.estimate_bytes = admission_bytes(r)
            if r.estimate_bytes > self.budget:
                r.error = f"needs ~{r.estimate_bytes} bytes, over the {self.budget}-byte budget"
        t0 = time.perf_counter()
        threads = []
        for r in reqs:
            if r.error:
                continue
            if realtime:
                wait = r.arrival - (time.perf_counter() - t0)
                if wait > 0:
                    time.sleep(wait)
            else:
                r.arrival = time.perf_counter() - t0
            with self._lock:
                while self._active >= self.max_active or self._used + r.estimate_bytes > self.budget:
                    self._lock.wait()
                self._active += 1
                self._used += r.estimate_bytes
                self.peak_active = max(self.peak_active, self._active)
                self.peak_bytes = max(self.peak_bytes, self._used)
            r.t_admit = time.perf_counter() - t0
            th = threading.Thread(target=self._run_one, args=(r, t0), daemon=True)
            th.start()
            threads.append(th)
        for th in threads:
            th.join()
        self.makespan = time.perf_counter() - t0
        return reqs


def metrics(reqs, makespan):
    """Latency percentiles (arrival to result), queueing delay and aggregate throughput."""
    done = [r for r in reqs if r.error is None and r.t_done is not None]
    lat = np.array([r.latency for r in done]) if done else np.zeros(1)
    wait = np.array([r.t_admit - r.arrival for r in done]) if done else np.zeros(1)
    steps = sum(r.converged_steps for r in done)
    dof_steps = sum(r.dof * r.converged_steps for r in done)
    # mean number of requests in service over the run (time-weighted slot occupancy)
    busy = sum(r.t_done - r.t_admit for r in done)
    slowest = sorted(done, key=lambda r: r.latency, reverse=True)[:3]
    return {
        "requests": len(reqs), "completed": len(done), "failed": len(reqs) - len(done),
        "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
        "queue_wait_p50_s": float(np.percentile(wait, 50)), "queue_wait_p99_s": float(np.percentile(wait, 99)),
        "makespan_s": makespan, "steps_per_s": steps / makespan, "dof_per_s": dof_steps / makespan,
        "mean_active": busy / makespan if makespan > 0 else 0.0,
        "slowest": [{"rid": r.rid, "case": r.case, "dim": r.mesh.dim,
                     "kind": "wc" if r.kind == api.KIND_WC_CDS_DPDT else "incomp", "nodes": r.mesh.n_nodes,
                     "steps": r.steps, "queue_wait_s": round(r.t_admit - r.arrival, 3),
                     "service_s": round(r.t_done - r.t_admit, 3), "device_step_s": round(r.t_device, 3),
                     "host_remesh_s": round(r.t_remesh, 3)} for r in slowest],
    }
