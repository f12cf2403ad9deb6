"""Host-side solver classes: the reference's time loop around the GPU per-step solve.

    SolverIncompNewtonGPU   srcs/simulation/physics/IncompNewton/Solver.cpp (PSPG, no temperature)
    SolverWCompNewtonGPU    srcs/simulation/physics/WCompNewton/Solver.cpp  (CDS_dpdt, no temperature)
    Problem                 srcs/simulation/Problem.cpp:320-380 (Problem::simulate)

A solver owns one library context (the device keeps positions and states between steps);
`solve_one_time_step` and `compute_next_dt` keep the reference's contract (`Solver.hpp:53,56`):
a failed incompressible step returns False with positions and states restored, and the next
time step shrinks.  After each accepted step the host remeshes (`Mesh::remesh`, restated in
`remesh.py`) and hands the library only the new mesh and the remapped states.
"""
from __future__ import annotations

import numpy as np

from . import api
from . import mesh as M
from . import remesh as RM


class _SolverBase:
    kind = None

    def __init__(self, mesh: M.HostMesh, states, params=None, remesh_params: RM.RemeshParams | None = None,
                 precision=api.PREC_FP64, dirichlet=None):
        p = params if params is not None else api.default_params(self.kind, mesh.dim)
        p.precision = precision
        self.params = p
        self.remesh_params = remesh_params
        self.ctx = api.Context(p)
        self.mesh = mesh
        self.dirichlet = dirichlet        # callable(pos, flags, t) -> (nodes, values d x n) or None
        self.time = 0.0
        self.steps = 0
        self._upload(mesh, np.asarray(states, float))

    def _upload(self, mesh, states):
        self.mesh = mesh
        self.ctx.upload_mesh(mesh)
        self.ctx.set_states(states)
        self._apply_dirichlet()

    def _apply_dirichlet(self):
        if self.dirichlet is None:
            return
        nodes, values = self.dirichlet(self.mesh.pos, self.mesh.flags, self.time)
        if len(nodes):
            self.ctx.set_dirichlet(nodes, values)

    def states(self):
        return self.ctx.get_states()

    def positions(self):
        return self.ctx.get_positions()

    def remesh(self):
        """`Mesh::remesh` on the host, then the new mesh and remapped states go to the device."""
        if self.remesh_params is None:
            return
        cur = self.mesh.copy()
        cur.pos = self.ctx.get_positions()
        cur.flags = self.ctx.get_flags() & np.uint8(0x0F)
        new, st = RM.remesh(cur, self.ctx.get_states(), self.remesh_params)
        self._upload(new, st)

    def close(self):
        self.ctx.close()


class SolverIncompNewtonGPU(_SolverBase):
    """PSPG Picard step on the GPU with the reference's dt control (`IncompNewton/Solver.cpp:216-247`):
    dt /= coeffDTDecrease after a failed step, dt = min(maxDT, dt * coeffDTincrease) after a
    successful one (with adaptDT; a failed step without it raises, like the reference)."""
    kind = api.KIND_INCOMP_PSPG

    def __init__(self, mesh, states, params=None, remesh_params=None, precision=api.PREC_FP64, dirichlet=None,
                 initial_dt=1e-3, max_dt=1e-3, adapt_dt=True, coeff_dt_increase=1.5, coeff_dt_decrease=2.0):
        super().__init__(mesh, states, params, remesh_params, precision, dirichlet)
        self.dt = initial_dt
        self.max_dt = max_dt
        self.adapt_dt = adapt_dt
        self.coeff_inc = coeff_dt_increase
        self.coeff_dec = coeff_dt_decrease
        self.solve_succeeded = True
        self.last_status = None

    def solve_one_time_step(self) -> bool:
        """`SolverIncompNewton::m_solveIncompNewtonNoT`: Picard solve; on success the time
        advances and the mesh is rebuilt."""
        st = self.ctx.picard_step(self.dt)
        self.last_status = st
        self.solve_succeeded = bool(st.converged)
        if self.solve_succeeded:
            self.time += self.dt
            self.steps += 1
            self.remesh()
        return self.solve_succeeded

    def compute_next_dt(self):
        if not self.solve_succeeded:
            if not self.adapt_dt:
                raise RuntimeError("solving the precedent time step was not successful!")
            self.dt /= self.coeff_dec
        elif self.adapt_dt:
            self.dt = min(self.max_dt, self.dt * self.coeff_inc)


class SolverWCompNewtonGPU(_SolverBase):
    """CDS_dpdt explicit step on the GPU (`WCompNewton/Solver.cpp:236-276`) with the CFL time
    step of `computeNextDT` (`:192-234`) kept on the device; the mesh is rebuilt once the
    simulated time passes the next remeshing time, which then advances by maxDT."""
    kind = api.KIND_WC_CDS_DPDT

    def __init__(self, mesh, states, params=None, remesh_params=None, precision=api.PREC_FP64, dirichlet=None):
        super().__init__(mesh, states, params, remesh_params, precision, dirichlet)
        self.ctx.set_time(0.0, self.ctx.next_dt())
        self.next_remesh = self.params.max_dt
        self.dt = None

    def solve_one_time_step(self) -> bool:
        st = self.ctx.wc_step(0.0, 1)
        self.dt = st.dt
        self.time = st.time
        self.steps += 1
        if self.remesh_params is not None and self.time > self.next_remesh:
            self.remesh()
            self.ctx.set_time(self.time, self.ctx.next_dt())
            self.next_remesh += self.params.max_dt
        return True

    def compute_next_dt(self):
        """The device already holds the CFL step of the current state; nothing to do on the host."""


class Problem:
    """`Problem::simulate` (`Problem.cpp:320-380`): step until the simulated time reaches
    `max_time`, calling the extractors after every accepted step."""

    def __init__(self, solver, max_time, extractors=()):
        self.solver = solver
        self.max_time = max_time
        self.extractors = list(extractors)

    def simulate(self, max_steps=None):
        n = 0
        while self.solver.time < self.max_time and (max_steps is None or n < max_steps):
            ok = self.solver.solve_one_time_step()
            if ok:
                for ex in self.extractors:
                    ex(self.solver)
            self.solver.compute_next_dt()
            n += 1
        return n


def mass_extractor(out):
    """`MassExtractor` (`extractors/MassExtractor.cpp:26-37`): (time, volume or mass)."""
    def ex(solver):
        v = solver.ctx.mass() if solver.kind == api.KIND_WC_CDS_DPDT else solver.ctx.volume()
        out.append((solver.time, v))
    return ex


def tip_extractor(out, coordinate=0, want_max=True):
    """`MinMaxExtractor` (`extractors/MinMaxExtractor.cpp:28-62`): (time, front position)."""
    def ex(solver):
        out.append((solver.time, solver.ctx.tip(coordinate, want_max)))
    return ex
