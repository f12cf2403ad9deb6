"""Host-side solver classes: the reference's time loop around the GPU per-step solve.

    SolverIncompNewtonGPU   srcs/simulation/physics/IncompNewton/Solver.cpp (PSPG; problems
                            "IncompNewtonNoT", "Bingham", "Boussinesq", "Conduction")
    SolverWCompNewtonGPU    srcs/simulation/physics/WCompNewton/Solver.cpp  (CDS_dpdt, no temperature)
    Problem                 srcs/simulation/Problem.cpp:320-380 (Problem::simulate)

A solver owns one library context (the device keeps positions and states between steps);
`solve_one_time_step` and `compute_next_dt` keep the reference's contract (`Solver.hpp:53,56`):
a failed incompressible step returns False with positions and states restored, and the next
time step shrinks.  After each accepted step the host remeshes (`Mesh::remesh`, restated in
`remesh.py`) and hands the library only the new mesh and the remapped states.
"""
from __future__ import annotations

import time

import numpy as np

from . import api
from . import heat as H
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
        """`Mesh::remesh` on the host, then the new mesh and the states remapped on the host
        (`RM.apply_origin`) go to the device."""
        if self.remesh_params is None:
            return
        cur = self.mesh.copy()
        cur.pos = self.ctx.get_positions()
        cur.flags = self.ctx.get_flags() & np.uint8(0x0F)
        new, origin = RM.remesh_map(cur, self.remesh_params)
        self._upload(new, RM.apply_origin(self.ctx.get_states(), origin, cur.n_nodes))

    def close(self):
        self.ctx.close()


class SolverIncompNewtonGPU(_SolverBase):
    """PSPG Picard step on the GPU with the reference's dt control (`IncompNewton/Solver.cpp:216-247`):
    dt /= coeffDTDecrease after a failed step, dt = min(maxDT, dt * coeffDTincrease) after a
    successful one (with adaptDT; a failed step without it raises, like the reference).

    `problem` selects the reference's solve function (`Solver.cpp:95-175`): "IncompNewtonNoT"
    (and "Bingham", through params.tau0) solve the momentum-continuity equation; "Boussinesq"
    (params.boussinesq = 1) adds the heat equation before or after it (`solve_heat_first`,
    `m_solveBoussinesq`, :249-284); "Conduction" solves the heat equation alone on a fixed mesh
    (`m_solveConduction`, :286-296).  Heat problems take the initial node temperatures, a BC
    callable heat_bc(pos, flags, t) -> (heat flags (N,) uint8, Dirichlet temperatures (N,)) and
    optionally a flux callable q(x, t) -> (dim,) evaluated at the facet Gauss points; both are
    evaluated at t + dt before each heat solve, as the reference's m_applyBC does."""
    kind = api.KIND_INCOMP_PSPG

    def __init__(self, mesh, states, params=None, remesh_params=None, precision=api.PREC_FP64, dirichlet=None,
                 initial_dt=1e-3, max_dt=1e-3, adapt_dt=True, coeff_dt_increase=1.5, coeff_dt_decrease=2.0,
                 problem="IncompNewtonNoT", temperature=None, heat_bc=None, heat_flux=None, solve_heat_first=True):
        if problem not in ("IncompNewtonNoT", "Bingham", "Boussinesq", "Conduction"):
            raise ValueError(f"unknown problem {problem!r}")
        if problem in ("Boussinesq", "Conduction") and temperature is None:
            raise ValueError(f"problem {problem!r} needs the initial temperatures")
        self.problem = problem
        self.heat_bc = heat_bc
        self.heat_flux = heat_flux
        self.solve_heat_first = solve_heat_first
        self._t0 = None if temperature is None else np.asarray(temperature, float)
        super().__init__(mesh, states, params, remesh_params, precision, dirichlet)
        self.dt = initial_dt
        self.max_dt = max_dt
        self.adapt_dt = adapt_dt
        self.coeff_inc = coeff_dt_increase
        self.coeff_dec = coeff_dt_decrease
        self.solve_succeeded = True
        self.last_status = None
        self.t_device = 0.0   # wall seconds in the device step calls
        self.t_remesh = 0.0   # wall seconds in the host remesh and re-upload

    def _upload(self, mesh, states, temperature=None):
        super()._upload(mesh, states)
        t = temperature if temperature is not None else self._t0
        if t is not None:
            self.ctx.set_temperature(t)

    def temperature(self):
        return self.ctx.get_temperature()

    def remesh(self):
        """`Mesh::remesh` on the host (positions and flags only); the node states and
        temperatures are remapped on the device from the new nodes' origins
        (`pfg_upload_mesh_remap`), so they never cross to the host."""
        if self.remesh_params is None:
            return
        cur = self.mesh.copy()
        cur.pos = self.ctx.get_positions()
        cur.flags = self.ctx.get_flags() & np.uint8(0x0F)
        new, origin = RM.remesh_map(cur, self.remesh_params)
        self.mesh = new
        self.ctx.upload_mesh_remap(new, origin)
        self._apply_dirichlet()

    def _heat(self):
        """`HeatEqIncompNewton::solve` with the BCs evaluated at t + dt on the current positions."""
        t = self.time + self.dt
        pos = self.ctx.get_positions()
        if self.heat_bc is not None:
            flags, tbc = self.heat_bc(pos, self.mesh.flags, t)
            self.ctx.heat_set_bc(flags, tbc)
        if self.heat_flux is not None and self.mesh.facets.shape[1]:
            self.ctx.heat_set_flux(H.flux_at_gauss_points(pos, self.mesh.facets, self.heat_flux, t))
        st = self.ctx.heat_step(self.dt)
        self.last_heat_status = st
        return bool(st.converged)

    def solve_one_time_step(self) -> bool:
        """`SolverIncompNewton::m_solveIncompNewtonNoT` / `m_solveBoussinesq` / `m_solveConduction`:
        on success the time advances and (but for Conduction) the mesh is rebuilt.  As in the
        reference, a Boussinesq step whose momentum solve fails keeps the temperatures of its
        heat solve (the node list is saved after it)."""
        if self.problem == "Conduction":
            self.solve_succeeded = self._heat()
            if self.solve_succeeded:
                self.time += self.dt
                self.steps += 1
            return self.solve_succeeded
        heat = self.problem == "Boussinesq"
        if heat and self.solve_heat_first and not self._heat():
            self.solve_succeeded = False
            return False
        t0 = time.perf_counter()
        st = self.ctx.picard_step(self.dt)
        self.t_device += time.perf_counter() - t0
        self.last_status = st
        self.solve_succeeded = bool(st.converged)
        if self.solve_succeeded and heat and not self.solve_heat_first:
            self.solve_succeeded = self._heat()
        if self.solve_succeeded:
            self.time += self.dt
            self.steps += 1
            t0 = time.perf_counter()
            self.remesh()
            self.t_remesh += time.perf_counter() - t0
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
