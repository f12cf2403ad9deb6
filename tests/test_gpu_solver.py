"""Host solver classes (time loop, dt control, remesh handoff) driving the GPU library,
against the same loop driven by the FP64 oracle.  Tolerance: states within 1e-8 relative per
field after several remeshed steps (the host remesh sees positions that agree to ~1e-13)."""
import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import api
from pfem_gb300 import mesh as M
from pfem_gb300 import remesh as R
from pfem_gb300 import solver as S

pytestmark = pytest.mark.gpu

PRM = R.RemeshParams(hchar=0.1, omega=0.7, gamma=0.2, bounding_box=(-0.01, -1.0, 4.01, 100.0))


def test_incomp_solver_with_remesh_matches_oracle_loop(gpu_lib):
    mesh = M.dam_break_2d(0.1)
    q0 = M.incomp_initial_states(mesh)
    sol = S.SolverIncompNewtonGPU(mesh, q0, remesh_params=PRM)
    vols = []
    prob = S.Problem(sol, max_time=1.0, extractors=[S.mass_extractor(vols)])
    n = prob.simulate(max_steps=6)
    assert n == 6 and sol.steps >= 5
    # same loop on the oracle
    m, q, dt, t = mesh, q0.copy(), 1e-3, 0.0
    for _ in range(6):
        om = O.OracleMesh(m)
        qn, res = O.pspg_picard_step(om, q, dt)
        if res.converged:
            t += dt
            cur = m.copy()
            cur.pos = om.positions
            m, q = R.remesh(cur, qn, PRM)
            dt = min(1e-3, dt * 1.5)
        else:
            dt /= 2
    assert sol.mesh.n_nodes == m.n_nodes and np.array_equal(sol.mesh.conn, m.conn)
    qg = sol.states()
    N = m.n_nodes
    for f in range(3):
        a, b = qg[f * N:(f + 1) * N], q[f * N:(f + 1) * N]
        assert np.linalg.norm(a - b) <= 1e-8 * max(np.linalg.norm(b), 1e-30)
    assert sol.time == pytest.approx(t)
    assert all(v > 0 for _, v in vols)
    sol.close()


def test_wc_solver_remeshes_on_schedule(gpu_lib):
    mesh = M.dam_break_2d(0.05)
    p = api.default_params(api.KIND_WC_CDS_DPDT, 2)
    p.max_dt = 2e-4
    sol = S.SolverWCompNewtonGPU(mesh, M.wc_initial_states(mesh), params=p,
                                 remesh_params=R.RemeshParams(hchar=0.05, omega=0.6, gamma=0.6, add_on_fs=True))
    masses = []
    prob = S.Problem(sol, max_time=1e-3, extractors=[S.mass_extractor(masses)])
    prob.simulate(max_steps=400)
    assert sol.time >= 1e-3 or sol.steps == 400
    assert sol.next_remesh > 2e-4                      # at least one remesh happened
    assert np.all(np.isfinite(sol.states()))
    m0 = masses[0][1]
    assert all(abs(mm - m0) / m0 < 0.05 for _, mm in masses)
    sol.close()


def test_extractors_write_gmsh_and_csv(gpu_lib, tmp_path):
    from pfem_gb300 import output as OUT

    mesh = M.dam_break_2d(0.1)
    sol = S.SolverIncompNewtonGPU(mesh, M.incomp_initial_states(mesh), remesh_params=PRM)
    gm = OUT.GmshExtractor(str(tmp_path / "results.msh"), 2e-3, what=("p", "ke", "u", "v"))
    mass = OUT.CsvExtractor(str(tmp_path / "mass.txt"), 1e-3, "mass")
    tip = OUT.CsvExtractor(str(tmp_path / "tip.txt"), 1e-3, "minmax", coordinate=0, min_max="max")
    S.Problem(sol, max_time=1.0, extractors=[gm, mass, tip]).simulate(max_steps=4)
    assert len(gm.written) >= 2
    rows = [list(map(float, l.split(","))) for l in open(tmp_path / "mass.txt")]
    assert len(rows) >= 3 and all(r[1] > 0 for r in rows)
    tips = [list(map(float, l.split(","))) for l in open(tmp_path / "tip.txt")]
    assert all(0.9 < t[1] < 4.0 for t in tips)
    sol.close()


def test_boussinesq_solver_matches_oracle_loop(gpu_lib):
    """`m_solveBoussinesq` with solveHeatFirst (heat, then momentum on the new temperatures)
    against the oracle-driven loop; wall nodes held at a hot bottom / cold rest, free-surface
    convection.  Without remesh: the remesh carrying T is checked bitwise by the device-remap
    test, and with independent host remeshes both loops may break a Delaunay tie of the lattice
    differently once their positions differ in the last bits."""
    mesh = M.dam_break_2d(0.1)
    q0 = M.incomp_initial_states(mesh)
    T0 = np.full(mesh.n_nodes, 650.0)
    alpha, tr, h, tinf = 69e-6, 650.0, 5.0, 300.0

    def heat_bc(pos, flags, t):
        bound = (flags & M.BOUND) != 0
        fl = np.where(bound, api.HEAT_T, 0).astype(np.uint8)
        return fl, np.where(pos[1] < 0.05, 1000.0, 650.0) * bound

    p = api.default_params(api.KIND_INCOMP_PSPG, 2)
    p.boussinesq, p.alpha_t, p.t_ref = 1, alpha, tr
    p.heat_k, p.heat_cv, p.heat_h, p.heat_t_inf, p.heat_fs_flags = 0.6, 4.0, h, tinf, api.HEAT_QH
    sol = S.SolverIncompNewtonGPU(mesh, q0, params=p, problem="Boussinesq", temperature=T0, heat_bc=heat_bc)
    S.Problem(sol, max_time=1.0).simulate(max_steps=4)
    hp = O.heat_params(1000.0, 4.0, 0.6, h=h, t_inf=tinf, fs_flags=O.HT_QH)
    m, q, T, dt = mesh.copy(), q0.copy(), T0.copy(), 1e-3
    for _ in range(4):
        om = O.OracleMesh(m)
        fl, tbc = heat_bc(m.pos, m.flags, 0.0)
        T = O.heat_step(om, hp, dt, T, fl, tbc)
        q, res = O.pspg_picard_step(om, q, dt, boussinesq=(alpha, tr, T))
        assert res.converged
        m = m.copy()
        m.pos = om.positions
        dt = min(1e-3, dt * 1.5)
    assert sol.steps == 4
    assert np.abs(sol.positions() - m.pos).max() < 1e-12
    assert np.abs(sol.temperature() - T).max() <= 1e-10 * np.abs(T).max()
    qg, N = sol.states(), m.n_nodes
    for f in range(3):
        a, b = qg[f * N:(f + 1) * N], q[f * N:(f + 1) * N]
        assert np.linalg.norm(a - b) <= 1e-8 * max(np.linalg.norm(b), 1e-30)
    sol.close()


def test_conduction_solver_keeps_the_mesh(gpu_lib):
    """`m_solveConduction`: heat only, fixed mesh, time advances by dt per accepted step."""
    mesh = M.dam_break_2d(0.1)
    p = api.default_params(api.KIND_INCOMP_PSPG, 2)
    p.rho, p.heat_k, p.heat_cv = 1.0, 237.0, 1000.0
    T0 = 10 * np.exp(-((mesh.pos[0] - 0.5) ** 2 + (mesh.pos[1] - 0.5) ** 2) / 0.05)
    sol = S.SolverIncompNewtonGPU(mesh, M.incomp_initial_states(mesh), params=p, problem="Conduction",
                                  temperature=T0, initial_dt=0.025, max_dt=0.1)
    S.Problem(sol, max_time=0.2).simulate(max_steps=10)
    assert sol.time >= 0.2 - 1e-12 and np.array_equal(sol.positions(), mesh.pos)
    om = O.OracleMesh(mesh)
    hp = O.heat_params(1.0, 1000.0, 237.0)
    T, dt, t = T0.copy(), 0.025, 0.0
    while t < 0.2:
        T = O.heat_step(om, hp, dt, T, np.zeros(mesh.n_nodes, np.uint8))
        t += dt
        dt = min(0.1, dt * 1.5)
    assert np.abs(sol.temperature() - T).max() <= 1e-10 * np.abs(T).max()
    sol.close()


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_device_state_remap_equals_host_remap(gpu_lib, precision):
    """`pfg_upload_mesh_remap` gathers the states and temperatures of the new nodes on the device
    from the host remesh's origin table: bitwise the host remap (`remesh.remesh`)."""
    mesh = M.dam_break_2d(0.1)
    rng = np.random.default_rng(5)
    N = mesh.n_nodes
    q = rng.standard_normal(3 * N)
    T = 300 + 50 * rng.random(N)
    p = api.default_params(api.KIND_INCOMP_PSPG, 2)
    p.precision = precision
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    ctx.set_states(q)
    ctx.set_temperature(T)
    cur = mesh.copy()
    cur.pos = mesh.pos + 0.02 * rng.standard_normal(mesh.pos.shape) * ((mesh.flags & M.BOUND) == 0)
    new, origin = R.remesh_map(cur, PRM)
    new_h, st_h = R.remesh(cur, np.concatenate([q, T]), PRM)
    assert np.array_equal(new.conn, new_h.conn) and (origin[:, 1] >= 0).any()
    ctx.upload_mesh_remap(new, origin)
    n2 = new.n_nodes
    assert np.array_equal(ctx.get_states(), st_h[:3 * n2])
    assert np.array_equal(ctx.get_temperature(), st_h[3 * n2:])
    bad = origin.copy()
    bad[0, 0] = 10 ** 6
    with pytest.raises(api.PfgError):
        ctx.upload_mesh_remap(new, bad)
    ctx.close()
