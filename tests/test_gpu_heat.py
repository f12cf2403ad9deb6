"""GPU parity of the heat equation (HeatEqIncompNewton, IncompNewton/HeatEquation.inl) and of the
Boussinesq coupling of the PSPG momentum (problem "Boussinesq", MomContEquation.inl:164-199)
against the FP64 oracle, through the C ABI.

Tolerances: heat steps within 1e-10 of the oracle relative to the largest temperature (the
device solves the SPD system by CG to ||r|| <= 1e-14 ||b||, the oracle by sparse LU);
Boussinesq Picard steps 1e-8 relative per field with the oracle's Picard iteration counts, as
for the Newtonian fluid.
"""
import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import api
from pfem_gb300 import heat as H
from pfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu

RHO, CV, K = 1000.0, 4.0, 0.6
ALPHA, TR = 69e-6, 650.0


def gravity(d):
    return (0.0, -9.81) if d == 2 else (0.0, 0.0, -9.81)


def make_ctx(mesh, precision=api.PREC_FP64, **kw):
    p = api.default_params(api.KIND_INCOMP_PSPG, mesh.dim)
    p.precision = precision
    p.rho, p.heat_cv, p.heat_k = RHO, CV, K
    for k, v in kw.items():
        setattr(p, k, v)
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    return ctx


def _flux(x, t):
    return np.array([30.0 + 5.0 * x[0], -20.0 + 8.0 * x[1], 4.0 * x[-1]][:len(x)])


def _scenario(mesh, name):
    """(node flags, Dirichlet values, params overrides, free-surface flags, flux at facet GPs)"""
    N, d = mesh.n_nodes, mesh.dim
    bound = (mesh.flags & M.BOUND) != 0
    fl = np.zeros(N, np.uint8)
    tbc = np.zeros(N)
    kw, fs, q = {}, 0, None
    if name == "dirichlet_convection_radiation":
        fl[bound] = api.HEAT_T
        tbc[bound] = 300.0 + 20.0 * mesh.pos[0, bound]
        kw = dict(heat_h=8.0, heat_t_inf=250.0, heat_eps_rad=0.8)
        fs = api.HEAT_QH | api.HEAT_QR
    elif name == "flux_convection":
        fl[bound] = api.HEAT_Q
        q = H.flux_at_gauss_points(mesh.pos, mesh.facets, _flux, 0.0)
        kw = dict(heat_h=5.0, heat_t_inf=280.0)
        fs = api.HEAT_QH
    return fl, tbc, kw, fs, q


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
@pytest.mark.parametrize("name", ["none", "dirichlet_convection_radiation", "flux_convection"])
@pytest.mark.parametrize("which", ["c1", "3d"])
def test_heat_steps_match_oracle(gpu_lib, which, name, precision, c1_mesh, small3d_mesh):
    """FP64 Jacobi CG, or (mixed precision) FP32 CG corrections under FP64 refinement to the same
    tolerance: within 1e-10 of the oracle's LU steps either way."""
    mesh = c1_mesh if which == "c1" else small3d_mesh
    N = mesh.n_nodes
    fl, tbc, kw, fs, q = _scenario(mesh, name)
    ctx = make_ctx(mesh, precision, heat_fs_flags=fs, **kw)
    t0 = 300.0 + 100.0 * np.exp(-((mesh.pos[0] - 0.3) ** 2 + (mesh.pos[1] - 0.3) ** 2) / 0.05)
    ctx.set_temperature(t0)
    ctx.heat_set_bc(fl, tbc)
    if q is not None:
        ctx.heat_set_flux(q)
    om = O.OracleMesh(mesh)
    p = O.heat_params(RHO, CV, K, h=kw.get("heat_h", 0.0), t_inf=kw.get("heat_t_inf", 0.0),
                      eps_rad=kw.get("heat_eps_rad", 0.0), fs_flags=fs)
    to = t0.copy()
    for step in range(3):
        dt = 0.05 * (step + 1)
        st = ctx.heat_step(dt)
        to = O.heat_step(om, p, dt, to, fl, tbc, q)
        assert st.converged == 1 and st.krylov_iterations > 0
        t = ctx.get_temperature()
        err = np.abs(t - to).max() / np.abs(to).max()
        assert err < 1e-10, (step, err)
    assert np.abs(to - t0).max() > 1e-6 * np.abs(t0).max()  # the step changed the field


def test_heat_conditions_checked(gpu_lib, c1_mesh):
    ctx = make_ctx(c1_mesh)
    N = c1_mesh.n_nodes
    fl = np.zeros(N, np.uint8)
    bad = fl.copy()
    bad[0] = api.HEAT_T | api.HEAT_QH
    with pytest.raises(api.PfgError):
        ctx.heat_set_bc(bad, np.zeros(N))
    fl[(c1_mesh.flags & M.BOUND) != 0] = api.HEAT_Q
    ctx.heat_set_bc(fl)
    with pytest.raises(api.PfgError):  # Q facets without flux vectors
        ctx.heat_step(0.01)
    with pytest.raises(api.PfgError):
        ctx.heat_step(-1.0)
    p = api.default_params(api.KIND_WC_CDS_DPDT, 2)
    p.boussinesq = 1
    with pytest.raises(api.PfgError):
        api.Context(p)


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
@pytest.mark.parametrize("which", ["c1", "3d"])
def test_boussinesq_picard_steps_match_oracle(gpu_lib, which, precision, c1_mesh, small3d_mesh):
    """A stratified temperature field (hot at the bottom) under the Boussinesq body force."""
    mesh = c1_mesh if which == "c1" else small3d_mesh
    d, N = mesh.dim, mesh.n_nodes
    column = (1.0, 2.0) if d == 2 else (0.2, 0.3, 0.3)
    q0 = M.incomp_initial_states(mesh, column=column)
    T = 900.0 - 200.0 * mesh.pos[d - 1] + 30.0 * np.sin(7 * mesh.pos[0])
    ctx = make_ctx(mesh, precision, boussinesq=1, alpha_t=ALPHA, t_ref=TR)
    ctx.set_states(q0)
    ctx.set_temperature(T)
    om = O.OracleMesh(mesh)
    qo = q0.copy()
    for step in range(3):
        st = ctx.picard_step(1e-3)
        qo, res = O.pspg_picard_step(om, qo, 1e-3, g=gravity(d), boussinesq=(ALPHA, TR, T))
        assert st.converged == 1 and res.converged
        assert st.picard_iterations == res.iterations
        q = ctx.get_states()
        errs = [np.linalg.norm(q[f * N:(f + 1) * N] - qo[f * N:(f + 1) * N]) /
                max(np.linalg.norm(qo[f * N:(f + 1) * N]), 1e-30) for f in range(d + 1)]
        assert max(errs) < 1e-8, (step, errs)
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-12
    # the buoyancy matters: the same steps without it differ
    ctx0 = make_ctx(mesh, precision)
    ctx0.set_states(q0)
    for _ in range(3):
        ctx0.picard_step(1e-3)
    q0n = ctx0.get_states()
    assert np.linalg.norm(q0n[d * N:] - q[d * N:]) > 1e-6 * np.linalg.norm(q[d * N:])


def test_boussinesq_coupled_steps_match_oracle(gpu_lib, c1_mesh):
    """SolverIncompNewton::m_solveBoussinesq (Solver.cpp:249-284) with solveHeatFirst: heat
    step, then the momentum Picard step on the new temperatures, three times (no remesh)."""
    mesh = c1_mesh
    d, N = 2, mesh.n_nodes
    q0 = M.incomp_initial_states(mesh)
    T = 650.0 + 300.0 * (mesh.pos[1] < 0.2)
    bound = (mesh.flags & M.BOUND) != 0
    fl = np.zeros(N, np.uint8)
    fl[bound] = api.HEAT_T
    tbc = np.where(mesh.pos[1] < 0.05, 1000.0, 650.0) * bound
    ctx = make_ctx(mesh, boussinesq=1, alpha_t=ALPHA, t_ref=TR, heat_h=5.0, heat_t_inf=300.0,
                   heat_fs_flags=api.HEAT_QH)
    ctx.set_states(q0)
    ctx.set_temperature(T)
    ctx.heat_set_bc(fl, tbc)
    om = O.OracleMesh(mesh)
    p = O.heat_params(RHO, CV, K, h=5.0, t_inf=300.0, fs_flags=O.HT_QH)
    qo, to = q0.copy(), T.copy()
    for step in range(3):
        sth = ctx.heat_step(1e-3)
        to = O.heat_step(om, p, 1e-3, to, fl, tbc)
        st = ctx.picard_step(1e-3)
        qo, res = O.pspg_picard_step(om, qo, 1e-3, g=gravity(d), boussinesq=(ALPHA, TR, to))
        assert sth.converged == 1 and st.converged == 1 and res.converged
        t = ctx.get_temperature()
        assert np.abs(t - to).max() / np.abs(to).max() < 1e-10
        q = ctx.get_states()
        errs = [np.linalg.norm(q[f * N:(f + 1) * N] - qo[f * N:(f + 1) * N]) /
                max(np.linalg.norm(qo[f * N:(f + 1) * N]), 1e-30) for f in range(d + 1)]
        assert max(errs) < 1e-8, (step, errs)


TM, DTM, LM = 933.15, 20.0, 396000.0  # the reference's phase-change example (aluminium)


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
@pytest.mark.parametrize("residual", [api.RES_T, api.RES_AX_F])
@pytest.mark.parametrize("which", ["c1", "3d"])
def test_heat_phase_change_picard_matches_oracle(gpu_lib, which, residual, precision, c1_mesh, small3d_mesh):
    """HeatEqIncompNewton with phase change: Picard iterations on the latent-heat mass factor
    (HeatEquation.inl:60-66, 131-138), the same outcome and iteration count as the oracle.  The
    absolute "Ax_f" residual of this system contracts ~5x per iteration, so in 3D neither side
    reaches minRes within maxIter: both fail and restore."""
    mesh = c1_mesh if which == "c1" else small3d_mesh
    N = mesh.n_nodes
    kw = dict(heat_h=500.0, heat_t_inf=300.0, heat_fs_flags=api.HEAT_QH)
    ctx = make_ctx(mesh, precision, rho=2385.0, heat_cv=1080.0, heat_k=94.03, heat_phase_change=1, heat_tm=TM,
                   heat_dt_melt=DTM, heat_lm=LM, heat_residual=residual, **kw)
    t0 = np.full(N, TM + 5.0) + 2 * np.sin(3 * mesh.pos[0])
    ctx.set_temperature(t0)
    om = O.OracleMesh(mesh)
    p = O.heat_params(2385.0, 1080.0, 94.03, h=500.0, t_inf=300.0, fs_flags=O.HT_QH, phase_change=(TM, DTM, LM))
    fl = np.zeros(N, np.uint8)
    to = t0.copy()
    for step in range(2):
        st = ctx.heat_step(1.0)
        r = {}
        to = O.heat_step(om, p, 1.0, to, fl, residual="T" if residual == api.RES_T else "Ax_f", result=r)
        assert st.converged == int(r["converged"]) and st.picard_iterations == r["iterations"]
        assert st.picard_iterations >= 2
        if residual == api.RES_T or which == "c1":
            assert st.converged == 1
        t = ctx.get_temperature()
        assert np.abs(t - to).max() / np.abs(to).max() < 1e-10, step


def test_heat_phase_change_failure_restores(gpu_lib, c1_mesh):
    """A Picard loop that does not reach minRes in maxIter + 1 passes fails and restores the
    temperatures, as PicardAlgo::solve does (PicardAlgo.cpp:52-61), like the oracle."""
    mesh = c1_mesh
    N = mesh.n_nodes
    ctx = make_ctx(mesh, rho=2385.0, heat_cv=1080.0, heat_k=94.03, heat_phase_change=1, heat_tm=TM,
                   heat_dt_melt=DTM, heat_lm=LM, heat_max_iter=1, heat_min_res=1e-14, heat_h=500.0,
                   heat_t_inf=300.0, heat_fs_flags=api.HEAT_QH)
    t0 = np.full(N, TM + 5.0) + 2 * np.sin(3 * mesh.pos[0])
    ctx.set_temperature(t0)
    st = ctx.heat_step(1.0)
    om = O.OracleMesh(mesh)
    r = {}
    to = O.heat_step(om, O.heat_params(2385.0, 1080.0, 94.03, h=500.0, t_inf=300.0, fs_flags=O.HT_QH,
                                       phase_change=(TM, DTM, LM)), 1.0, t0, np.zeros(N, np.uint8),
                     max_iter=1, min_res=1e-14, result=r)
    assert st.converged == 0 and not r["converged"]
    assert st.picard_iterations == r["iterations"] == 2
    assert np.array_equal(ctx.get_temperature(), t0) and np.array_equal(to, t0)


def test_heat_free_nodes(gpu_lib, c1_mesh):
    """Nodes in no element (flying drops after a remesh): identity rows, T kept, or set when the
    node is a Dirichlet node (HeatEquation.inl:287-293, 380-389), as in the oracle."""
    base = c1_mesh
    m = base.copy()
    extra = np.array([[3.5, 3.6], [2.5, 2.6]])
    m.pos = np.concatenate([base.pos, extra], axis=1)
    m.flags = np.concatenate([base.flags, np.zeros(2, np.uint8)])
    N = m.n_nodes
    ctx = make_ctx(m, heat_h=5.0, heat_t_inf=300.0, heat_fs_flags=api.HEAT_QH)
    t0 = 300.0 + 50.0 * np.sin(2 * m.pos[0])
    fl = np.zeros(N, np.uint8)
    fl[N - 1] = api.HEAT_T
    tbc = np.zeros(N)
    tbc[N - 1] = 777.0
    ctx.set_temperature(t0)
    ctx.heat_set_bc(fl, tbc)
    st = ctx.heat_step(0.05)
    om = O.OracleMesh(m)
    assert om.is_free()[N - 2] and om.is_free()[N - 1]
    to = O.heat_step(om, O.heat_params(RHO, CV, K, h=5.0, t_inf=300.0, fs_flags=O.HT_QH), 0.05, t0, fl, tbc)
    t = ctx.get_temperature()
    assert st.converged == 1
    # identity rows: exact in the oracle's LU, to the CG tolerance on the device
    assert t[N - 2] == pytest.approx(t0[N - 2], rel=1e-12) and t[N - 1] == pytest.approx(777.0, rel=1e-12)
    assert np.abs(t - to).max() / np.abs(to).max() < 1e-10
