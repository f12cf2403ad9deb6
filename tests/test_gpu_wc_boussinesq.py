"""GPU parity of problem "BoussinesqWC" (SolverWCompNewton::m_solveBoussinesqWC,
WCompNewton/Solver.cpp:278-320) against the FP64 oracle, through the C ABI: the explicit
lumped-mass heat step of HeatEqWCompNewton between the half-step prediction and the continuity
equation (with Dirichlet, prescribed-flux, convection and radiation conditions), the
momentum's body force rho (1 - alpha (T - Tr)) and, with phase change, its Carman-Kozeny
damping, and the heat diffusion in the CFL time step.

Plain FP64 form, 20 adaptive steps: every state field and the temperatures within 1e-10
relative, the time step within 1e-11 (as for the Newtonian WC step).
"""
import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import api
from pfem_gb300 import heat as H
from pfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu

ALPHA, TR, K, CV = 2e-4, 300.0, 50.0, 500.0
PHASE = dict(C=1e3, eps=1e-3, Tm=300.0, DT=20.0, Lm=1e4)


def _flux(x, t):
    return np.array([3e3 + 5e2 * x[0], -2e3 + 8e2 * x[1], 4e2 * x[-1]][:len(x)])


def _scenario(mesh, name):
    """(heat flags, Dirichlet temperatures, parameter overrides, free-surface flags, flux at
    the facet Gauss points, initial temperatures, phase change)"""
    N = mesh.n_nodes
    y = mesh.pos[1]
    bound = (mesh.flags & M.BOUND) != 0
    fl = np.zeros(N, np.uint8)
    tbc = np.zeros(N)
    if name == "dirichlet_convection_radiation":
        fl[bound] = api.HEAT_T
        tbc[bound] = np.where(y[bound] < 0.05, 350.0, 300.0)
        T0 = 300.0 + 50.0 * (y < 0.3)
        return fl, tbc, dict(heat_h=10.0, heat_t_inf=280.0, heat_eps_rad=0.8), api.HEAT_QH | api.HEAT_QR, None, \
            T0, False
    fl[bound] = api.HEAT_Q
    q = H.flux_at_gauss_points(mesh.pos, mesh.facets, _flux, 0.0)
    T0 = 290.0 + 20.0 * (mesh.pos[0] < 0.5) + 5.0 * y
    return fl, tbc, dict(heat_h=5.0, heat_t_inf=280.0), api.HEAT_QH, q, T0, True


@pytest.mark.parametrize("name", ["dirichlet_convection_radiation", "flux_phase_change"])
@pytest.mark.parametrize("which", ["2d", "3d"])
def test_boussinesq_wc_matches_oracle(gpu_lib, which, name, c1_mesh, small3d_mesh):
    mesh = c1_mesh if which == "2d" else small3d_mesh
    d, N = mesh.dim, mesh.n_nodes
    fl, tbc, kw, fs, q, T0, pc = _scenario(mesh, name)
    p = api.default_params(api.KIND_WC_CDS_DPDT, d)
    p.precision = api.PREC_FP64
    p.boussinesq, p.alpha_t, p.t_ref, p.heat_k, p.heat_cv, p.heat_fs_flags = 1, ALPHA, TR, K, CV, fs
    for k, v in kw.items():
        setattr(p, k, v)
    if pc:
        p.heat_phase_change, p.heat_tm, p.heat_dt_melt, p.heat_lm = 1, PHASE["Tm"], PHASE["DT"], PHASE["Lm"]
        p.ck_c, p.ck_eps = PHASE["C"], PHASE["eps"]
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    s0 = M.wc_initial_states(mesh)
    ctx.set_states(s0)
    ctx.set_temperature(T0)
    ctx.heat_set_bc(fl, tbc)
    if q is not None:
        ctx.heat_set_flux(q.ravel())
    om = O.OracleMesh(mesh)
    po = O.wc_params(g=tuple(p.gravity[:d]))
    bq = O.wc_bq_params(ALPHA, TR, K, CV, h=kw.get("heat_h", 0.0), t_inf=kw.get("heat_t_inf", 0.0),
                        eps_rad=kw.get("heat_eps_rad", 0.0), fs_flags=fs, phase_change=PHASE if pc else None)
    so = np.concatenate([s0, T0])
    dt_o = O.wc_bq_next_dt(om, po, bq, so)
    dt_g = ctx.next_dt()
    assert dt_g == pytest.approx(dt_o, rel=1e-13)
    ctx.set_time(0.0, dt_g)
    for _ in range(20):
        O.wc_bq_step(om, po, bq, dt_o, so, fl, t_bc=tbc, q_gp=q)
        dt_o = O.wc_bq_next_dt(om, po, bq, so)
    st = ctx.wc_step(0.0, 20)
    assert st.dt == pytest.approx(dt_o, rel=1e-11)
    s = ctx.get_states()
    errs = [np.linalg.norm(s[f * N:(f + 1) * N] - so[f * N:(f + 1) * N]) /
            max(np.linalg.norm(so[f * N:(f + 1) * N]), 1e-30) for f in range(2 * d + 2)]
    assert max(errs) < 1e-10, errs
    t = ctx.get_temperature()
    to = so[(2 * d + 2) * N:]
    assert np.abs(t - to).max() / np.abs(to).max() < 1e-10
    assert np.abs(t - T0).max() > 1e-9  # the heat step did something
    assert np.abs(ctx.get_positions() - om.positions).max() < 1e-13


def test_boussinesq_wc_changes_the_flow(gpu_lib, c1_mesh):
    """The buoyancy term acts: with alpha > 0 and a temperature contrast the velocities differ
    from alpha = 0, and alpha = 0 gives the Newtonian WC step's states (to rounding: the body
    force is summed over the Gauss points instead of through the mass table)."""
    mesh = c1_mesh
    d, N = 2, mesh.n_nodes
    s0 = M.wc_initial_states(mesh)
    T0 = 300.0 + 80.0 * (mesh.pos[0] < 0.5)
    out = {}
    for alpha in (0.0, ALPHA, None):
        p = api.default_params(api.KIND_WC_CDS_DPDT, d)
        p.precision = api.PREC_FP64
        if alpha is not None:
            p.boussinesq, p.alpha_t, p.t_ref, p.heat_k, p.heat_cv = 1, alpha, TR, 1e-9, CV
        ctx = api.Context(p)
        ctx.upload_mesh(mesh)
        ctx.set_states(s0)
        if alpha is not None:
            ctx.set_temperature(T0)
        ctx.set_time(0.0, 1e-5)
        ctx.wc_step(1e-5, 10)
        out[alpha] = ctx.get_states()
    np.testing.assert_allclose(out[0.0], out[None], rtol=1e-12, atol=1e-12 * np.abs(out[None]).max())
    assert np.abs(out[ALPHA][:d * N] - out[0.0][:d * N]).max() > 1e-9


def test_boussinesq_wc_rejected_in_mixed_precision(gpu_lib):
    p = api.default_params(api.KIND_WC_CDS_DPDT, 2)
    p.precision = api.PREC_MIXED
    p.boussinesq, p.heat_cv, p.heat_k = 1, CV, K
    with pytest.raises(api.PfgError):
        api.Context(p)
