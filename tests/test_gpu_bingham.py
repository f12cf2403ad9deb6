"""GPU parity of the Bingham viscosity (problem "Bingham": mu + tau0 (1 - exp(-mReg gd)) / gd per
element, gd the strain-rate norm of the Picard iterate; MomContEquation.inl:54-58,102-121)
against the FP64 oracle.  Material of the reference's Bingham example (dbDellaVecchia:
mu = 300, tau0 = 50, mReg = 1000, rho = 1000).

Tolerances as for the Newtonian fluid: assembled values and RHS 1e-12 relative to their row
scale, Picard steps 1e-8 relative per field with the oracle's Picard iteration counts.
"""
import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import api
from pfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu

MU, TAU0, MREG = 300.0, 50.0, 1000.0


DT, MIN_RES = 5e-6, 1e-4  # the example's initial time step and Picard minRes: the Picard
                          # iteration on the strongly nonlinear viscosity contracts ~10x per
                          # iteration there, only ~2x at dt = 1e-4 (the oracle then fails too)


def make_ctx(mesh, precision=api.PREC_FP64, **kw):
    p = api.default_params(api.KIND_INCOMP_PSPG, mesh.dim)
    p.precision = precision
    p.mu, p.tau0, p.m_reg = MU, TAU0, MREG
    p.picard_min_res = MIN_RES
    for k, v in kw.items():
        setattr(p, k, v)
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    return ctx


def gravity(d):
    return (0.0, -9.81) if d == 2 else (0.0, 0.0, -9.81)


@pytest.mark.parametrize("which", ["c1", "3d"])
def test_bingham_assembly_matches_oracle(gpu_lib, which, c1_mesh, small3d_mesh):
    mesh = c1_mesh if which == "c1" else small3d_mesh
    d, N = mesh.dim, mesh.n_nodes
    rng = np.random.default_rng(21)
    q_iter = rng.uniform(-0.05, 0.05, (d + 1) * N)
    q_iter[:N] = 0.0  # a sheared patch: some elements near gd = 0, most well above 1/mReg
    q_prev = rng.uniform(-0.05, 0.05, (d + 1) * N)
    ctx = make_ctx(mesh)
    ctx.pspg_assemble(1e-3, q_iter, q_prev, apply_bc=True)
    rp, ci, va, b = ctx.get_csr()
    om = O.OracleMesh(mesh)
    A, b_o = O.pspg_assemble(om, 1000.0, MU, 1e-3, gravity(d), q_iter, q_prev, tau0=TAU0, m_reg=MREG)
    A0, _ = O.pspg_assemble(om, 1000.0, MU, 1e-3, gravity(d), q_iter, q_prev)
    csr, csr0 = A.tocsr(), A0.tocsr()
    csr.sort_indices()
    csr0.sort_indices()
    assert np.abs(csr.data - csr0.data).max() > 1e-3 * np.abs(csr.data).max()  # the law matters here
    assert np.array_equal(ci, csr.indices)
    worst = 0.0
    for r in range(len(rp) - 1):
        a, o = va[rp[r]:rp[r + 1]], csr.data[rp[r]:rp[r + 1]]
        worst = max(worst, np.abs(a - o).max() / max(np.abs(o).max(), 1e-300))
    assert worst < 1e-12
    bscale = np.maximum(np.abs(b_o), np.abs(csr).max(axis=1).toarray().ravel() * 1e-3)
    assert (np.abs(b - b_o) / np.maximum(bscale, 1e-300)).max() < 1e-12


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_bingham_picard_steps_match_oracle(gpu_lib, c1_mesh, precision):
    mesh = c1_mesh
    d, N = mesh.dim, mesh.n_nodes
    q0 = M.incomp_initial_states(mesh)
    ctx = make_ctx(mesh, precision)
    ctx.set_states(q0)
    om = O.OracleMesh(mesh)
    qo = q0.copy()
    for step in range(3):
        st = ctx.picard_step(DT)
        qo, res = O.pspg_picard_step(om, qo, DT, mu=MU, g=gravity(d), tau0=TAU0, m_reg=MREG, min_res=MIN_RES)
        assert st.converged == 1 and res.converged
        assert st.picard_iterations == res.iterations
        q = ctx.get_states()
        errs = [np.linalg.norm(q[f * N:(f + 1) * N] - qo[f * N:(f + 1) * N]) /
                max(np.linalg.norm(qo[f * N:(f + 1) * N]), 1e-30) for f in range(d + 1)]
        assert max(errs) < 1e-8, (step, errs)
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-12


def test_yield_stress_slows_the_collapse(gpu_lib, c1_mesh):
    """Same column, Newtonian (mu) against Bingham (mu, tau0): the yield stress stiffens the
    slowly sheared fluid, so after a few steps it moves less."""
    q0 = M.incomp_initial_states(c1_mesh)
    vmax = []
    for tau0 in (0.0, TAU0):
        ctx = make_ctx(c1_mesh, api.PREC_MIXED, tau0=tau0)
        ctx.set_states(q0)
        for _ in range(5):
            assert ctx.picard_step(DT).converged == 1
        v = ctx.get_states()[:2 * c1_mesh.n_nodes]
        vmax.append(np.abs(v).max())
    assert vmax[1] < vmax[0]


def test_bingham_parameters_checked(gpu_lib):
    p = api.default_params(api.KIND_INCOMP_PSPG, 2)
    p.tau0 = 10.0  # m_reg missing
    with pytest.raises(api.PfgError):
        api.Context(p)
    q = api.default_params(api.KIND_WC_CDS_DPDT, 2)
    q.tau0, q.m_reg = 10.0, 100.0
    with pytest.raises(api.PfgError):
        api.Context(q)
