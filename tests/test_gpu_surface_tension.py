"""GPU parity of the surface tension term (gamma > 0) against the FP64 oracle, through the C ABI.

Cases: the reference's surface tension example, a free unit square of fluid relaxing to a disk
(`examples/2D/squareToDisk`: no walls, h = 0.025, rho = 100, mu = 1, gamma = 1.9; WC variant
K0 = 2.2e5, K0' = 7.6, rho* = 100, securityCoeff = 0.025), a free disk and a free ball.

Tolerances: the assembled right-hand side 1e-12 relative to its row scale (as with gamma = 0);
Picard steps 1e-8 relative per field (both precisions stop on the same FP64 residual test);
WC steps 1e-10 relative per field in FP64, 1e-5 for v, p, rho in the mixed form (FP32
arithmetic, double-float state).
"""
import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import api
from pfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu

GAMMA = 1.9


@pytest.fixture(scope="module")
def square():
    return M.square_to_disk_2d(0.025)


@pytest.fixture(scope="module")
def ball():
    return M.ball_3d(0.1, 0.02)


def disk(R=0.1, h=0.01):
    pts = [np.zeros((1, 2))]
    nr = int(round(R / h))
    for k in range(1, nr + 1):
        r = R * k / nr
        m = max(6, int(round(2 * np.pi * r / h)))
        a = 0.37 * k + 2 * np.pi * np.arange(m) / m
        pts.append(r * np.stack([np.cos(a), np.sin(a)], 1))
    pos = np.concatenate(pts).T.copy()
    return M.alpha_shape(pos, np.zeros(pos.shape[1], np.uint8), h, 1.2)


def incomp_ctx(mesh, precision=api.PREC_FP64, **kw):
    p = api.default_params(api.KIND_INCOMP_PSPG, mesh.dim)
    p.precision = precision
    p.gamma = GAMMA
    p.rho, p.mu = 100.0, 1.0
    p.gravity[:] = [0.0, 0.0, 0.0]
    for k, v in kw.items():
        setattr(p, k, v)
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    return ctx


def field_errs(q, qo, nf, N):
    return [np.linalg.norm(q[f * N:(f + 1) * N] - qo[f * N:(f + 1) * N]) /
            max(np.linalg.norm(qo[f * N:(f + 1) * N]), 1e-30) for f in range(nf)]


@pytest.mark.parametrize("which", ["square", "ball"])
def test_assembly_rhs_matches_oracle(gpu_lib, which, square, ball):
    mesh = square if which == "square" else ball
    d, N = mesh.dim, mesh.n_nodes
    rng = np.random.default_rng(11)
    q_iter = rng.uniform(-0.05, 0.05, (d + 1) * N)
    q_prev = rng.uniform(-0.05, 0.05, (d + 1) * N)
    ctx = incomp_ctx(mesh)
    ctx.pspg_assemble(2.5e-3, q_iter, q_prev, apply_bc=True)
    rp, ci, va, b = ctx.get_csr()
    om = O.OracleMesh(mesh)
    A, b_o = O.pspg_assemble(om, 100.0, 1.0, 2.5e-3, (0.0,) * 3, q_iter, q_prev, gamma=GAMMA)
    _, b0 = O.pspg_assemble(om, 100.0, 1.0, 2.5e-3, (0.0,) * 3, q_iter, q_prev, gamma=0.0)
    assert np.abs(b_o - b0).max() > 1e-3 * np.abs(b0).max()    # the term is not negligible here
    bscale = np.maximum(np.abs(b_o), np.abs(A.tocsr()).max(axis=1).toarray().ravel() * 1e-3)
    assert (np.abs(b - b_o) / np.maximum(bscale, 1e-300)).max() < 1e-12


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_square_to_disk_picard_steps(gpu_lib, square, precision):
    mesh = square
    d, N = mesh.dim, mesh.n_nodes
    ctx = incomp_ctx(mesh, precision)
    q0 = np.zeros((d + 1) * N)
    ctx.set_states(q0)
    om = O.OracleMesh(mesh)
    qo = q0.copy()
    for step in range(3):
        st = ctx.picard_step(2.5e-3)
        qo, res = O.pspg_picard_step(om, qo, 2.5e-3, rho=100.0, mu=1.0, g=(0.0, 0.0), gamma=GAMMA)
        assert st.converged == 1 and res.converged
        assert st.picard_iterations == res.iterations
        errs = field_errs(ctx.get_states(), qo, d + 1, N)
        assert max(errs) < 1e-8, (step, errs)
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-12
    # the corners move inwards: the square starts to round off
    x = ctx.get_positions()
    corner = np.argmin(np.hypot(mesh.pos[0], mesh.pos[1]))
    assert x[0, corner] > 0 and x[1, corner] > 0


def test_disk_laplace_pressure(gpu_lib):
    """A disk at rest: one step gives the Laplace pressure gamma / R inside, within 0.5 %."""
    mesh = disk()
    fs = (mesh.flags & M.FREE_SURFACE) != 0
    N = mesh.n_nodes
    ctx = incomp_ctx(mesh, rho=1000.0, mu=1e-3, gamma=0.0728)
    ctx.set_states(np.zeros(3 * N))
    st = ctx.picard_step(1e-3)
    assert st.converged == 1
    q = ctx.get_states()
    p = q[2 * N:]
    assert abs(p[~fs].mean() / (0.0728 / 0.1) - 1) < 5e-3
    assert np.abs(q[:2 * N]).max() < 1e-9


def wc_ctx(mesh, precision):
    p = api.default_params(api.KIND_WC_CDS_DPDT, mesh.dim)
    p.precision = precision
    p.gamma = GAMMA
    p.mu, p.K0, p.K0p, p.rho_star = 1.0, 2.2e5, 7.6, 100.0
    p.security_coeff, p.max_dt = 0.025, 1e-3
    p.gravity[:] = [0.0, 0.0, 0.0]
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    return ctx


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_square_to_disk_wc_steps(gpu_lib, square, precision):
    mesh = square
    d, N = mesh.dim, mesh.n_nodes
    s0 = np.zeros((2 * d + 2) * N)
    s0[(d + 1) * N:(d + 2) * N] = 100.0
    ctx = wc_ctx(mesh, precision)
    ctx.set_states(s0)
    om = O.OracleMesh(mesh)
    p = O.wc_params(K0=2.2e5, K0p=7.6, rho_star=100.0, mu=1.0, g=(0.0, 0.0), sc=0.025, max_dt=1e-3, gamma=GAMMA)
    so = s0.copy()
    dt_o = O.wc_next_dt(om, p, so)
    ctx.set_time(0.0, ctx.next_dt())
    for _ in range(30):
        O.wc_step(om, p, dt_o, so)
        dt_o = O.wc_next_dt(om, p, so)
    ctx.wc_step(0.0, 30)
    errs = field_errs(ctx.get_states(), so, 2 * d + 2, N)
    if precision == api.PREC_FP64:
        assert max(errs) < 1e-10, errs
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-13
    else:
        assert max(errs[:d + 2]) < 1e-5, errs
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-9
    # without surface tension nothing would move: the square is at rest with no body force
    assert np.abs(so[:d * N]).max() > 1e-6


def test_gamma_needs_facets(gpu_lib, square):
    bare = square.copy()
    bare.facets = np.zeros((2, 0), np.int32)
    bare.facet_elm = np.zeros(0, np.int32)
    ctx = incomp_ctx(bare)
    ctx.set_states(np.zeros(3 * bare.n_nodes))
    with pytest.raises(api.PfgError, match="STATE"):
        ctx.picard_step(2.5e-3)
    bad = square.facets.copy()
    bad[0, 0] = (bad[0, 0] + 7) % square.n_nodes
    while bad[0, 0] in square.conn[:, square.facet_elm[0]]:
        bad[0, 0] = (bad[0, 0] + 1) % square.n_nodes
    with pytest.raises(api.PfgError, match="INVALID"):
        ctx.upload_facets(bad, square.facet_elm)
    ctx.upload_facets(square.facets, square.facet_elm)
    assert ctx.picard_step(2.5e-3).converged == 1


def _hot_spot(mesh):
    x = mesh.pos
    return 300.0 + 80.0 * np.exp(-((x[0] - 0.3) ** 2 + (x[1] - 0.4) ** 2) / 0.05)


DGDT = -5e-3  # Boussinesq surface tension slope DgammaDT (gamma + DgammaDT (T - Tr))


@pytest.mark.parametrize("which", ["square", "ball"])
def test_temperature_dependent_surface_tension_rhs(gpu_lib, which, square, ball):
    """Problem "Boussinesq": gamma + DgammaDT (T_g - Tr) at the facet Gauss points
    (MomContEquation.inl:174-179), with a non-uniform temperature and no buoyancy (alpha = 0)."""
    mesh = square if which == "square" else ball
    d, N = mesh.dim, mesh.n_nodes
    rng = np.random.default_rng(12)
    q_iter = rng.uniform(-0.05, 0.05, (d + 1) * N)
    q_prev = rng.uniform(-0.05, 0.05, (d + 1) * N)
    T = _hot_spot(mesh)
    ctx = incomp_ctx(mesh, boussinesq=1, alpha_t=0.0, t_ref=300.0, dgamma_dt=DGDT)
    ctx.set_temperature(T)
    ctx.pspg_assemble(2.5e-3, q_iter, q_prev, apply_bc=True)
    _, _, _, b = ctx.get_csr()
    om = O.OracleMesh(mesh)
    A, b_o = O.pspg_assemble(om, 100.0, 1.0, 2.5e-3, (0.0,) * 3, q_iter, q_prev, gamma=GAMMA,
                             boussinesq=(0.0, 300.0, T, DGDT))
    _, b1 = O.pspg_assemble(om, 100.0, 1.0, 2.5e-3, (0.0,) * 3, q_iter, q_prev, gamma=GAMMA)
    assert np.abs(b_o - b1).max() > 1e-4 * np.abs(b1 - O.pspg_assemble(
        om, 100.0, 1.0, 2.5e-3, (0.0,) * 3, q_iter, q_prev)[1]).max()  # the slope matters here
    bscale = np.maximum(np.abs(b_o), np.abs(A.tocsr()).max(axis=1).toarray().ravel() * 1e-3)
    assert (np.abs(b - b_o) / np.maximum(bscale, 1e-300)).max() < 1e-12


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_temperature_dependent_surface_tension_picard(gpu_lib, square, precision):
    mesh = square
    d, N = mesh.dim, mesh.n_nodes
    T = _hot_spot(mesh)
    ctx = incomp_ctx(mesh, precision, boussinesq=1, alpha_t=0.0, t_ref=300.0, dgamma_dt=DGDT)
    ctx.set_temperature(T)
    q0 = np.zeros((d + 1) * N)
    ctx.set_states(q0)
    om = O.OracleMesh(mesh)
    qo = q0.copy()
    for step in range(3):
        st = ctx.picard_step(2.5e-3)
        qo, res = O.pspg_picard_step(om, qo, 2.5e-3, rho=100.0, mu=1.0, g=(0.0, 0.0), gamma=GAMMA,
                                     boussinesq=(0.0, 300.0, T, DGDT))
        assert st.converged == 1 and res.converged
        assert st.picard_iterations == res.iterations
        errs = field_errs(ctx.get_states(), qo, d + 1, N)
        assert max(errs) < 1e-8, (step, errs)
