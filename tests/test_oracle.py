"""CPU checks of the FP64 oracle: known-answer element tests, the sparsity-pattern rule,
physics invariants (hydrostatic rest, mass conservation) and the Picard failure path."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import mesh as M

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "kat_elements.npz")


def _single_element_mesh(X):
    d = X.shape[1]
    return M.HostMesh(d, X.T.copy(), np.zeros(d + 1, np.uint8), np.arange(d + 1, dtype=np.int32).reshape(d + 1, 1))


@pytest.mark.parametrize("name", ["tri", "tri_skew", "tet", "tet_skew"])
def test_element_matrices_match_closed_forms(name):
    z = np.load(GOLDEN)
    rho, mu, dt = z["params"]
    X = z[name + "_X"]
    d = X.shape[1]
    om = O.OracleMesh(_single_element_mesh(X))
    N = d + 1
    qi = np.zeros((d + 1) * N)
    qp = np.zeros((d + 1) * N)
    qi[:d * N] = z[name + "_viter"].T.reshape(-1)
    qp[:d * N] = z[name + "_vprev"].T.reshape(-1)
    g = (0.0, -9.81, 0.0) if d == 2 else (0.0, 0.0, -9.81)
    Ae, be = O.pspg_element(om, 0, rho, mu, dt, g, qi, qp)
    tol = 1e-13 if d == 2 else 1e-12  # 3D Gauss points are 15-digit decimals in the reference
    assert np.abs(Ae - z[name + "_Ae"]).max() <= tol * np.abs(z[name + "_Ae"]).max()
    assert np.abs(be - z[name + "_be"]).max() <= tol * np.abs(z[name + "_be"]).max()
    _, det, _ = om.geometry()
    assert det[0] == pytest.approx(float(z[name + "_detJ"]), rel=1e-14)


def rule_pattern(mesh):
    """CSR pattern from the adjacency rule used by the GPU library (pfg_mesh.cu)."""
    d, N = mesh.dim, mesh.n_nodes
    free = mesh.is_free()
    bound = (mesh.flags & M.BOUND) != 0
    nbr = [set([n]) for n in range(N)]
    for e in range(mesh.n_elems):
        nodes = mesh.conn[:, e]
        for a in nodes:
            nbr[a].update(int(b) for b in nodes)
    rows, cols = [], []
    for f in range(d + 1):
        for n in range(N):
            r = n + f * N
            if free[n] or (bound[n] and f < d):
                rows.append(r)
                cols.append(r)
                continue
            ns = sorted(nbr[n])
            for f2 in range(d + 1):
                for m in ns:
                    rows.append(r)
                    cols.append(m + f2 * N)
    return np.array(rows), np.array(cols)


@pytest.mark.parametrize("which", ["c1", "3d"])
def test_pattern_rule_matches_set_from_triplets(which, c1_mesh, small3d_mesh):
    mesh = c1_mesh if which == "c1" else small3d_mesh
    om = O.OracleMesh(mesh)
    d, N = mesh.dim, mesh.n_nodes
    q = np.zeros((d + 1) * N)
    g = (0.0, -9.81) if d == 2 else (0.0, 0.0, -9.81)
    A, _ = O.pspg_assemble(om, 1000.0, 1e-3, 1e-3, g, q, q)
    csr = A.tocsr()
    csr.sort_indices()
    rows, cols = rule_pattern(mesh)
    R = (d + 1) * N
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order]
    rp = np.zeros(R + 1, np.int64)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp)
    assert np.array_equal(csr.indptr, rp)
    assert np.array_equal(csr.indices, cols)


def test_hydrostatic_column_stays_at_rest():
    """KAT-3: a column filling the tank width is at equilibrium under hydrostatic pressure."""
    mesh = M.dam_break_2d(0.05, tank=(1.05, 3.0))
    om = O.OracleMesh(mesh)
    q0 = M.incomp_initial_states(mesh)
    q, res = O.pspg_picard_step(om, q0, 1e-3)
    N = mesh.n_nodes
    assert res.converged
    assert np.abs(q[:2 * N]).max() < 5e-3           # m/s, after one step from rest
    inner = ~mesh.is_free() & ((mesh.flags & M.FREE_SURFACE) == 0)
    p_err = np.abs(q[2 * N:] - q0[2 * N:])[inner]
    assert p_err.max() < 0.02 * q0[2 * N:].max()


def test_wc_mass_conserved_over_steps(wc_small_mesh):
    """KAT-4: the WC step keeps sum |e| mean(rho) nearly constant over many steps."""
    mesh = wc_small_mesh
    om = O.OracleMesh(mesh)
    s = M.wc_initial_states(mesh)
    p = O.wc_params()
    m0 = O.wc_mass(om, s)
    dt = O.wc_next_dt(om, p, s)
    for _ in range(50):
        O.wc_step(om, p, dt, s)
        dt = O.wc_next_dt(om, p, s)
    m1 = O.wc_mass(om, s)
    assert np.all(np.isfinite(s))
    assert abs(m1 - m0) / m0 < 1e-4
    assert 0 < dt <= p.maxDT


def test_picard_failure_restores_positions(c1_mesh):
    om = O.OracleMesh(c1_mesh)
    q0 = M.incomp_initial_states(c1_mesh)
    x0 = om.positions.copy()
    q, res = O.pspg_picard_step(om, q0, 1e-3, max_iter=0, min_res=1e-30)
    assert not res.converged
    assert np.array_equal(om.positions, x0)
    assert np.array_equal(q, q0)


def test_volume_and_tip(c1_mesh):
    om = O.OracleMesh(c1_mesh)
    assert om.volume() == pytest.approx(2.0, rel=2e-2)
    assert 0.95 < om.tip() < 1.06


def _disk(R=0.1, h=0.01):
    pts = [np.zeros((1, 2))]
    nr = int(round(R / h))
    for k in range(1, nr + 1):
        r = R * k / nr
        m = max(6, int(round(2 * np.pi * r / h)))
        a = 0.37 * k + 2 * np.pi * np.arange(m) / m
        pts.append(r * np.stack([np.cos(a), np.sin(a)], 1))
    pos = np.concatenate(pts).T.copy()
    return M.alpha_shape(pos, np.zeros(pos.shape[1], np.uint8), h, 1.2)


def test_surface_tension_forces_are_translation_free():
    """sum_i dN_i/dx = 0 in every element, so each facet's forces sum to zero; every force
    sits on a node of a free-surface facet's element."""
    for mesh in (M.square_to_disk_2d(0.05), M.ball_3d(0.1, 0.025)):
        om = O.OracleMesh(mesh)
        st = om.surface_tension(1.9)
        assert np.abs(st).max() > 1e-3
        assert np.abs(st.sum(axis=1)).max() < 1e-12 * np.abs(st).max()
        touched = np.zeros(mesh.n_nodes, bool)
        touched[mesh.conn[:, mesh.facet_elm].ravel()] = True
        assert np.all(st[:, ~touched] == 0.0)
        assert np.array_equal(om.surface_tension(0.0), np.zeros_like(st))


@pytest.mark.parametrize("dim", [2, 3])
def test_laplace_pressure_of_a_drop(dim):
    """A drop at rest with no gravity: one PSPG step gives the Laplace pressure jump inside
    (gamma / R in 2D, 2 gamma / R in 3D) and no motion."""
    mesh = _disk() if dim == 2 else M.ball_3d(0.1, 0.02)
    gamma, R = 0.0728, 0.1
    N = mesh.n_nodes
    fs = (mesh.flags & M.FREE_SURFACE) != 0
    om = O.OracleMesh(mesh)
    q, res = O.pspg_picard_step(om, np.zeros((dim + 1) * N), 1e-3, g=(0.0,) * dim, gamma=gamma)
    assert res.converged
    p = q[dim * N:]
    expect = (dim - 1) * gamma / R
    assert abs(p[~fs].mean() / expect - 1) < (5e-3 if dim == 2 else 2e-2)
    assert np.abs(q[:dim * N]).max() < (1e-9 if dim == 2 else 1e-3)


def test_invalid_facets_rejected(c1_mesh):
    om = O.OracleMesh(c1_mesh)
    bad = c1_mesh.facet_elm.copy()
    bad[0] = c1_mesh.n_elems
    with pytest.raises(ValueError):
        om.set_facets(c1_mesh.facets, bad)


def test_bingham_viscosity_in_simple_shear():
    """KAT: u = s y on one triangle is a simple shear with gd = s, so the viscous block of the
    Bingham element is (mu + tau0 (1 - exp(-mReg s)) / s) / mu times the Newtonian one."""
    X = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])  # nodes x coordinates
    mesh = _single_element_mesh(X)
    om = O.OracleMesh(mesh)
    N = mesh.n_nodes
    s = 0.37
    q = np.zeros(3 * N)
    q[:N] = s * X[:, 1]
    mu, tau0, mreg, dt = 2.0, 5.0, 40.0, 1e-3
    args = (1000.0, mu, dt, (0.0, -9.81))
    A_n, _ = O.pspg_element(om, 0, *args, q, q)
    A_b, _ = O.pspg_element(om, 0, *args, q, q, tau0=tau0, m_reg=mreg)
    A_m, _ = O.pspg_element(om, 0, 1000.0, 0.0, dt, (0.0, -9.81), q, q)  # mass part only (mu = 0)
    K_n, K_b = (A_n - A_m)[:6, :6], (A_b - A_m)[:6, :6]
    mue = mu + tau0 * (1 - np.exp(-mreg * s)) / s
    assert np.allclose(K_b, K_n * (mue / mu), rtol=1e-12, atol=1e-12 * np.abs(K_b).max())


# ---- heat equation and Boussinesq coupling (HeatEquation.inl, MomContEquation.inl:164-199) ----

def _heat_mesh(dim):
    return M.dam_break_2d(0.1, column=(1.0, 2.0), seed=5) if dim == 2 else M.dam_break_3d(0.1)


def _mass_total(om, t):
    """1^T M T: the heat content of the consistent mass matrix (cv rho = 1)."""
    A, _ = O.heat_assemble(om, O.heat_params(1.0, 1.0, 0.0), 1.0, t, np.zeros(om.N, np.uint8))
    return float(np.ones(om.N) @ (A @ t))


@pytest.mark.parametrize("dim", [2, 3])
def test_heat_conserves_energy_without_boundary_terms(dim):
    m = _heat_mesh(dim)
    om = O.OracleMesh(m)
    t0 = 300 + 50 * np.random.default_rng(1).random(m.n_nodes)
    p = O.heat_params(1000.0, 4.0, 0.6)
    t1 = O.heat_step(om, p, 0.05, t0, np.zeros(m.n_nodes, np.uint8))
    # L has zero row sums and is symmetric, so 1^T (M + dt L) = 1^T M: sum(M T) is conserved
    assert _mass_total(om, t1) == pytest.approx(_mass_total(om, t0), rel=1e-13)
    assert np.ptp(t1) < np.ptp(t0)  # diffusion flattens the field


@pytest.mark.parametrize("dim", [2, 3])
def test_heat_keeps_a_linear_field_with_matching_dirichlet_walls(dim):
    m = _heat_mesh(dim)
    om = O.OracleMesh(m)
    lin = 300 + 7 * m.pos[0] - 3 * m.pos[dim - 1]
    fl = np.where(m.flags & M.BOUND, O.HT_T, 0).astype(np.uint8)
    fl[(m.flags & M.FREE_SURFACE) != 0] = O.HT_T  # the whole boundary prescribed
    p = O.heat_params(1.0, 1.0, 5.0)
    t1 = O.heat_step(om, p, 0.1, lin, fl, t_bc=lin)
    # P1 Laplacian of a linear field vanishes at interior nodes, M T = M T_prev
    assert np.abs(t1 - lin).max() < 1e-9 * np.abs(lin).max()


@pytest.mark.parametrize("dim", [2, 3])
def test_heat_flux_and_convection_energy_balance(dim):
    m = _heat_mesh(dim)
    om = O.OracleMesh(m)
    N = m.n_nodes
    dt, h, tinf = 0.2, 8.0, 250.0
    t0 = np.full(N, 300.0)
    # convection on the free surface: with T uniform, energy change = -dt h (T - Tinf) |free surface|
    p = O.heat_params(1.0, 1.0, 0.3, h=h, t_inf=tinf, fs_flags=O.HT_QH)
    A, b = O.heat_assemble(om, p, dt, t0, np.zeros(N, np.uint8))
    fs_measure = 0.0
    for f in range(m.facets.shape[1]):
        nd = m.facets[:, f]
        if all(m.flags[nd] & M.FREE_SURFACE):
            X = m.pos[:, nd]
            fs_measure += (np.linalg.norm(X[:, 1] - X[:, 0]) if dim == 2 else
                           0.5 * np.linalg.norm(np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0])))
    assert fs_measure > 0
    assert b.sum() - _mass_total(om, t0) == pytest.approx(-dt * h * (300.0 - tinf) * fs_measure, rel=1e-12)
    # a uniform flux q through the wall facets: energy change = -dt sum_f (q . n) |f|, n outward
    fl = np.where(m.flags & M.BOUND, O.HT_Q, 0).astype(np.uint8)
    q = np.array([0.7, -1.3, 0.4][:dim])
    qgp = np.broadcast_to(q, (m.facets.shape[1], 3, dim)).copy()
    A, b = O.heat_assemble(om, O.heat_params(1.0, 1.0, 0.3), dt, t0, fl, q_gp=qgp)
    flow = 0.0
    cen = m.pos.mean(axis=1)
    for f in range(m.facets.shape[1]):
        nd = m.facets[:, f]
        if not all(fl[nd] & O.HT_Q):
            continue
        X = m.pos[:, nd]
        if dim == 2:
            n = np.array([X[1, 1] - X[1, 0], X[0, 0] - X[0, 1]])
        else:
            n = np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]) / 2
        e = m.facet_elm[f]
        out = [v for v in m.conn[:, e] if v not in nd][0]
        if n @ (m.pos[:, out] - X[:, 0]) > 0:
            n = -n
        flow += q @ n  # |n| is the facet measure
    assert flow != 0
    # the balance is a small difference of two sums of the heat content: round-off of that scale
    e0 = _mass_total(om, t0)
    assert b.sum() - e0 == pytest.approx(-dt * flow, abs=1e-13 * e0)


def test_heat_gauss_positions_helper_matches_oracle():
    from pfem_gb300 import heat as H

    for dim in (2, 3):
        m = _heat_mesh(dim)
        om = O.OracleMesh(m)
        assert np.abs(O.facet_gauss_positions(om) - H.facet_gauss_positions(m.pos, m.facets)).max() < 1e-14


@pytest.mark.parametrize("dim", [2, 3])
def test_boussinesq_uniform_temperature_scales_gravity(dim):
    """A uniform T turns the Boussinesq factors into the constant 1 - alpha (T - Tr): the
    right-hand side equals the plain one with gravity scaled by it."""
    m = _heat_mesh(dim)
    om = O.OracleMesh(m)
    R = (dim + 1) * m.n_nodes
    rng = np.random.default_rng(3)
    q = np.zeros(R)
    q[:dim * m.n_nodes] = 0.01 * rng.standard_normal(dim * m.n_nodes)
    alpha, tr, T = 69e-6, 650.0, 900.0
    fac = 1 - alpha * (T - tr)
    g = (0.0, -9.81, 0.0) if dim == 2 else (0.0, 0.0, -9.81)
    _, b1 = O.pspg_assemble(om, 1000.0, 1e-3, 1e-3, g, q, q, boussinesq=(alpha, tr, np.full(m.n_nodes, T)),
                            apply_bc=False)
    _, b0 = O.pspg_assemble(om, 1000.0, 1e-3, 1e-3, tuple(fac * x for x in g), q, q, apply_bc=False)
    assert np.abs(b1 - b0).max() < 1e-12 * np.abs(b0).max()


def test_uniform_temperature_surface_tension_equals_shifted_gamma():
    """With a uniform T the Boussinesq factor gamma + DgammaDT (T - Tr) is a constant."""
    m = M.square_to_disk_2d(0.05)
    om = O.OracleMesh(m)
    N = m.n_nodes
    q = np.zeros(3 * N)
    gamma, dgdt, T, tr = 1.9, -2e-3, 420.0, 300.0
    _, b1 = O.pspg_assemble(om, 100.0, 1.0, 1e-3, (0.0, 0.0, 0.0), q, q, gamma=gamma,
                            boussinesq=(0.0, tr, np.full(N, T), dgdt), apply_bc=True)
    _, b0 = O.pspg_assemble(om, 100.0, 1.0, 1e-3, (0.0, 0.0, 0.0), q, q, gamma=gamma + dgdt * (T - tr),
                            apply_bc=True)
    assert np.abs(b0).max() > 0
    assert np.abs(b1 - b0).max() < 1e-13 * np.abs(b0).max()


@pytest.mark.parametrize("dim", [2, 3])
def test_heat_phase_change_latent_heat(dim):
    """Phase change (HeatEquation.inl:60-66): below the melting range the latent term is zero
    and the Picard loop reproduces the single pass; inside it the latent heat slows the cooling
    through the free surface (Qh)."""
    m = _heat_mesh(dim)
    om = O.OracleMesh(m)
    N = m.n_nodes
    fl = np.zeros(N, np.uint8)
    tm, dtm, lm = 933.15, 20.0, 396000.0
    kw = dict(h=500.0, t_inf=300.0, fs_flags=O.HT_QH)
    plain = O.heat_params(2385.0, 1080.0, 94.03, **kw)
    latent = O.heat_params(2385.0, 1080.0, 94.03, phase_change=(tm, dtm, lm), **kw)
    # without facet terms (they read the iterate) the rebuilt system equals the first one
    cold = np.full(N, 500.0) + 2 * np.sin(3 * m.pos[0])
    r = {}
    t_pc = O.heat_step(om, O.heat_params(2385.0, 1080.0, 94.03, phase_change=(tm, dtm, lm)), 1.0, cold, fl, result=r)
    assert r["converged"] and r["iterations"] == 2
    assert np.abs(t_pc - O.heat_step(om, O.heat_params(2385.0, 1080.0, 94.03), 1.0, cold, fl)).max() < 1e-12 * 500
    melt = np.full(N, tm + 5.0) + 2 * np.sin(3 * m.pos[0])
    r = {}
    t_pc = O.heat_step(om, latent, 1.0, melt, fl, result=r)
    t_pl = O.heat_step(om, plain, 1.0, melt, fl)
    assert r["converged"] and r["iterations"] >= 3
    assert np.abs(t_pc - melt).max() < 0.1 * np.abs(t_pl - melt).max()


def test_boussinesq_wc_reduces_to_the_wc_step_and_keeps_a_uniform_temperature():
    """BoussinesqWC (WCompNewton/Solver.cpp:278-320) with alpha = 0 moves the flow exactly as the
    Newtonian WC step; with no heat boundary terms a uniform temperature stays uniform (the
    Laplacian rows sum to zero and the lumped mass cancels); a temperature contrast with
    alpha > 0 changes the velocities."""
    m = M.dam_break_2d(0.05)
    N, d = m.n_nodes, 2
    s0 = M.wc_initial_states(m)
    p = O.wc_params()
    fl = np.zeros(N, np.uint8)
    om1, om2, om3 = O.OracleMesh(m), O.OracleMesh(m), O.OracleMesh(m)
    s1 = s0.copy()
    s2 = np.concatenate([s0, np.full(N, 300.0)])
    s3 = np.concatenate([s0, 300.0 + 80.0 * (m.pos[0] < 0.5)])
    b0 = O.wc_bq_params(alpha=0.0, t_ref=300.0, k=0.6, cv=4180.0)
    b1 = O.wc_bq_params(alpha=2e-4, t_ref=300.0, k=1e-9, cv=4180.0)
    for _ in range(5):
        dt = O.wc_next_dt(om1, p, s1)
        assert O.wc_bq_next_dt(om2, p, b0, s2) == dt
        O.wc_step(om1, p, dt, s1)
        O.wc_bq_step(om2, p, b0, dt, s2, fl)
        O.wc_bq_step(om3, p, b1, dt, s3, fl)
    assert np.array_equal(s1, s2[:(2 * d + 2) * N])
    T = s2[(2 * d + 2) * N:]
    assert np.abs(T - 300.0).max() < 1e-10
    assert np.abs(s3[:d * N] - s1[:d * N]).max() > 1e-9


def test_fracstep_keeps_a_hydrostatic_tank_at_rest():
    """Fractional step (MomContEquationFracStep.inl) on water filling an unjittered tank to the
    top of its walls, at rest with the hydrostatic pressure and p = 0 pinned on the free surface:
    the prediction's body force balances D^T p_prev exactly (P1 pressure linear in y), the
    pressure solve returns p_prev and the correction vanishes, so the velocities stay at
    rounding level and the pressure is unchanged."""
    h = 0.05
    pos, flags = M.dam_break_nodes_2d(h, tank=(1.0, 0.6), column=(1.0 - h, 0.6), jitter=0.0)
    m = M.alpha_shape(pos, flags, h, 1.2, delete_flying_nodes=True)
    N, d = m.n_nodes, 2
    q0 = M.incomp_initial_states(m, column=(1.0, 0.6))
    fs = ((m.flags & 2) != 0).astype(np.uint8)
    om = O.OracleMesh(m)
    q = q0.copy()
    for _ in range(2):
        q, res = O.fracstep_picard_step(om, q, 1e-3, gauge=fs)
        assert res.converged
    assert np.abs(q[:d * N]).max() < 1e-12
    assert np.abs(q[d * N:] - q0[d * N:]).max() < 1e-12 * np.abs(q0[d * N:]).max()


def test_fracstep_gauge_is_one_node_per_element_group():
    m = M.dam_break_2d(0.05)
    g = O.fs_gauge(m)
    assert g.sum() == 1 and (m.flags[g.astype(bool)] & 2).all()
    # two separate meshes side by side: one gauge each
    U, off = M.concat_meshes([m, m])
    g2 = O.fs_gauge(U)
    assert g2.sum() == 2 and g2[:off[1]].sum() == 1


def _lumped_mass(mesh, pos):
    """|e| / (d + 1) summed per node: the row sums of the P1 consistent mass."""
    d = mesh.dim
    X = pos[:, mesh.conn]
    J = X[:, 1:, :] - X[:, :1, :]
    vol = np.abs(np.linalg.det(np.moveaxis(J, 2, 0))) / (2.0 if d == 2 else 6.0)
    ml = np.zeros(mesh.n_nodes)
    for k in range(d + 1):
        np.add.at(ml, mesh.conn[k], vol / (d + 1))
    return ml, vol


def test_wc_drhodt_keeps_a_uniform_density_at_rest(wc_small_mesh):
    """CDS_drhodt (ContEquation.inl:232-302) at rest without gravity: D v = 0 and the mass
    terms give rho back, so interior densities stay, free-surface and free nodes take rho*, and
    p follows from Tait-Murnaghan (:305-317)."""
    mesh = wc_small_mesh
    d, N = mesh.dim, mesh.n_nodes
    om = O.OracleMesh(mesh)
    for meduri in (True, False):
        p = O.wc_params(g=(0.0,) * d, meduri=meduri, version=O.WC_DRHODT)
        s = np.zeros((2 * d + 2) * N)
        rho0 = 1000.0 * 1.001
        s[(d + 1) * N:(d + 2) * N] = rho0
        O.wc_step(om, p, 1e-5, s)
        rho, P = s[(d + 1) * N:(d + 2) * N], s[d * N:(d + 1) * N]
        fs = ((mesh.flags & M.FREE_SURFACE) != 0) | mesh.is_free()
        assert np.allclose(rho[~fs], rho0, rtol=1e-14)
        assert np.all(rho[fs] == p.rhoStar) and np.all(P[fs] == 0.0)
        expect = (p.K0 / p.K0p) * ((rho0 / p.rhoStar) ** p.K0p - 1)
        assert np.allclose(P[~fs], expect, rtol=1e-12)


def test_wc_rho_conserves_the_discrete_mass(wc_small_mesh):
    """CDS_rho (m_buildF0 before the move, lumped mass after it, ContEquation.inl:171-230):
    every node off the free surface has ML_new rho_new = (M_old rho_old) with the consistent P1
    mass M_ij = |e| (1 + delta_ij) / ((d + 1)(d + 2)), restated here in numpy."""
    mesh = wc_small_mesh
    d, N = mesh.dim, mesh.n_nodes
    om = O.OracleMesh(mesh)
    p = O.wc_params(version=O.WC_RHO)
    s = M.wc_initial_states(mesh)
    rng = np.random.default_rng(3)
    s[:d * N] = rng.uniform(-0.05, 0.05, d * N) * np.tile(~mesh.is_free(), d)
    rho_old = s[(d + 1) * N:(d + 2) * N].copy()
    x_old = om.positions.copy()
    _, vol = _lumped_mass(mesh, x_old)
    f0 = np.zeros(N)
    c = 1.0 / ((d + 1) * (d + 2))
    for i in range(d + 1):
        for j in range(d + 1):
            np.add.at(f0, mesh.conn[i], vol * c * (2.0 if i == j else 1.0) * rho_old[mesh.conn[j]])
    dt = 1e-4
    O.wc_step(om, p, dt, s)
    ml_new, _ = _lumped_mass(mesh, om.positions)
    rho = s[(d + 1) * N:(d + 2) * N]
    fs = ((mesh.flags & M.FREE_SURFACE) != 0) | mesh.is_free()
    assert not np.array_equal(om.positions, x_old)
    assert np.allclose(ml_new[~fs] * rho[~fs], f0[~fs], rtol=1e-13)
    assert np.all(rho[fs] == p.rhoStar)
    P = s[d * N:(d + 1) * N]
    assert np.allclose(P, (p.K0 / p.K0p) * ((rho / p.rhoStar) ** p.K0p - 1), rtol=1e-12, atol=1e-9)


def test_wc_density_forms_agree_with_dpdt_to_first_order(wc_small_mesh):
    """The three continuity forms discretise the same equation (dp = (K0 + K0' p) / rho drho):
    over three CFL steps from the hydrostatic column they give interior pressures that agree to
    a small fraction of the hydrostatic range.  They differ next to the free surface, where the
    density forms set rho* (p = 0) on the surface nodes and CDS_dpdt solves for them, so the
    bound is on the median and the 90th percentile."""
    mesh = wc_small_mesh
    d, N = mesh.dim, mesh.n_nodes
    om0 = O.OracleMesh(mesh)
    s0 = M.wc_initial_states(mesh)
    dt = O.wc_next_dt(om0, O.wc_params(), s0)
    out = {}
    for ver in (O.WC_DPDT, O.WC_RHO, O.WC_DRHODT):
        om = O.OracleMesh(mesh)
        s = s0.copy()
        for _ in range(3):
            O.wc_step(om, O.wc_params(version=ver), dt, s)
        out[ver] = s[d * N:(d + 1) * N]
    inner = ~mesh.is_free() & ((mesh.flags & M.FREE_SURFACE) == 0)
    scale = s0[d * N:(d + 1) * N].max()
    for ver in (O.WC_RHO, O.WC_DRHODT):
        e = np.abs(out[ver] - out[O.WC_DPDT])[inner]
        assert np.median(e) < 1e-5 * scale and np.quantile(e, 0.9) < 1e-3 * scale, (ver, np.quantile(e, [0.5, 0.9]))
