"""GPU parity of the incompressible PSPG path against the FP64 oracle, through the C ABI.

Tolerances: integer outputs (CSR pattern, flags) bit-exact; FP64 element geometry 1e-13
relative; assembled values and RHS 1e-12 relative to the largest entry of their row (the
element contributions are summed in the same order as the reference's setFromTriplets, only
the element arithmetic is ordered differently); a full Picard step 1e-8 relative per field
(the linear solve is Krylov here, a sparse LU in the reference).
"""
import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import api
from pfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def make_ctx(mesh, **kw):
    p = api.default_params(api.KIND_INCOMP_PSPG, mesh.dim)
    for k, v in kw.items():
        setattr(p, k, v)
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    return ctx


def oracle_csr(A):
    csr = A.tocsr()
    csr.sort_indices()
    return csr


def gravity(d):
    return (0.0, -9.81) if d == 2 else (0.0, 0.0, -9.81)


def rel_rowwise(gpu_vals, ora_vals, rp):
    worst = 0.0
    for r in range(len(rp) - 1):
        a, b = gpu_vals[rp[r]:rp[r + 1]], ora_vals[rp[r]:rp[r + 1]]
        scale = max(np.abs(b).max(), 1e-300)
        worst = max(worst, np.abs(a - b).max() / scale)
    return worst


@pytest.fixture(params=["c1", "3d"])
def mesh(request, c1_mesh, small3d_mesh):
    return c1_mesh if request.param == "c1" else small3d_mesh


def test_flags_and_geometry(gpu_lib, mesh):
    ctx = make_ctx(mesh)
    flags = ctx.get_flags()
    free = (flags & api.NODE_FREE) != 0
    assert np.array_equal(free, mesh.is_free())
    assert np.array_equal(flags & 0x0F, mesh.flags & 0x0F)
    det, inv = ctx.get_geometry()
    om = O.OracleMesh(mesh)
    _, det_o, inv_o = om.geometry()
    assert np.allclose(det, det_o, rtol=1e-13, atol=0)
    d = mesh.dim
    scale = np.abs(inv_o).max(axis=(1, 2), keepdims=True)
    assert (np.abs(inv[:, :d, :d] - inv_o[:, :d, :d]) / scale).max() < 1e-13


@pytest.mark.parametrize("apply_bc", [False, True])
def test_assembly_pattern_bitexact_and_values(gpu_lib, mesh, apply_bc):
    d, N = mesh.dim, mesh.n_nodes
    rng = np.random.default_rng(3)
    q_iter = rng.uniform(-0.5, 0.5, (d + 1) * N)
    q_prev = rng.uniform(-0.5, 0.5, (d + 1) * N)
    q_prev[d * N:] *= 1e4
    ctx = make_ctx(mesh)
    dt = 1e-3
    ctx.pspg_assemble(dt, q_iter, q_prev, apply_bc=apply_bc)
    rp, ci, va, b = ctx.get_csr()
    om = O.OracleMesh(mesh)
    A, b_o = O.pspg_assemble(om, 1000.0, 1e-3, dt, gravity(d), q_iter, q_prev, apply_bc=apply_bc)
    csr = oracle_csr(A)
    assert np.array_equal(rp, csr.indptr.astype(np.int64))
    assert np.array_equal(ci, csr.indices)
    assert rel_rowwise(va, csr.data, rp) < 1e-12
    bscale = np.maximum(np.abs(b_o), np.abs(csr).max(axis=1).toarray().ravel() * 1e-3)
    assert (np.abs(b - b_o) / np.maximum(bscale, 1e-300)).max() < 1e-12


def test_dirichlet_column_elimination(gpu_lib, c1_mesh):
    mesh = c1_mesh
    d, N = mesh.dim, mesh.n_nodes
    dir_nodes = np.nonzero((mesh.flags & M.DIRICHLET) != 0)[0].astype(np.int32)
    rng = np.random.default_rng(5)
    vals = rng.uniform(-1, 1, (d, dir_nodes.size))
    vbc = np.zeros((d, N))
    vbc[:, dir_nodes] = vals
    q = rng.uniform(-0.1, 0.1, (d + 1) * N)
    ctx = make_ctx(mesh)
    ctx.set_dirichlet(dir_nodes, vals.reshape(-1))
    ctx.pspg_assemble(1e-3, q, q, apply_bc=True)
    rp, ci, va, b = ctx.get_csr()
    om = O.OracleMesh(mesh)
    A, b_o = O.pspg_assemble(om, 1000.0, 1e-3, 1e-3, gravity(d), q, q, vbc=vbc.reshape(-1))
    csr = oracle_csr(A)
    assert np.array_equal(ci, csr.indices)
    # eliminated columns: every off-diagonal entry of a Dirichlet velocity column is exactly 0
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    dcols = np.zeros((d + 1) * N, bool)
    for f in range(d):
        dcols[dir_nodes + f * N] = True
    elim = dcols[ci] & (ci != rows)
    assert elim.sum() > 0
    assert np.all(va[elim] == 0.0) and np.all(csr.data[elim] == 0.0)
    assert rel_rowwise(va, csr.data, rp) < 1e-12
    assert np.abs(b - b_o).max() <= 1e-12 * np.abs(b_o).max()


def test_linear_solve_matches_direct(gpu_lib, c1_mesh):
    from scipy.sparse.linalg import splu

    mesh = c1_mesh
    q0 = M.incomp_initial_states(mesh)
    ctx = make_ctx(mesh)
    ctx.set_states(q0)
    ctx.pspg_assemble(1e-3, None, None, apply_bc=True)
    x, it, res = ctx.linear_solve(q0)
    om = O.OracleMesh(mesh)
    A, b = O.pspg_assemble(om, 1000.0, 1e-3, 1e-3, (0.0, -9.81), q0, q0)
    xd = splu(A.tocsc(), permc_spec="COLAMD").solve(b)
    N = mesh.n_nodes
    for f in range(3):
        sl = slice(f * N, (f + 1) * N)
        assert np.linalg.norm(x[sl] - xd[sl]) <= 1e-9 * max(np.linalg.norm(xd[sl]), 1e-12), (f, it, res)
    assert np.linalg.norm(A @ x - b) < 1e-7


def _fields_rel_err(q, qo, d, N):
    out = []
    for f in range(d + 1):
        sl = slice(f * N, (f + 1) * N)
        out.append(np.linalg.norm(q[sl] - qo[sl]) / max(np.linalg.norm(qo[sl]), 1e-30))
    return out


@pytest.mark.parametrize("which", ["c1", "3d"])
def test_picard_steps_match_oracle(gpu_lib, which, c1_mesh, small3d_mesh):
    mesh = c1_mesh if which == "c1" else small3d_mesh
    d, N = mesh.dim, mesh.n_nodes
    column = (1.0, 2.0) if d == 2 else (0.2, 0.3, 0.3)
    q0 = M.incomp_initial_states(mesh, column=column)
    ctx = make_ctx(mesh)
    ctx.set_states(q0)
    om = O.OracleMesh(mesh)
    qo = q0.copy()
    for step in range(3):
        st = ctx.picard_step(1e-3)
        qo, res = O.pspg_picard_step(om, qo, 1e-3, g=gravity(d))
        assert st.converged == 1 and res.converged
        assert st.picard_iterations == res.iterations
        q = ctx.get_states()
        errs = _fields_rel_err(q, qo, d, N)
        assert max(errs) < 1e-8, (step, errs)
        x = ctx.get_positions()
        assert np.abs(x - om.positions).max() < 1e-12
    assert ctx.volume() == pytest.approx(om.volume(), rel=1e-13)
    assert ctx.tip(0, True) == pytest.approx(om.tip(0, True), rel=1e-12)


def test_picard_failure_restores_state(gpu_lib, c1_mesh):
    mesh = c1_mesh
    q0 = M.incomp_initial_states(mesh)
    ctx = make_ctx(mesh, picard_max_iter=0, picard_min_res=1e-30)
    ctx.set_states(q0)
    x0 = ctx.get_positions()
    st = ctx.picard_step(1e-3)
    assert st.converged == 0
    assert np.array_equal(ctx.get_positions(), x0)
    assert np.array_equal(ctx.get_states(), q0)


def test_invalid_mesh_rejected(gpu_lib, c1_mesh):
    bad = c1_mesh.copy()
    bad.conn = bad.conn.copy()
    bad.conn[0, 5] = bad.n_nodes + 3
    p = api.default_params(api.KIND_INCOMP_PSPG, 2)
    ctx = api.Context(p)
    with pytest.raises(api.PfgError, match="INVALID"):
        ctx.upload_mesh(bad)
    with pytest.raises(api.PfgError, match="STATE"):
        ctx.picard_step(1e-3)
