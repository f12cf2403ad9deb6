"""The plain form with the device sparse LU (PFG_LINSOLVE_LU: nested-dissection ordering,
multifrontal factorisation, FP64 refinement), the reference's own solver choice, through the C
ABI: Picard steps against the FP64 oracle (SuperLU with COLAMD, like Eigen's SparseLU) within
1e-10 per field with equal Picard iteration counts, 2D and 3D, and against the plain form with
BiCGSTAB solved to the same accuracy."""
import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import api
from pfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def lu_ctx(mesh, **kw):
    p = api.default_params(api.KIND_INCOMP_PSPG, mesh.dim)
    p.precision = api.PREC_FP64
    p.linear_solver = api.LINSOLVE_LU
    for k, v in kw.items():
        setattr(p, k, v)
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    return ctx


def field_errs(q, qo, d, N):
    return [np.linalg.norm(q[f * N:(f + 1) * N] - qo[f * N:(f + 1) * N]) /
            max(np.linalg.norm(qo[f * N:(f + 1) * N]), 1e-30) for f in range(d + 1)]


@pytest.mark.parametrize("which", ["c1", "3d"])
def test_lu_picard_matches_oracle(gpu_lib, which, c1_mesh, small3d_mesh):
    mesh = c1_mesh if which == "c1" else small3d_mesh
    d, N = mesh.dim, mesh.n_nodes
    column = (1.0, 2.0) if d == 2 else (0.2, 0.3, 0.3)
    g = (0.0, -9.81) if d == 2 else (0.0, 0.0, -9.81)
    q0 = M.incomp_initial_states(mesh, column=column)
    ctx = lu_ctx(mesh)
    ctx.set_states(q0)
    om = O.OracleMesh(mesh)
    qo = q0.copy()
    for step in range(3):
        st = ctx.picard_step(1e-3)
        qo, res = O.pspg_picard_step(om, qo, 1e-3, g=g)
        assert st.converged == 1 and res.converged
        assert st.picard_iterations == res.iterations
        errs = field_errs(ctx.get_states(), qo, d, N)
        assert max(errs) < 1e-10, (step, errs)
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-13


def test_lu_matches_bicgstab_on_a_larger_2d_mesh(gpu_lib):
    """A 2D instance with large fronts (the blocked factorisation path): one step of the LU plain
    form against the BiCGSTAB plain form solved to 1e-14."""
    from pfem_gb300 import workloads as W

    inst = W.c4_instance(0)
    m = inst.mesh
    out = {}
    for solver in (api.LINSOLVE_LU, api.LINSOLVE_BICGSTAB):
        p = api.default_params(api.KIND_INCOMP_PSPG, 2)
        p.precision = api.PREC_FP64
        p.mu = inst.mu
        p.linear_solver = solver
        p.krylov_rel_tol, p.krylov_abs_tol, p.krylov_max_iter = 1e-14, 0.0, 50000
        ctx = api.Context(p)
        ctx.upload_mesh(m)
        ctx.set_states(inst.q0)
        st = ctx.picard_step(1e-3)
        assert st.converged == 1
        out[solver] = (st.picard_iterations, ctx.get_states())
        ctx.close()
    assert out[api.LINSOLVE_LU][0] == out[api.LINSOLVE_BICGSTAB][0]
    assert max(field_errs(out[api.LINSOLVE_LU][1], out[api.LINSOLVE_BICGSTAB][1], 2, m.n_nodes)) < 1e-9


def test_lu_rejected_for_the_mixed_form(gpu_lib, c1_mesh):
    p = api.default_params(api.KIND_INCOMP_PSPG, 2)
    p.precision = api.PREC_MIXED
    p.linear_solver = api.LINSOLVE_LU
    with pytest.raises(api.PfgError):
        api.Context(p)
