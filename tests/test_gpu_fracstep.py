"""GPU parity of the fractional-step solver (solver "FracStep", MomContEquationFracStep.inl:
7-630) against the FP64 oracle, through the C ABI.

Both sides pin the same pressure gauge (the smallest free-surface node of each connected group
of elements, or every free-surface node with fs_pressure_dirichlet; the reference's pressure
system is singular without it).  The device solves its three SPD systems by Jacobi CG to
relative residual 1e-14, the oracle by SuperLU: Picard iteration counts equal, every field
within 1e-9 relative, positions within 1e-12.
"""
import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import api
from pfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def make_ctx(mesh, fs_dir=False, residual=api.RES_U, **kw):
    p = api.default_params(api.KIND_INCOMP_PSPG, mesh.dim)
    p.precision = api.PREC_FP64
    p.frac_step, p.gamma_fs, p.fs_pressure_dirichlet = 1, 1.0, int(fs_dir)
    p.residual = residual
    p.krylov_rel_tol, p.krylov_abs_tol, p.krylov_max_iter = 1e-14, 0.0, 20000
    for k, v in kw.items():
        setattr(p, k, v)
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    return ctx


def gravity(d):
    return (0.0, -9.81) if d == 2 else (0.0, 0.0, -9.81)


@pytest.mark.parametrize("case", [("c1", False, 1e-4, "U"), ("c1", True, 1e-3, "U_P"), ("3d", True, 1e-3, "U"),
                                  ("3d", False, 1e-4, "U_P")])
def test_fracstep_matches_oracle(gpu_lib, case, c1_mesh, small3d_mesh):
    which, fs_dir, dt, res_kind = case
    mesh = c1_mesh if which == "c1" else small3d_mesh
    d, N = mesh.dim, mesh.n_nodes
    column = (1.0, 2.0) if d == 2 else (0.2, 0.3, 0.3)
    q0 = M.incomp_initial_states(mesh, column=column)
    ctx = make_ctx(mesh, fs_dir, api.RES_U if res_kind == "U" else api.RES_U_P)
    ctx.set_states(q0)
    om = O.OracleMesh(mesh)
    gauge = ((mesh.flags & 2) != 0).astype(np.uint8) if fs_dir else O.fs_gauge(mesh)
    qo = q0.copy()
    for step in range(2):
        st = ctx.picard_step(dt)
        qo, res = O.fracstep_picard_step(om, qo, dt, g=gravity(d), gauge=gauge, residual=res_kind, mesh=mesh)
        # with the single gauge the reference's Picard loop stops converging after one step at
        # these time steps: both sides then report the failure and restore the step's start
        # (the oracle after maxIter + 1 iterations, the device possibly sooner, when a CG
        # solve of the diverging iterate breaks down)
        assert st.converged == int(res.converged), (step, res.residuals, st.residual)
        if res.converged:
            assert st.picard_iterations == res.iterations
        if step == 0 or fs_dir:
            assert res.converged
        q = ctx.get_states()
        errs = [np.linalg.norm(q[f * N:(f + 1) * N] - qo[f * N:(f + 1) * N]) /
                max(np.linalg.norm(qo[f * N:(f + 1) * N]), 1e-30) for f in range(d + 1)]
        assert max(errs) < 1e-9, (step, errs)
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-12


def test_fracstep_configuration_checked(gpu_lib):
    p = api.default_params(api.KIND_INCOMP_PSPG, 2)
    p.frac_step, p.gamma_fs = 1, 1.0
    p.residual = api.RES_AX_F  # unsupported by the reference's fractional step
    with pytest.raises(api.PfgError):
        api.Context(p)
    p.residual = api.RES_U
    p.precision = api.PREC_MIXED
    with pytest.raises(api.PfgError):
        api.Context(p)
    p.precision = api.PREC_FP64
    p.gamma_fs = 1.5
    with pytest.raises(api.PfgError):
        api.Context(p)
