"""GPU parity of the weakly compressible solver's density forms, CDS_rho and CDS_drhodt
(ContEquation.inl:171-302, selected by the SolverWCompNewton id, WCompNewton/Solver.cpp:22-23),
against the FP64 oracle: 20 adaptive steps of the plain FP64 form, every state field within
1e-10 relative, positions within 1e-13, dt within 1e-11; both stabilisations; 2D and 3D."""
import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import api
from pfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def field_errs(s, so, d, N):
    return [np.linalg.norm(s[f * N:(f + 1) * N] - so[f * N:(f + 1) * N]) /
            max(np.linalg.norm(so[f * N:(f + 1) * N]), 1e-30) for f in range(2 * d + 2)]


def run(mesh, version, meduri, column=None, nsteps=20):
    d, N = mesh.dim, mesh.n_nodes
    g = (0.0, -9.81) if d == 2 else (0.0, 0.0, -9.81)
    p = api.default_params(api.KIND_WC_CDS_DPDT, d)
    p.wc_version = version
    p.meduri = int(meduri)
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    s0 = M.wc_initial_states(mesh, column=column) if column else M.wc_initial_states(mesh)
    ctx.set_states(s0)
    om = O.OracleMesh(mesh)
    po = O.wc_params(g=g, meduri=meduri, version=version)
    so = s0.copy()
    dt_o = O.wc_next_dt(om, po, so)
    ctx.set_time(0.0, ctx.next_dt())
    for _ in range(nsteps):
        O.wc_step(om, po, dt_o, so)
        dt_o = O.wc_next_dt(om, po, so)
    st = ctx.wc_step(0.0, nsteps)
    return ctx, om, so, dt_o, st


@pytest.mark.parametrize("version", [api.WC_RHO, api.WC_DRHODT])
@pytest.mark.parametrize("meduri", [True, False])
def test_density_forms_match_oracle_2d(gpu_lib, wc_small_mesh, version, meduri):
    mesh = wc_small_mesh
    d, N = mesh.dim, mesh.n_nodes
    ctx, om, so, dt_o, st = run(mesh, version, meduri)
    assert st.converged and st.steps_done == 20
    assert st.dt == pytest.approx(dt_o, rel=1e-11)
    errs = field_errs(ctx.get_states(), so, d, N)
    assert max(errs) < 1e-10, errs
    assert np.abs(ctx.get_positions() - om.positions).max() < 1e-13
    s = ctx.get_states()
    fs = ((ctx.get_flags() & api.NODE_FREE_SURFACE) != 0) | ((ctx.get_flags() & api.NODE_FREE) != 0)
    assert np.all(s[(d + 1) * N:(d + 2) * N][fs] == 1000.0)


@pytest.mark.parametrize("version", [api.WC_RHO, api.WC_DRHODT])
def test_density_forms_match_oracle_3d(gpu_lib, small3d_mesh, version):
    mesh = small3d_mesh
    d, N = mesh.dim, mesh.n_nodes
    ctx, om, so, dt_o, st = run(mesh, version, True, column=(0.2, 0.3, 0.3))
    assert st.dt == pytest.approx(dt_o, rel=1e-11)
    errs = field_errs(ctx.get_states(), so, d, N)
    assert max(errs) < 1e-10, errs
    assert np.abs(ctx.get_positions() - om.positions).max() < 1e-13


def test_density_forms_reject_the_mixed_form(gpu_lib):
    p = api.default_params(api.KIND_WC_CDS_DPDT, 2)
    p.wc_version = api.WC_RHO
    p.precision = api.PREC_MIXED
    with pytest.raises(api.PfgError):
        api.Context(p)
    p.precision = api.PREC_FP64
    p.wc_version = 3
    with pytest.raises(api.PfgError):
        api.Context(p)
