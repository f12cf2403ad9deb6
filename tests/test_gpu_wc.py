"""GPU parity of the weakly compressible explicit step against the FP64 oracle.

FP64 plain form: every state field within 1e-11 relative (same operations, different
rounding order inside an element), dt from the device CFL reduction within 1e-13.
FP32 mixed form: within 2e-4 relative after 20 steps (FP32 state rounding), mass (FP64 sum)
within 1e-6.  Full C2 size (h = 0.005, 82k nodes): size-independent properties only.
"""
import numpy as np
import pytest

from oracle import oracle as O
from pfem_gb300 import api
from pfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def make_ctx(mesh, precision=api.PREC_FP64):
    p = api.default_params(api.KIND_WC_CDS_DPDT, mesh.dim)
    p.precision = precision
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    return ctx


def field_errs(s, so, d, N):
    errs = []
    for f in range(2 * d + 2):
        sl = slice(f * N, (f + 1) * N)
        errs.append(np.linalg.norm(s[sl] - so[sl]) / max(np.linalg.norm(so[sl]), 1e-30))
    return errs


def run_pair(mesh, nsteps, precision):
    d, N = mesh.dim, mesh.n_nodes
    s0 = M.wc_initial_states(mesh)
    ctx = make_ctx(mesh, precision)
    ctx.set_states(s0)
    om = O.OracleMesh(mesh)
    p = O.wc_params()
    so = s0.copy()
    dt_o = O.wc_next_dt(om, p, so)
    dt_g = ctx.next_dt()
    ctx.set_time(0.0, dt_g)
    for _ in range(nsteps):
        O.wc_step(om, p, dt_o, so)
        dt_o = O.wc_next_dt(om, p, so)
    st = ctx.wc_step(0.0, nsteps)
    return ctx, om, so, dt_o, dt_g, st


def test_wc_fp64_matches_oracle(gpu_lib, wc_small_mesh):
    mesh = wc_small_mesh
    d, N = mesh.dim, mesh.n_nodes
    om0 = O.OracleMesh(mesh)
    s0 = M.wc_initial_states(mesh)
    p = O.wc_params()
    ctx, om, so, dt_o, dt_g0, st = run_pair(mesh, 20, api.PREC_FP64)
    assert dt_g0 == pytest.approx(O.wc_next_dt(om0, p, s0), rel=1e-13)
    assert st.dt == pytest.approx(dt_o, rel=1e-11)
    s = ctx.get_states()
    errs = field_errs(s, so, d, N)
    # acceleration and velocity start at zero; compare them absolutely against their scale
    assert max(errs) < 1e-10, errs
    assert np.abs(ctx.get_positions() - om.positions).max() < 1e-13
    assert ctx.mass() == pytest.approx(O.wc_mass(om, so), rel=1e-13)


def test_wc_fixed_dt(gpu_lib, wc_small_mesh):
    mesh = wc_small_mesh
    d, N = mesh.dim, mesh.n_nodes
    s0 = M.wc_initial_states(mesh)
    ctx = make_ctx(mesh)
    ctx.set_states(s0)
    om = O.OracleMesh(mesh)
    p = O.wc_params()
    so = s0.copy()
    for _ in range(5):
        O.wc_step(om, p, 1e-5, so)
    st = ctx.wc_step(1e-5, 5)
    assert st.time == pytest.approx(5e-5, rel=1e-12)
    assert max(field_errs(ctx.get_states(), so, d, N)) < 1e-10


def test_wc_fp32_mixed_error(gpu_lib, wc_small_mesh):
    """Mixed form (FP32 element arithmetic, FP64 state): velocity, pressure, density and
    positions within 1e-6 of the FP64 oracle after 20 adaptive steps."""
    mesh = wc_small_mesh
    d, N = mesh.dim, mesh.n_nodes
    ctx, om, so, dt_o, _, st = run_pair(mesh, 20, api.PREC_MIXED)
    s = ctx.get_states()
    errs = field_errs(s, so, d, N)
    assert max(errs[:d + 2]) < 1e-6, errs       # v, p, rho
    assert max(errs[d + 2:]) < 1e-3, errs       # accelerations (a = F/M of nearly balanced forces)
    assert np.abs(ctx.get_positions() - om.positions).max() < 1e-10
    assert ctx.mass() == pytest.approx(O.wc_mass(om, so), rel=1e-9)


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_wc_graph_matches_direct_launches(gpu_lib, wc_small_mesh, precision):
    """Steps replayed from the captured CUDA graph and steps launched kernel by kernel (the
    profiling path) run the same kernels: results are bitwise equal."""
    mesh = wc_small_mesh
    s0 = M.wc_initial_states(mesh)
    out = []
    for prof in (False, True):
        ctx = make_ctx(mesh, precision)
        ctx.set_states(s0)
        ctx.set_time(0.0, ctx.next_dt())
        ctx.set_profiling(prof)
        st = ctx.wc_step(0.0, 30)
        ctx.set_profiling(False)
        out.append((ctx.get_states(), ctx.get_positions(), st.dt, st.time))
        ctx.close()
    (sa, xa, dta, ta), (sb, xb, dtb, tb) = out
    assert np.array_equal(sa, sb) and np.array_equal(xa, xb)
    assert dta == dtb and ta == tb


def test_wc_one_call_equals_step_by_step(gpu_lib, wc_small_mesh):
    """nsteps in one call == nsteps calls of one step (device-side dt and time carry over)."""
    mesh = wc_small_mesh
    s0 = M.wc_initial_states(mesh)
    res = []
    for chunk in (7, 1):
        ctx = make_ctx(mesh, api.PREC_MIXED)
        ctx.set_states(s0)
        ctx.set_time(0.0, ctx.next_dt())
        for _ in range(7 // chunk):
            ctx.wc_step(0.0, chunk)
        res.append(ctx.get_states())
        ctx.close()
    assert np.array_equal(res[0], res[1])


def test_wc_full_size_properties(gpu_lib):
    """C2 size: mass conservation, finite states, positive CFL step, fluid stays in the tank."""
    mesh = M.dam_break_2d(0.005)
    s0 = M.wc_initial_states(mesh)
    for prec in (api.PREC_FP64, api.PREC_MIXED):
        ctx = make_ctx(mesh, prec)
        ctx.set_states(s0)
        m0 = ctx.mass()
        ctx.set_time(0.0, ctx.next_dt())
        st = ctx.wc_step(0.0, 200)
        s = ctx.get_states()
        assert np.all(np.isfinite(s))
        assert 0 < st.dt <= 1e-3
        assert abs(ctx.mass() - m0) / m0 < 1e-4
        x = ctx.get_positions()
        assert x[0].min() >= -1e-9 and x[1].min() >= -1e-9


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_wc_3d_matches_oracle(gpu_lib, small3d_mesh, precision):
    """3D (tetrahedra): 20 adaptive steps of both forms against the FP64 oracle.  FP64 as in 2D;
    mixed: velocity, pressure and density within 1e-6 relative.  (With the element size taken
    from an FP32 determinant of the Jacobian, which cancels in 3D, the mixed velocity was 1.8e-6
    off, uniformly over free-surface and interior nodes from the first steps on: the lumped mass
    carried the determinant's rounding.  The size now comes from the double-float adjugate.)"""
    mesh = small3d_mesh
    d, N = mesh.dim, mesh.n_nodes
    column = (0.2, 0.3, 0.3)
    s0 = M.wc_initial_states(mesh, column=column)
    ctx = make_ctx(mesh, precision)
    ctx.set_states(s0)
    om = O.OracleMesh(mesh)
    p = O.wc_params(g=(0.0, 0.0, -9.81))
    so = s0.copy()
    dt_o = O.wc_next_dt(om, p, so)
    ctx.set_time(0.0, ctx.next_dt())
    for _ in range(20):
        O.wc_step(om, p, dt_o, so)
        dt_o = O.wc_next_dt(om, p, so)
    st = ctx.wc_step(0.0, 20)
    errs = field_errs(ctx.get_states(), so, d, N)
    if precision == api.PREC_FP64:
        assert st.dt == pytest.approx(dt_o, rel=1e-11)
        assert max(errs) < 1e-10, errs
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-13
    else:
        assert max(errs[:d + 2]) < 1e-6, errs
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-10
    assert ctx.mass() == pytest.approx(O.wc_mass(om, so), rel=1e-9)


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_wc_c2_full_size_matches_oracle(gpu_lib, precision):
    """The full C2 mesh (h = 0.005, 82k nodes, 160k triangles): 200 adaptive steps of each form
    against 200 steps of the FP64 oracle.  FP64: every field within 1e-10.  Mixed (FP32
    arithmetic on double-float state): velocity, pressure and density within 1e-6, positions
    within 1e-10 absolute, mass within 1e-9 (its CFL step is computed in FP32, so its time
    differs from the oracle's by ~1e-7 relative)."""
    mesh = M.dam_break_2d(0.005)
    d, N = mesh.dim, mesh.n_nodes
    ctx, om, so, dt_o, _, st = run_pair(mesh, 200, precision)
    errs = field_errs(ctx.get_states(), so, d, N)
    if precision == api.PREC_FP64:
        assert max(errs) < 1e-10, errs
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-13
        assert st.dt == pytest.approx(dt_o, rel=1e-11)
    else:
        assert max(errs[:d + 2]) < 1e-6, errs
        assert np.abs(ctx.get_positions() - om.positions).max() < 1e-10
    assert ctx.mass() == pytest.approx(O.wc_mass(om, so), rel=1e-9)
