"""Batched weakly compressible steps (mixed precision): several independent meshes in one
context, stepped by one launch sequence with a time step of their own, against each mesh
stepped alone in its own context, through the C ABI.  Every instance's states, positions, dt
and time are bitwise those of its solo run: the kernels evaluate each node and element with
the same operations, and the per-instance CFL minimum (atomic min of the FP32 bit patterns)
is exact in any order, as is the single mesh's block reduction."""
import numpy as np
import pytest

from pfem_gb300 import api
from pfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu

SPECS = [(0.04, (1.0, 2.0), 1e-3), (0.05, (0.8, 1.5), 1e-2), (0.03, (1.2, 1.0), 5e-2)]


def _meshes():
    meshes, states, mus = [], [], []
    for i, (h, col, mu) in enumerate(SPECS):
        m = M.dam_break_2d(h, column=col, seed=20261203 + i)
        meshes.append(m)
        states.append(M.wc_initial_states(m, column=col))
        mus.append(mu)
    return meshes, states, mus


def _ctx(mesh, mu):
    p = api.default_params(api.KIND_WC_CDS_DPDT, mesh.dim)
    p.precision = api.PREC_MIXED
    p.mu = mu
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    return ctx


@pytest.mark.parametrize("fixed_dt", [0.0, 2e-5])
def test_wc_batch_equals_instances_alone(gpu_lib, fixed_dt):
    meshes, states, mus = _meshes()
    U, off = M.concat_meshes(meshes)
    ctx = _ctx(U, mus[0])
    ctx.set_instances(off, 1000.0, mus)
    ctx.set_states(M.concat_states(states, meshes))
    ctx.next_dt()  # each instance's CFL step of its initial state
    ctx.wc_step_batch(fixed_dt, 25)
    sts = ctx.wc_step_batch(fixed_dt, 15)
    sb = M.split_states(ctx.get_states(), meshes)
    xb = ctx.get_positions()
    for i, m in enumerate(meshes):
        solo = _ctx(m, mus[i])
        solo.set_states(states[i])
        solo.next_dt()
        solo.wc_step(fixed_dt, 25)
        st = solo.wc_step(fixed_dt, 15)
        assert st.dt == sts[i].dt and st.time == sts[i].time
        assert np.array_equal(solo.get_states(), sb[i])
        assert np.array_equal(solo.get_positions(), xb[:, off[i]:off[i + 1]])
        solo.close()
    if fixed_dt == 0.0:
        assert len({s.dt for s in sts}) == len(sts)  # the instances' own CFL steps differ


def test_wc_batch_rejects_mixed_rho_and_plain_form(gpu_lib):
    meshes, states, mus = _meshes()
    U, off = M.concat_meshes(meshes)
    ctx = _ctx(U, 1e-3)
    with pytest.raises(api.PfgError, match="UNSUPPORTED"):
        ctx.set_instances(off, [1000.0, 900.0, 1000.0], mus)
    p = api.default_params(api.KIND_WC_CDS_DPDT, 2)
    plain = api.Context(p)
    plain.upload_mesh(U)
    with pytest.raises(api.PfgError, match="STATE"):
        plain.set_instances(off, 1000.0, mus)
