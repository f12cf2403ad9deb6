"""GPU test of pfg_wc_next_dt_noalloc, the CFL time step that allocates no device memory.

Callers that may not call cudaMalloc at the point where they need a time step (an application
whose pool allocator owns the GPU memory, a loop under someone else's stream capture, a plugin
that only gets device pointers) call this entry point with their own device arrays.  Its result
must equal the context-based pfg_next_dt on the same state, on consecutive calls that share the
library's static scratch array.  This file is collected last so that a run stopping at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_arrays(torch, ctx, mesh):
    conn = torch.from_numpy(np.ascontiguousarray(mesh.conn, np.int32)).cuda()
    pos = torch.from_numpy(np.ascontiguousarray(ctx.get_positions(), np.float64)).cuda()
    st = torch.from_numpy(np.ascontiguousarray(ctx.get_states(), np.float64)).cuda()
    return conn, pos, st


def _noalloc_dt(lib, params, mesh, conn, pos, st, out):
    rc = lib.pfg_wc_next_dt_noalloc(ctypes.byref(params), mesh.n_nodes, mesh.n_elems, conn.data_ptr(),
                                    pos.data_ptr(), st.data_ptr(), out.data_ptr(), None)
    return rc


@pytest.mark.parametrize("dim", [2, 3])
def test_noalloc_dt_matches_context_dt_on_consecutive_calls(gpu_lib, dim):
    torch = pytest.importorskip("torch")
    from pfem_gb300 import api
    from pfem_gb300 import mesh as M

    if dim == 2:
        mesh, column = M.dam_break_2d(0.02), (1.0, 2.0)
    else:
        mesh, column = M.dam_break_3d(0.05, tank=(0.6, 0.3, 0.5), column=(0.2, 0.3, 0.3)), (0.2, 0.3, 0.3)
    p = api.default_params(api.KIND_WC_CDS_DPDT, dim)
    ctx = api.Context(p)
    ctx.upload_mesh(mesh)
    s0 = M.wc_initial_states(mesh, column=column)
    rng = np.random.default_rng(11)
    # velocities matter in the CFL bound
    s0[:dim * mesh.n_nodes] = rng.uniform(-0.5, 0.5, dim * mesh.n_nodes)
    ctx.set_states(s0)
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")

    # first call
    dt_ref = ctx.next_dt()
    conn, pos, st = _device_arrays(torch, ctx, mesh)
    assert _noalloc_dt(gpu_lib, p, mesh, conn, pos, st, out) == 0
    torch.cuda.synchronize()
    assert float(out.item()) == pytest.approx(dt_ref, rel=1e-13)

    # second call on a different state: the shared scratch must not carry anything over
    ctx.set_time(0.0, dt_ref)
    ctx.wc_step(0.0, 25)
    dt_ref2 = ctx.next_dt()
    conn2, pos2, st2 = _device_arrays(torch, ctx, mesh)
    out.fill_(-1.0)
    assert _noalloc_dt(gpu_lib, p, mesh, conn2, pos2, st2, out) == 0
    torch.cuda.synchronize()
    assert float(out.item()) == pytest.approx(dt_ref2, rel=1e-13)
    assert dt_ref2 != dt_ref

    # sizes beyond the static scratch are refused before any device access
    big = 1 << 20
    assert gpu_lib.pfg_wc_next_dt_noalloc(ctypes.byref(p), big + 1, 10, conn.data_ptr(), pos.data_ptr(),
                                          st.data_ptr(), out.data_ptr(), None) == -1
    ctx.close()
