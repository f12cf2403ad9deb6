"""Serving (pfem_gb300/serve.py): memory estimate, admission under the HBM budget, and every
request's result bitwise the same alone and in the mix (contexts share no device data and all
reductions are deterministic)."""
import numpy as np
import pytest

from pfem_gb300 import api
from pfem_gb300 import mesh as M
from pfem_gb300 import serve as SV

pytestmark = pytest.mark.gpu


def _requests():
    out = []
    specs = [(api.KIND_WC_CDS_DPDT, 0.05, (1.0, 2.0), 40), (api.KIND_INCOMP_PSPG, 0.1, (1.0, 2.0), 3),
             (api.KIND_WC_CDS_DPDT, 0.04, (0.8, 1.5), 60), (api.KIND_INCOMP_PSPG, 0.08, (1.2, 1.6), 2),
             (api.KIND_INCOMP_PSPG, 0.12, (0.9, 1.9), 3)]
    for i, (kind, h, col, steps) in enumerate(specs):
        m = M.dam_break_2d(h, column=col, seed=100 + i)
        st = M.wc_initial_states(m, column=col) if kind == api.KIND_WC_CDS_DPDT else \
            M.incomp_initial_states(m, column=col)
        out.append(SV.Request(kind, m, st, steps, precision=api.PREC_MIXED if i % 2 == 0 else api.PREC_FP64,
                              mu=1e-3 * (1 + i)))
    return out


def test_estimate_covers_context_memory(gpu_lib, c1_mesh, small3d_mesh):
    for kind in (api.KIND_INCOMP_PSPG, api.KIND_WC_CDS_DPDT):
        for prec in (api.PREC_FP64, api.PREC_MIXED):
            for mesh in (c1_mesh, small3d_mesh):
                p = api.default_params(kind, mesh.dim)
                p.precision = prec
                ctx = api.Context(p)
                ctx.upload_mesh(mesh)
                used = ctx.device_bytes()
                est = SV.estimate_device_bytes(kind, prec, mesh)
                assert used <= est <= 3 * used + (8 << 20), (kind, prec, mesh.dim, used, est)
                ctx.close()


def test_results_same_alone_and_in_mix(gpu_lib):
    mix = SV.Server(hbm_budget_bytes=8 << 30, max_active=5).run(_requests(), realtime=False)
    assert all(r.error is None for r in mix)
    for r in mix:
        alone = SV.Server(hbm_budget_bytes=8 << 30, max_active=1).run([_requests()[r.rid]], realtime=False)[0]
        assert alone.error is None
        assert np.array_equal(alone.result, r.result) and np.array_equal(alone.positions, r.positions)
        assert alone.converged_steps == r.converged_steps


def test_admission_respects_budget(gpu_lib):
    reqs = _requests()
    est = max(SV.admission_bytes(r) for r in reqs)
    srv = SV.Server(hbm_budget_bytes=int(1.2 * est), max_active=8)
    out = srv.run(reqs, realtime=False)
    assert all(r.error is None for r in out)
    assert srv.peak_bytes <= int(1.2 * est)
    m = SV.metrics(out, srv.makespan)
    assert m["completed"] == len(reqs) and m["latency_p99_s"] >= m["latency_p50_s"] > 0
