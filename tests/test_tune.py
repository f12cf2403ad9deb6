"""The launch-shape autotuner's host logic (pfem_gb300.tune) against a fake context: candidate
sets per dimension, the per-knob choice from the phase timers, the cache round trip."""
import json

from pfem_gb300 import tune


class FakeCtx:
    """Phase times that depend on the launch shape the way a device might: the SpMV prefers 4
    lanes, the pair kernel 128 threads, the element prep 256, the residual 32."""

    def __init__(self):
        self.t = {}
        self.prof = False
        self.steps = 0
        self.restores = 0

    def set_tuning(self, **kw):
        self.t.update({k: v for k, v in kw.items() if v})

    def set_profiling(self, on):
        self.prof = on

    def reset_phase_times(self):
        pass

    def phase_times(self):
        t = self.t
        return {"Krylov SpMV": (0.05 * (1 + abs(t["spmv_lanes"] - 4)), 10),
                "PSPG matrix": (0.2 * (1 + abs(t["pair_block"] - 128) / 64), 2),
                "PSPG element prep": (0.1 * (1 + abs(t["elem_block"] - 256) / 64), 2),
                "Picard residual": (0.3 if t["res_block"] == 64 else 0.2, 4),
                "Multigrid cycle": (0.1 * (1 + abs(t["mg_lanes"] - 8)), 10)}


def test_candidates_cover_each_knob():
    for dim, l0 in ((2, 4), (3, 8)):
        c = tune.candidates(dim)
        assert sorted({x["spmv_lanes"] for x in c}) == sorted({l0 // 2, l0, 2 * l0})
        assert {x["pair_block"] for x in c} == {64, 128, 256}
        assert {x["res_block"] for x in c} == {32, 64}


def test_autotune_picks_fastest_and_caches(tmp_path):
    path = str(tmp_path / "tune.json")
    ctx = FakeCtx()
    steps = []
    choice, src = tune.autotune(ctx, 3, 330251, "GB300", lambda: steps.append(1), lambda: None, path=path)
    assert src == "measured" and len(steps) == 3
    assert (choice["spmv_lanes"], choice["pair_block"], choice["elem_block"], choice["res_block"],
            choice["mg_lanes"]) == (4, 128, 256, 32, 8)
    assert ctx.t == {k: choice[k] for k in tune.PHASE}
    table = json.load(open(path))
    assert tune.cache_key("GB300", 3, 330251) in table
    # same size class: read back without running steps
    ctx2 = FakeCtx()
    choice2, src2 = tune.autotune(ctx2, 3, 300000, "GB300", lambda: steps.append(1), lambda: None, path=path)
    assert src2 == "cache" and len(steps) == 3 and ctx2.t["pair_block"] == 128
    # another size class or device: measured again
    _, src3 = tune.autotune(FakeCtx(), 3, 1000, "GB300", lambda: steps.append(1), lambda: None, path=path)
    assert src3 == "measured"
