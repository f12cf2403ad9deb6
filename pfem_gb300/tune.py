"""Autotuner of the mixed incompressible form's launch shapes (pfg_set_tuning).

The shape of five kernels is chosen per device, dimension and mesh size: lanes per node of the
Krylov SpMV and of the multigrid's level-0 sweeps, the pair assembly's form and threads per
block, threads per block of the element prep and of the refinement residual's element kernel.  Each candidate runs one full Picard step from the same saved state
with the library's phase timers on (direct launches bracketed by CUDA events), and each knob
takes the value whose phase was fastest per launch; the knobs belong to different phases, so
one sweep of three steps covers them all (the residual kernel's two shapes alternate).  The
choice is cached in a JSON file (PFEM_GB300_TUNE_CACHE, default ~/.cache/pfem_gb300/tune.json)
under the key device name / dimension / log2 of the node count, so later contexts of the same
size class apply it without running steps.

The reference has no counterpart (its assembly and solve are CPU code, MomContEquationPSPG.inl);
the launch shapes only change the order of the SpMV's lane sums, not the arithmetic.
"""
from __future__ import annotations

import json
import math
import os

LANES0 = {2: 4, 3: 8}
PHASE = {"spmv_lanes": "Krylov SpMV", "pair_block": "PSPG matrix", "elem_block": "PSPG element prep",
         "res_block": "Picard residual", "mg_lanes": "Multigrid cycle"}


def candidates(dim):
    l0 = LANES0[dim]
    lanes = (l0, l0 // 2, 2 * l0)
    blocks = (128, 256, 64)  # pair assembly: 128 row-staged, 256 item-parallel, 64 pair-parallel
    res = (64, 32, 64)
    return [dict(spmv_lanes=lanes[i], pair_block=blocks[i], elem_block=blocks[i], res_block=res[i],
                 mg_lanes=lanes[i]) for i in range(3)]


def cache_path():
    return os.environ.get("PFEM_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "pfem_gb300", "tune.json"))


def cache_key(device, dim, n_nodes):
    return f"{device}|dim{dim}|n2^{max(0, int(math.log2(max(n_nodes, 1))))}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, table):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def autotune(ctx, dim, n_nodes, device, step, restore, path=None, force=False):
    """Choose and apply the launch shapes of `ctx`.  step(): one Picard step (or batched step);
    restore(): put back the state the steps start from.  Returns (choice, source) with source
    "cache" or "measured"; the measured per-launch microseconds are in choice["us"]."""
    path = path or cache_path()
    key = cache_key(device, dim, n_nodes)
    table = _load(path)
    if not force and key in table:
        choice = table[key]
        ctx.set_tuning(**{k: choice[k] for k in PHASE})
        return choice, "cache"
    per = {k: {} for k in PHASE}
    for cand in candidates(dim):
        ctx.set_tuning(**cand)
        restore()
        ctx.set_profiling(True)
        ctx.reset_phase_times()
        step()
        phases = ctx.phase_times()
        ctx.set_profiling(False)
        for knob, ph in PHASE.items():
            ms, n = phases.get(ph, (0.0, 0))
            if n:
                us = 1e3 * ms / n
                v = cand[knob]
                per[knob][v] = min(us, per[knob].get(v, float("inf")))
    choice = {}
    for knob in PHASE:
        if per[knob]:
            choice[knob] = min(per[knob], key=per[knob].get)
        else:
            choice[knob] = candidates(dim)[0][knob]
    choice["us"] = {k: {str(v): round(t, 2) for v, t in per[k].items()} for k in PHASE}
    ctx.set_tuning(**{k: choice[k] for k in PHASE})
    restore()
    table[key] = choice
    try:
        _store(path, table)
    except OSError:
        pass  # a read-only home keeps the choice for this process only
    return choice, "measured"
