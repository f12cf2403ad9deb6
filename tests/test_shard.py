"""Instance sharding across ranks (pfem_gb300.shard): the partitioner, and a world-size-2 gloo
run on CPU in which each rank solves its own share of a batch of independent dam breaks (with
the FP64 oracle standing in for the rank's GPU) and the ranks gather the per-instance results
on the host.  Every instance's result must be bitwise the one a single process computes."""
import os
import socket

import numpy as np
import pytest

from pfem_gb300 import shard


def test_partition_covers_every_instance_once_and_balances():
    rng = np.random.default_rng(3)
    work = rng.integers(500, 50000, size=64).astype(float)
    shards = shard.partition(work, 4)
    owned = sorted(i for s in shards for i in s.instances)
    assert owned == list(range(64))
    loads = [s.work for s in shards]
    assert max(loads) - min(loads) <= work.max()  # LPT bound
    assert shard.partition(work, 4)[2].instances == shards[2].instances  # deterministic
    assert all(s.instances == sorted(s.instances) for s in shards)


def test_partition_respects_the_budget():
    work = [10.0, 9.0, 8.0, 1.0]
    sizes = [6.0, 5.0, 5.0, 1.0]
    shards = shard.partition(work, 2, sizes, budget=11.0)
    assert all(s.bytes <= 11.0 for s in shards)
    assert sorted(i for s in shards for i in s.instances) == [0, 1, 2, 3]
    with pytest.raises(ValueError, match="fits on no rank"):
        shard.partition([1.0, 1.0], 2, [20.0, 1.0], budget=11.0)
    assert shard.instance_bytes(1000, 2) == 1000 * shard.BYTES_PER_NODE[2]


def _instances():
    from pfem_gb300 import workloads as WL

    return [WL.c4_instance(i, lo=300, hi=900) for i in range(5)]


def _solve(inst):
    from oracle import oracle as O

    om = O.OracleMesh(inst.mesh)
    q, res = O.pspg_picard_step(om, inst.q0, 1e-3, mu=inst.mu)
    return {"q": q, "x": om.positions.copy(), "iterations": res.iterations, "converged": res.converged}


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist

    os.environ["OMP_NUM_THREADS"] = "1"
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        insts = _instances()
        work = [i.mesh.n_nodes for i in insts]
        mine = shard.my_share(work, world, rank)
        local = {i: _solve(insts[i]) for i in mine}
        allres = shard.gather_results(local, world)
        if rank == 0:
            np.savez(out_path, **{f"{k}_{f}": np.asarray(v[f]) for k, v in allres.items() for f in v},
                     owners=np.array([shard.my_share(work, world, r) for r in range(world)], dtype=object))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_gather_the_single_process_results(tmp_path):
    import multiprocessing as mp

    os.environ["OMP_NUM_THREADS"] = "1"
    out = str(tmp_path / "gathered.npz")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = np.load(out, allow_pickle=True)
    owners = got["owners"]
    assert len(owners[0]) > 0 and len(owners[1]) > 0  # both ranks did work
    for i, inst in enumerate(_instances()):
        ref = _solve(inst)
        assert bool(got[f"{i}_converged"]) == ref["converged"]
        assert int(got[f"{i}_iterations"]) == ref["iterations"]
        assert np.array_equal(got[f"{i}_q"], ref["q"])
        assert np.array_equal(got[f"{i}_x"], ref["x"])
