"""Sharding independent instances across GPUs (one process per GPU).

A batch of independent meshes (the batched workload) or a stream of requests has no coupling
between instances, so the multi-GPU form needs no collective on the data path: the instances are
partitioned across the ranks, each rank runs its share as one batched context on its own GPU,
and the ranks exchange only per-instance metrics on the host at the end (an all-gather of small
Python objects over the process group: gloo on CPU, NCCL or gloo with GPUs).

A single mesh does not shard (domain decomposition would need a halo exchange per product and
global reductions per Krylov iteration): single-mesh workloads run as replicas.

The reference runs one `Problem` per process (srcs/simulation/Problem.cpp:303-374) and has no
batching or sharding of its own; this module only decides which rank owns which instance.
"""
from __future__ import annotations

from dataclasses import dataclass

# Device bytes per node of a mixed-precision incompressible context (mesh, topology, node-pair
# blocks in FP32 and bfloat16, FP64 CSR, Krylov and multigrid vectors, element data and
# records), by dimension.  Upper estimates from the allocations for Delaunay meshes (valence ~7
# in 2D, ~15 in 3D; about 2 triangles or 5.3 tetrahedra per node); a caller with a GPU can pass
# its own figure measured with pfg_device_bytes.
BYTES_PER_NODE = {2: 4096, 3: 16384}


@dataclass
class Shard:
    rank: int
    instances: list      # instance indices owned by the rank, ascending
    work: float          # sum of the owned instances' work estimates
    bytes: float         # sum of their device-memory estimates


def instance_bytes(n_nodes: int, dim: int, bytes_per_node: float | None = None) -> float:
    return float(n_nodes) * (bytes_per_node if bytes_per_node else BYTES_PER_NODE[dim])


def partition(work, world: int, sizes=None, budget: float | None = None) -> list[Shard]:
    """Assign instance i (work[i], device bytes sizes[i]) to one of `world` ranks.

    Longest-processing-time greedy: instances in decreasing work (ties by index) go to the rank
    with the least work so far (ties to the lowest rank) among those whose memory stays within
    `budget`.  Deterministic, so every rank computes the same partition without communicating.
    Raises ValueError if an instance fits on no rank."""
    n = len(work)
    if world < 1:
        raise ValueError("world size must be >= 1")
    sizes = list(sizes) if sizes is not None else [0.0] * n
    if len(sizes) != n:
        raise ValueError("work and sizes differ in length")
    shards = [Shard(r, [], 0.0, 0.0) for r in range(world)]
    for i in sorted(range(n), key=lambda k: (-float(work[k]), k)):
        best = None
        for s in shards:
            if budget is not None and s.bytes + sizes[i] > budget:
                continue
            if best is None or s.work < best.work:
                best = s
        if best is None:
            raise ValueError(f"instance {i} ({sizes[i]:.3g} bytes) fits on no rank within the budget {budget:.3g}")
        best.instances.append(i)
        best.work += float(work[i])
        best.bytes += sizes[i]
    for s in shards:
        s.instances.sort()
    return shards


def my_share(work, world: int, rank: int, sizes=None, budget=None) -> list[int]:
    return partition(work, world, sizes, budget)[rank].instances


def gather_results(local: dict, world: int) -> dict:
    """Host-side aggregation: every rank contributes {instance index: result} for the instances
    it owns and receives the union (torch.distributed all_gather_object; no device data moves).
    With world == 1 the input is returned."""
    if world == 1:
        return dict(local)
    import torch.distributed as dist

    parts = [None] * world
    dist.all_gather_object(parts, local)
    out = {}
    for p in parts:
        for k, v in p.items():
            if k in out:
                raise RuntimeError(f"instance {k} reported by two ranks")
            out[k] = v
    return out
