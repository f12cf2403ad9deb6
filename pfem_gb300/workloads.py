"""Seeded synthetic dam-break workloads.

The reference's dam-break examples (`examples/2D/damBreakKoshizuka`, `examples/3D/...`)
ship no mesh files, so every workload here is generated: nodes on a lattice jittered by
+-0.1 h with a seeded draw, walls at spacing h, Delaunay + alpha shape (alpha = 1.2).

  C1  2D incompressible PSPG, h = 0.05 (~1.0k nodes), dt = 1e-3, 200 steps
  C2  2D weakly compressible, h = 0.005 (~82k nodes, ~160k triangles), 2000 steps
  C3  3D incompressible, h = 0.01: column 0.5 x 0.5 x 1.0 in a 2.0 x 0.5 x 1.5 tank
  C4  256 independent 2D incompressible instances: fluid nodes log-uniform in [500, 50k],
      column aspect ratio (height / width) uniform in [0.5, 2], mu log-uniform in
      [1e-3, 1e-1], instance seed = base seed + i
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import mesh as M

SEED = 20261203


def c1():
    return M.dam_break_2d(0.05)


def c2():
    return M.dam_break_2d(0.005)


def c3(h=0.01):
    return M.dam_break_3d(h)


@dataclass
class Instance:
    mesh: M.HostMesh
    q0: np.ndarray
    mu: float
    column: tuple
    fluid_target: int


def c4_instance(i, seed=SEED, lo=500, hi=50000, area=2.0):
    """Instance i of the batched workload: its own draw of size, aspect ratio and viscosity."""
    rng = np.random.default_rng([seed, i])
    nf = math.exp(rng.uniform(math.log(lo), math.log(hi)))
    aspect = rng.uniform(0.5, 2.0)
    mu = math.exp(rng.uniform(math.log(1e-3), math.log(1e-1)))
    w, hgt = math.sqrt(area / aspect), math.sqrt(area * aspect)
    h = math.sqrt(area / nf)
    mesh = M.dam_break_2d(h, column=(w, hgt), seed=seed + i)
    return Instance(mesh, M.incomp_initial_states(mesh, column=(w, hgt)), mu, (w, hgt), int(round(nf)))


def c4(n=256, seed=SEED, lo=500, hi=50000):
    return [c4_instance(i, seed, lo, hi) for i in range(n)]
