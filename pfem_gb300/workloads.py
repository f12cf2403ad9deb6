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

# C3's linear solves stop at relative residual 1e-8 (the configuration).  The mixed form's FP64
# refinement is taken to 1e-10: measured on the C3 mesh over two steps from rest against the
# plain FP64 form solved to 1e-14, the mixed form is 7.1e-6 away at 1e-8, 2.1e-6 at 1e-9 and
# 2.2e-9 at 1e-10 (the system's condition number is ~4e11; the plain FP64 form stopped at 1e-8 is
# 1.6e-4 away).  Its inner FP32 solves are unchanged.
C3_TOL = 1e-8
C3_MIXED_TOL = 1e-10
# C4: both forms solve to relative residual 1e-12 with no absolute floor (the reference's direct
# solver's accuracy; the default absolute floor 1e-10 is loose for the small instances' ||b||)
C4_TOL = 1e-12
C3_DT = 5e-4
C3_COLUMN = (0.5, 0.5, 1.0)


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


def c4_params(i, seed=SEED, lo=500, hi=50000):
    """The draws of instance i of the batched workload, without meshing it: fluid-node target,
    column aspect ratio (height / width) and viscosity."""
    rng = np.random.default_rng([seed, i])
    nf = math.exp(rng.uniform(math.log(lo), math.log(hi)))
    aspect = rng.uniform(0.5, 2.0)
    mu = math.exp(rng.uniform(math.log(1e-3), math.log(1e-1)))
    return nf, aspect, mu


def c4_instance(i, seed=SEED, lo=500, hi=50000, area=2.0):
    """Instance i of the batched workload: its own draw of size, aspect ratio and viscosity."""
    nf, aspect, mu = c4_params(i, seed, lo, hi)
    w, hgt = math.sqrt(area / aspect), math.sqrt(area * aspect)
    h = math.sqrt(area / nf)
    mesh = M.dam_break_2d(h, column=(w, hgt), seed=seed + i)
    return Instance(mesh, M.incomp_initial_states(mesh, column=(w, hgt)), mu, (w, hgt), int(round(nf)))


def c4(n=256, seed=SEED, lo=500, hi=50000, only=None):
    """The batched workload's instances (all n, or the indices in `only`)."""
    return [c4_instance(i, seed, lo, hi) for i in (range(n) if only is None else only)]
