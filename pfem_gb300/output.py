"""Result output on the host: the reference's extractors (`srcs/simulation/extractors/`).

* `writable_data`: the node quantities a problem can write (`ProbIncompNewton::
  getWrittableDataName/getWrittableData`, `IncompNewton/Problem.cpp:43-140`; the WC problem's
  `WCompNewton/Problem.cpp:44-170`): u, v, (w), p, [rho, ax, ay, (az)], ke = |v|^2/2, magV, velocity.
* `write_msh`: `GMSHExtractor::update` (`GMSHExtractor.cpp:57-178`) writes, per output time,
  `<base>_<time>.msh` with the nodes, the elements (triangles = gmsh type 2, tetrahedra = 4)
  and one NodeData view per requested quantity.  The reference goes through the gmsh API; gmsh
  is not available here, so the file is written directly in gmsh's ASCII MSH 2.2 format.
* `CsvExtractor`: the Mass and MinMax extractors (`MassExtractor.cpp:26-37`,
  `MinMaxExtractor.cpp:28-62`) append `time,value` lines every `time_between_writing` seconds,
  with the value a device reduction (`pfg_mass` / `pfg_volume`, `pfg_tip`).
"""
from __future__ import annotations

import numpy as np

from . import api


def writable_data(kind, dim, states, N):
    """{name: (N, ncomp) array} of the quantities the reference's problems write."""
    S = np.asarray(states, float).reshape(-1, N)
    vel = S[:dim]
    out = {name: S[i][:, None] for i, name in enumerate("uvw"[:dim])}
    out["p"] = S[dim][:, None]
    if kind == api.KIND_WC_CDS_DPDT:
        out["rho"] = S[dim + 1][:, None]
        for i, name in enumerate(["ax", "ay", "az"][:dim]):
            out[name] = S[dim + 2 + i][:, None]
    v2 = (vel * vel).sum(axis=0)
    out["ke"] = (0.5 * v2)[:, None]
    out["magV"] = np.sqrt(v2)[:, None]
    velocity = np.zeros((N, 3))
    velocity[:, :dim] = vel.T
    out["velocity"] = velocity
    return out


def write_msh(path, mesh, positions, states, kind, time, step=0, what=("p", "ke", "u", "v"), write_as="NodesElements"):
    """One GMSH output file (ASCII MSH 2.2) with the nodes, the elements and a NodeData view
    per quantity in `what`."""
    d, N, E = mesh.dim, mesh.n_nodes, mesh.n_elems
    data = writable_data(kind, d, states, N)
    unknown = [w for w in what if w not in data]
    if unknown:
        raise ValueError(f"cannot write {unknown}; available: {sorted(data)}")
    X = np.zeros((N, 3))
    X[:, :d] = np.asarray(positions, float).reshape(d, N).T
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(N)]
    lines += [f"{n + 1} {X[n, 0]:.17g} {X[n, 1]:.17g} {X[n, 2]:.17g}" for n in range(N)]
    lines.append("$EndNodes")
    elems = []
    if write_as in ("Elements", "NodesElements"):
        etype = 2 if d == 2 else 4
        conn = mesh.conn.T + 1
        elems += [f"{etype} 2 2 2 " + " ".join(map(str, conn[e])) for e in range(E)]
    if write_as in ("Nodes", "NodesElements"):
        elems += [f"15 2 1 1 {n + 1}" for n in range(N)]
    lines += ["$Elements", str(len(elems))]
    lines += [f"{i + 1} {s}" for i, s in enumerate(elems)]
    lines.append("$EndElements")
    for name in what:
        vals = data[name]
        nc = vals.shape[1]
        lines += ["$NodeData", "1", f'"{name}"', "1", f"{time:.17g}", "3", str(step), str(nc), str(N)]
        lines += [f"{n + 1} " + " ".join(f"{v:.17g}" for v in vals[n]) for n in range(N)]
        lines.append("$EndNodeData")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


class GmshExtractor:
    """Writes `<base>_<time>.msh` every `time_between_writing` seconds of simulated time."""

    def __init__(self, base, time_between_writing, what=("p", "ke", "u", "v"), write_as="NodesElements"):
        self.base = base[:-4] if base.endswith(".msh") else base
        self.dt = time_between_writing
        self.what = what
        self.write_as = write_as
        self.next = 0.0
        self.written = []

    def __call__(self, solver, force=False):
        if solver.time < self.next and not force:
            return
        path = f"{self.base}_{solver.time:.6f}.msh"
        write_msh(path, solver.mesh, solver.positions(), solver.states(), solver.kind, solver.time, solver.steps,
                  self.what, self.write_as)
        self.written.append(path)
        if not force:
            self.next += self.dt


class CsvExtractor:
    """Mass (WC) / volume (incompressible) or MinMax front position as `time,value` lines."""

    def __init__(self, path, time_between_writing, quantity="mass", coordinate=0, min_max="max"):
        self.path = path
        self.dt = time_between_writing
        self.quantity = quantity
        self.coordinate = coordinate
        self.want_max = min_max == "max"
        self.next = 0.0
        open(path, "w").close()

    def __call__(self, solver, force=False):
        if solver.time < self.next and not force:
            return
        if self.quantity == "mass":
            v = solver.ctx.mass() if solver.kind == api.KIND_WC_CDS_DPDT else solver.ctx.volume()
        else:
            v = solver.ctx.tip(self.coordinate, self.want_max)
        with open(self.path, "a") as f:
            f.write(f"{solver.time:.17g},{v:.17g}\n")
        if not force:
            self.next += self.dt
