"""Host-side PFEM mesh: synthetic dam-break node clouds and the alpha-shape triangulation.

This is the host half of the drop-in boundary.  The reference triangulates with CGAL
(`srcs/mesh/Mesh2D.cpp:32-251`, `srcs/mesh/Mesh3D.cpp:36-286`); CGAL is not available here,
so the Delaunay triangulation comes from Qhull (scipy.spatial.Delaunay) and the alpha-shape
classification is restated on top of it:

* a simplex is INTERIOR when its squared circumradius is <= (alpha*hchar)^2
  (`Mesh2D.cpp:54`, `Mesh3D.cpp:60`: CGAL alpha value of a face/cell of a Delaunay
  triangulation of unweighted points is its squared circumradius);
* INTERIOR simplices whose nodes are all boundary nodes are deleted unless one of their
  nodes touches an INTERIOR simplex with a non-boundary node (`checkFaceDeletion`,
  `Mesh2D.cpp:57-109`; 3D also drops all-boundary slivers of volume < 0.02 h^3,
  `Mesh3D.cpp:92`);
* facets are the REGULAR edges/faces (exactly one INTERIOR side) whose interior simplex was
  kept; nodes of a facet that is not entirely on the boundary are free-surface nodes
  (`Mesh2D.cpp:200-245`, `Mesh3D.cpp:224-280`);
* kept simplices are oriented positively (CGAL's convention; the reference never takes
  |detJ|).

Arrays are laid out the way the GPU library takes them: positions and connectivity are
structure-of-arrays (`pos[d, n]`, `conn[k, e]`), node flags are one byte per node.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# Node flag bits (same values as PFG_NODE_* in include/pfem_gpu.h).
BOUND = 1          # wall node (Node::isBound, srcs/mesh/Node.hpp:101)
FREE_SURFACE = 2   # on the free surface (Node::isOnFreeSurface)
FIXED = 4          # position never updated (Node::isFixed)
DIRICHLET = 8      # bound node whose tag carries a velocity BC (Solver::m_bcTagFlags bit 0)


@dataclass
class HostMesh:
    dim: int
    pos: np.ndarray                 # (dim, N) float64
    flags: np.ndarray               # (N,) uint8
    conn: np.ndarray                # (dim+1, E) int32, positively oriented
    facets: np.ndarray = field(default_factory=lambda: np.zeros((2, 0), np.int32))  # (dim, F)
    facet_elm: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))    # (F,)
    facet_out: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))    # (F,)
    hchar: float = 0.0
    alpha: float = 1.2

    @property
    def n_nodes(self) -> int:
        return self.pos.shape[1]

    @property
    def n_elems(self) -> int:
        return self.conn.shape[1]

    def is_free(self) -> np.ndarray:
        """Nodes belonging to no element (Node::isFree, `srcs/mesh/Node.inl:48-51`)."""
        used = np.zeros(self.n_nodes, bool)
        used[self.conn.ravel()] = True
        return ~used

    def copy(self) -> "HostMesh":
        return HostMesh(self.dim, self.pos.copy(), self.flags.copy(), self.conn.copy(),
                        self.facets.copy(), self.facet_elm.copy(), self.facet_out.copy(),
                        self.hchar, self.alpha)


# --------------------------------------------------------------------------------------
# Synthetic dam-break node clouds
# --------------------------------------------------------------------------------------

def _wall_line(a, b, h):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    n = int(round(np.linalg.norm(b - a) / h))
    t = np.arange(n + 1) / n
    return a[None, :] + t[:, None] * (b - a)[None, :]


def dam_break_nodes_2d(h, tank=(4.0, 3.0), column=(1.0, 2.0), jitter=0.1, seed=20261203):
    """Open-top tank with walls at spacing h (left, bottom, right; not jittered, bound and fixed)
    and a fluid column at the left wall on a lattice offset by h from the walls, each
    coordinate jittered by U(-jitter*h, +jitter*h) from a PCG64 generator seeded with `seed`.

    Stands in for the reference's `examples/2D/damBreakKoshizuka` case, whose gmsh mesh is
    not shipped.  Returns (pos (2,N), flags (N,))."""
    W, H = tank
    cw, ch = column
    walls = np.concatenate([
        _wall_line((0.0, H), (0.0, 0.0), h),      # left wall, top to bottom
        _wall_line((0.0, 0.0), (W, 0.0), h)[1:],  # bottom
        _wall_line((W, 0.0), (W, H), h)[1:],      # right wall
    ])
    nx = int(round(cw / h))
    ny = int(round(ch / h))
    gx, gy = np.meshgrid(h * np.arange(1, nx + 1), h * np.arange(1, ny + 1), indexing="ij")
    fluid = np.stack([gx.ravel(), gy.ravel()], axis=1)
    rng = np.random.default_rng(seed)
    fluid = fluid + rng.uniform(-jitter * h, jitter * h, size=fluid.shape)
    pos = np.concatenate([walls, fluid]).T.copy()
    flags = np.zeros(pos.shape[1], np.uint8)
    flags[:walls.shape[0]] = BOUND | FIXED | DIRICHLET
    return pos, flags


def sloshing_nodes_2d(h, width=1.0, wall_height=1.2, depth=1.0, amplitude=0.1, jitter=0.1, seed=20261203):
    """The tank of `examples/2D/sloshing` (geometry.geo: width b = 1, walls up to 1.2 b, free
    surface y = b + a sin(pi x / b - pi / 2) with a = 0.1, so the water starts at rest with a
    tilted-cosine surface and sloshes under gravity): walls at spacing h (left, bottom, right;
    bound and fixed), fluid nodes on a lattice offset by h from the walls under the surface,
    jittered like the dam break.  Stands in for the example's gmsh mesh, which is not shipped.
    Returns (pos (2,N), flags (N,))."""
    W, H = width, wall_height * width
    walls = np.concatenate([
        _wall_line((0.0, H), (0.0, 0.0), h),
        _wall_line((0.0, 0.0), (W, 0.0), h)[1:],
        _wall_line((W, 0.0), (W, H), h)[1:],
    ])
    nx = int(round(W / h))
    xs = h * np.arange(1, nx)
    pts = []
    for x in xs:
        top = depth + amplitude * np.sin(np.pi * x / W - np.pi / 2)
        ny = int(np.floor(top / h + 1e-9))
        for j in range(1, ny + 1):
            pts.append((x, h * j))
    fluid = np.asarray(pts, float)
    rng = np.random.default_rng(seed)
    fluid = fluid + rng.uniform(-jitter * h, jitter * h, size=fluid.shape)
    pos = np.concatenate([walls, fluid]).T.copy()
    flags = np.zeros(pos.shape[1], np.uint8)
    flags[:walls.shape[0]] = BOUND | FIXED | DIRICHLET
    return pos, flags


def dam_break_nodes_3d(h, tank=(2.0, 0.5, 1.5), column=(0.5, 0.5, 1.0), jitter=0.1, seed=20261203):
    """3D open-top tank (floor and four side walls at spacing h) with a fluid column in the
    x=0 corner region, interior lattice offset by h from the walls and jittered like the 2D
    case.  Returns (pos (3,N), flags (N,))."""
    W, D, H = tank
    cw, cd, chh = column
    nxw, nyw, nzw = (int(round(W / h)), int(round(D / h)), int(round(H / h)))
    xs = h * np.arange(nxw + 1)
    ys = h * np.arange(nyw + 1)
    zs = h * np.arange(nzw + 1)
    pts = []
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    pts.append(np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1))                 # floor
    for y in (0.0, D):                                                                # y walls
        X, Z = np.meshgrid(xs, zs[1:], indexing="ij")
        pts.append(np.stack([X.ravel(), np.full(X.size, y), Z.ravel()], 1))
    for x in (0.0, W):                                                                # x walls
        Y, Z = np.meshgrid(ys[1:-1], zs[1:], indexing="ij")
        pts.append(np.stack([np.full(Y.size, x), Y.ravel(), Z.ravel()], 1))
    walls = np.concatenate(pts)
    nx = int(round(cw / h)) - (1 if cw >= W else 0)
    ny = int(round(cd / h)) - (1 if cd >= D else 0)
    nz = int(round(chh / h))
    gx, gy, gz = np.meshgrid(h * np.arange(1, nx + 1), h * np.arange(1, ny + 1),
                             h * np.arange(1, nz + 1), indexing="ij")
    fluid = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], 1)
    rng = np.random.default_rng(seed)
    fluid = fluid + rng.uniform(-jitter * h, jitter * h, size=fluid.shape)
    pos = np.concatenate([walls, fluid]).T.copy()
    flags = np.zeros(pos.shape[1], np.uint8)
    flags[:walls.shape[0]] = BOUND | FIXED | DIRICHLET
    return pos, flags


# --------------------------------------------------------------------------------------
# Alpha-shape triangulation
# --------------------------------------------------------------------------------------

_TRIPLE = ((1, 3, 2), (0, 2, 3), (0, 3, 1), (0, 1, 2))


def _circumradius2(P, simp):
    """Squared circumradius of each simplex (rows of `simp` index columns of P^T)."""
    dim = P.shape[1]
    X = P[simp]                      # (E, d+1, d)
    A = X[:, 1:, :] - X[:, :1, :]    # (E, d, d)
    rhs = 0.5 * np.einsum("eij,eij->ei", A, A)
    det = np.linalg.det(A)
    scale = np.einsum("eij,eij->e", A, A) ** (dim / 2.0)
    ok = np.abs(det) > 1e-12 * scale          # flat simplices (coplanar wall nodes) never qualify
    r2 = np.full(simp.shape[0], np.inf)
    if ok.any():
        c = np.linalg.solve(A[ok], rhs[ok][..., None])[..., 0]
        r2[ok] = np.einsum("ei,ei->e", c, c)
    return r2


def _signed_measure(P, simp):
    X = P[simp]
    A = X[:, 1:, :] - X[:, :1, :]
    return np.linalg.det(A)


def alpha_shape(pos, flags, hchar, alpha=1.2, delete_flying_nodes=False, jitter=None):
    """Delaunay + alpha-shape remesh of a node cloud (`Mesh::triangulateAlphaShape2D/3D`).

    Returns a HostMesh.  Free-surface bits are recomputed; the other flag bits are kept.
    With `delete_flying_nodes`, nodes that end up in no element and are not bound are
    removed (`Mesh::deleteFlyingNodes`, `srcs/mesh/Mesh.cpp:251-331`) and the returned mesh
    carries `node_origin` (old index of each kept node) as an attribute.  `jitter` ((dim, n)
    array, or a callable of n giving one) replaces the default perturbation the triangulation
    sees (none in 2D, a seeded 1e-6 h in 3D)."""
    from scipy.spatial import Delaunay

    dim = pos.shape[0]
    P = np.ascontiguousarray(pos.T)
    if jitter is not None:
        jig = jitter(P.shape[0]) if callable(jitter) else jitter
        tri = Delaunay(P + np.ascontiguousarray(np.asarray(jig, float).T))
    elif dim == 3:
        # The unjittered wall lattice is full of co-spherical point sets, on which Qhull's
        # merging is an order of magnitude slower.  Triangulating a copy moved by 1e-6 h
        # (seeded) breaks the ties, as CGAL's symbolic perturbation does; all geometry below
        # uses the true positions, so flat wall simplices still drop out.
        jig = np.random.default_rng(7).uniform(-1.0, 1.0, P.shape) * (1e-6 * hchar)
        tri = Delaunay(P + jig)
    else:
        tri = Delaunay(P)
    simp = tri.simplices.astype(np.int64)
    nbr = tri.neighbors.astype(np.int64)
    vol = _signed_measure(P, simp)
    # positive orientation: swap the last two vertices (and their opposite neighbours)
    neg = vol < 0
    simp[neg, dim - 1], simp[neg, dim] = simp[neg, dim].copy(), simp[neg, dim - 1].copy()
    nbr[neg, dim - 1], nbr[neg, dim] = nbr[neg, dim].copy(), nbr[neg, dim - 1].copy()
    vol = np.abs(vol)
    alpha2 = (alpha * hchar) ** 2
    interior = _circumradius2(P, simp) <= alpha2
    interior &= vol > 0.0

    bound = (flags & BOUND) != 0
    sb = bound[simp]
    allbound = sb.all(axis=1)
    # a vertex is "wet" when an interior simplex incident to it has a non-bound vertex
    wet = np.zeros(P.shape[0], bool)
    wetting = interior & ~allbound
    wet[simp[wetting].ravel()] = True
    delete = interior & allbound & ~wet[simp].any(axis=1)
    if dim == 3:
        import math
        sliver = vol / math.factorial(3) < 0.02 * hchar ** 3
        delete |= interior & allbound & sliver
    keep = interior & ~delete

    elem_index = -np.ones(simp.shape[0], np.int64)
    elem_index[keep] = np.arange(int(keep.sum()))
    conn = simp[keep].T.astype(np.int32)

    # facets: REGULAR edges/faces of the alpha complex whose interior simplex was kept
    facets, facet_elm, facet_out = [], [], []
    ks, ls = np.nonzero(interior[:, None] & ~np.where(nbr >= 0, interior[np.maximum(nbr, 0)], False))
    for s, l in zip(ks, ls):
        if not keep[s]:
            continue
        v = simp[s]
        if dim == 2:
            f = [v[(l + 1) % 3], v[(l + 2) % 3]]
        else:
            # vertex order of the face opposite vertex l, as CGAL's vertex_triple_index
            # orders it for a positively oriented cell
            f = [v[i] for i in _TRIPLE[l]]
        facets.append(f)
        facet_elm.append(elem_index[s])
        facet_out.append(v[l])
    flags = flags.copy()
    flags &= np.uint8(~FREE_SURFACE & 0xFF)
    facets = np.array(facets, np.int32).reshape(-1, dim).T.copy()
    if facets.shape[1]:
        fb = bound[facets].all(axis=0)
        fs_nodes = facets[:, ~fb].ravel()
        flags[fs_nodes] |= FREE_SURFACE
    mesh = HostMesh(dim, pos.copy(), flags, np.ascontiguousarray(conn), facets,
                    np.array(facet_elm, np.int32), np.array(facet_out, np.int32), hchar, alpha)
    mesh.node_origin = np.arange(mesh.n_nodes, dtype=np.int32)
    if delete_flying_nodes:
        free = mesh.is_free()
        drop = free & ~bound
        if drop.any():
            keep_n = np.nonzero(~drop)[0]
            remap = -np.ones(mesh.n_nodes, np.int64)
            remap[keep_n] = np.arange(keep_n.size)
            mesh = HostMesh(dim, mesh.pos[:, keep_n].copy(), mesh.flags[keep_n].copy(),
                            remap[mesh.conn].astype(np.int32),
                            remap[mesh.facets].astype(np.int32), mesh.facet_elm,
                            remap[mesh.facet_out].astype(np.int32), hchar, alpha)
            mesh.node_origin = keep_n.astype(np.int32)
    return mesh


# --------------------------------------------------------------------------------------
# Dam-break cases and their initial conditions
# --------------------------------------------------------------------------------------

def dam_break_2d(h=0.05, alpha=1.2, seed=20261203, column=(1.0, 2.0), tank=(4.0, 3.0)):
    pos, flags = dam_break_nodes_2d(h, tank=tank, column=column, seed=seed)
    return alpha_shape(pos, flags, h, alpha, delete_flying_nodes=True)


def dam_break_3d(h=0.01, alpha=1.2, seed=20261203, column=(0.5, 0.5, 1.0), tank=(2.0, 0.5, 1.5)):
    pos, flags = dam_break_nodes_3d(h, tank=tank, column=column, seed=seed)
    return alpha_shape(pos, flags, h, alpha, delete_flying_nodes=True)


def sloshing_2d(h=0.02, alpha=1.2, seed=20261203, amplitude=0.1):
    pos, flags = sloshing_nodes_2d(h, amplitude=amplitude, seed=seed)
    return alpha_shape(pos, flags, h, alpha, delete_flying_nodes=True)


def square_nodes_2d(h, side=1.0, jitter=0.1, seed=20261203):
    """A free square of fluid, no walls: the lattice h * (i, j), 0 <= i, j <= side / h, with the
    interior nodes jittered like the dam-break column (the boundary stays straight).

    Stands in for the reference's surface tension case `examples/2D/squareToDisk` (unit
    square, gmsh size 0.025, no boundary conditions; the .msh is not shipped).
    Returns (pos (2,N), flags (N,))."""
    n = int(round(side / h))
    gx, gy = np.meshgrid(side * np.arange(n + 1) / n, side * np.arange(n + 1) / n, indexing="ij")
    pos = np.stack([gx.ravel(), gy.ravel()])
    inner = (gx.ravel() > 0) & (gx.ravel() < side) & (gy.ravel() > 0) & (gy.ravel() < side)
    rng = np.random.default_rng(seed)
    pos[:, inner] += rng.uniform(-jitter * h, jitter * h, size=(2, int(inner.sum())))
    return pos.copy(), np.zeros(pos.shape[1], np.uint8)


def square_to_disk_2d(h=0.025, alpha=1.2, seed=20261203):
    pos, flags = square_nodes_2d(h, seed=seed)
    return alpha_shape(pos, flags, h, alpha)


def ball_nodes_3d(R, h):
    """A free ball of fluid, no walls: the centre plus shells of radius R k / n (n = R / h)
    with Fibonacci-sphere points at spacing ~h (a 3D surface tension case).
    Returns (pos (3,N), flags (N,))."""
    pts = [np.zeros((1, 3))]
    nr = int(round(R / h))
    ga = np.pi * (3 - np.sqrt(5))
    for k in range(1, nr + 1):
        r = R * k / nr
        m = max(12, int(round(4.4 * np.pi * r * r / (h * h))))
        i = np.arange(m) + 0.5
        z = 1 - 2 * i / m
        rr = np.sqrt(1 - z * z)
        th = ga * i + 0.7 * k
        pts.append(r * np.stack([rr * np.cos(th), rr * np.sin(th), z], 1))
    pos = np.concatenate(pts).T.copy()
    return pos, np.zeros(pos.shape[1], np.uint8)


def ball_3d(R=0.1, h=0.02, alpha=1.3):
    pos, flags = ball_nodes_3d(R, h)
    return alpha_shape(pos, flags, h, alpha)


def incomp_initial_states(mesh, rho=1000.0, g=9.81, column=(1.0, 2.0)):
    """Hydrostatic column at rest (`damBreakKoshizukaIncomp.lua:73-81` with the column's
    width and height): q = [v (d fields), p], field-major, length (d+1)*N."""
    d, N = mesh.dim, mesh.n_nodes
    Hc = column[-1]
    y = mesh.pos[d - 1]
    inside = (y <= Hc) & (mesh.pos[0] <= column[0] + 2 * mesh.hchar)
    p = np.where(inside, rho * g * (Hc - y), 0.0)
    q = np.zeros((d + 1) * N)
    q[d * N:] = p
    return q


def wc_initial_states(mesh, rho_star=1000.0, K0=2.2e7, K0p=7.0, g=9.81, column=(1.0, 2.0)):
    """Tait-Murnaghan hydrostatic column (`damBreakKoshizukaComp.lua:86-100`): states
    [v (d), p, rho, a (d)] field-major, length (2d+2)*N."""
    d, N = mesh.dim, mesh.n_nodes
    z0 = column[-1]
    y = mesh.pos[d - 1]
    inside = (y <= z0) & (mesh.pos[0] <= column[0] + 1.1 * mesh.hchar)
    rho = np.where(inside,
                   rho_star * ((K0p - 1) / K0 * rho_star * g * (z0 - np.minimum(y, z0)) + 1) ** (1 / (K0p - 1)),
                   rho_star)
    p = np.where(inside, K0 / K0p * ((rho / rho_star) ** K0p - 1), 0.0)
    s = np.zeros((2 * d + 2) * N)
    s[d * N:(d + 1) * N] = p
    s[(d + 1) * N:(d + 2) * N] = rho
    return s


def sloshing_wc_initial_states(mesh, rho_star=1.0, K0=2.2e5, K0p=7.6, g=9.81, depth=1.0, amplitude=0.1):
    """`sloshingComp.lua:71-85`: Tait-Murnaghan hydrostatic field under the free surface
    z0(x) = depth + amplitude sin(pi x - pi / 2), at rest."""
    d, N = mesh.dim, mesh.n_nodes
    x, y = mesh.pos[0], mesh.pos[d - 1]
    z0 = depth + amplitude * np.sin(np.pi * x - np.pi / 2)
    inside = y <= z0
    rho = np.where(inside, rho_star * ((K0p - 1) / K0 * rho_star * g * (z0 - np.minimum(y, z0)) + 1) ** (1 / (K0p - 1)),
                   rho_star)
    p = np.where(inside, K0 / K0p * ((rho / rho_star) ** K0p - 1), 0.0)
    s = np.zeros((2 * d + 2) * N)
    s[d * N:(d + 1) * N] = p
    s[(d + 1) * N:(d + 2) * N] = rho
    return s


def concat_meshes(meshes):
    """Union of independent meshes in one numbering, instance i owning nodes
    [offsets[i], offsets[i+1]) and the elements among them (the layout pfg_set_instances
    takes).  Returns (mesh, offsets)."""
    dim = meshes[0].dim
    offs = np.zeros(len(meshes) + 1, np.int64)
    offs[1:] = np.cumsum([m.n_nodes for m in meshes])
    pos = np.concatenate([m.pos for m in meshes], axis=1)
    flags = np.concatenate([m.flags for m in meshes])
    conn = np.concatenate([m.conn + o for m, o in zip(meshes, offs[:-1])], axis=1).astype(np.int32)
    return HostMesh(dim, np.ascontiguousarray(pos), flags, np.ascontiguousarray(conn),
                    hchar=meshes[0].hchar, alpha=meshes[0].alpha), offs.astype(np.int32)


def concat_states(states, meshes):
    """Field-major per-instance state vectors -> one field-major vector of the union."""
    nf = len(states[0]) // meshes[0].n_nodes
    return np.concatenate([np.concatenate([s[f * m.n_nodes:(f + 1) * m.n_nodes] for s, m in zip(states, meshes)])
                           for f in range(nf)])


def split_states(q, meshes):
    """Inverse of concat_states."""
    N = sum(m.n_nodes for m in meshes)
    nf = len(q) // N
    out, o = [], 0
    for m in meshes:
        out.append(np.concatenate([q[f * N + o:f * N + o + m.n_nodes] for f in range(nf)]))
        o += m.n_nodes
    return out


def pspg_nnz(mesh):
    """Non-zeros of the PSPG matrix pattern: identity rows for free nodes and bound-node
    velocities, deg(n)(d+1) entries in every other row (deg counts the node itself)."""
    import scipy.sparse as sp

    d, N, E = mesh.dim, mesh.n_nodes, mesh.n_elems
    inc = sp.csr_matrix((np.ones(E * (d + 1)), (np.repeat(np.arange(E), d + 1), mesh.conn.T.ravel())), shape=(E, N))
    deg = np.diff((inc.T @ inc).tocsr().indptr)
    free = mesh.is_free()
    bound = (mesh.flags & BOUND) != 0
    per = np.where(free, d + 1, np.where(bound, d + deg * (d + 1), (d + 1) * deg * (d + 1)))
    return int(per.sum())
