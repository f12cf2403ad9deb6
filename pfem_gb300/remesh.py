"""Host remeshing between GPU steps: the reference's `Mesh::remesh` (`srcs/mesh/Mesh.cpp:919-926`).

    laplacianSmoothingBoundaries -> addNodes -> removeNodes -> checkBoundingBox -> triangulateAlphaShape

restated on structure-of-arrays node data.  Node states travel with their nodes: deleted nodes
drop their states, an added node gets the mean state of its element's nodes (`Mesh.cpp:59-67`),
and the triangulation's node deletions (flying nodes) are applied through `node_origin`.  The
result is what the GPU library is handed after a remesh: positions, flags, connectivity and the
remapped field-major states.

Neighbour lists are the nodes sharing an element with a node, in ascending index (the
reference builds them from its triangulation; the order only matters to `removeNodes`, which
deletes the second node of a too-close pair).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import mesh as M


@dataclass
class RemeshParams:
    """The `Mesh` block of a problem file (`damBreakKoshizukaIncomp.lua:6-17`)."""
    hchar: float
    alpha: float = 1.2
    omega: float = 0.7
    gamma: float = 0.2
    add_on_fs: bool = False
    delete_flying_nodes: bool = True
    laplacian_smoothing_boundaries: bool = True
    bounding_box: tuple | None = None   # (xmin, ymin[, zmin], xmax, ymax[, zmax])


def neighbours(mesh):
    """Sorted distinct neighbour nodes of every node (nodes sharing an element, itself excluded)."""
    import scipy.sparse as sp

    d, N, E = mesh.dim, mesh.n_nodes, mesh.n_elems
    inc = sp.csr_matrix((np.ones(E * (d + 1)), (np.repeat(np.arange(E), d + 1), mesh.conn.T.ravel())), shape=(E, N))
    adj = (inc.T @ inc).tocsr()
    adj.setdiag(0)
    adj.eliminate_zeros()
    adj.sort_indices()
    return adj.indptr, adj.indices


def laplacian_smoothing_boundaries(mesh, pos):
    """`Mesh::laplacianSmoothingBoundaries` (`Mesh.cpp:580-760`): for every element touching the
    walls with exactly `dim` bound nodes, a non-bound node closer than h/3 to the wall facet is
    pushed h/3 along the facet normal (free-surface node) or moved to the mean of its
    neighbours.  Elements are visited in order and see earlier moves."""
    d, h = mesh.dim, mesh.hchar
    bound = (mesh.flags & M.BOUND) != 0
    fs = (mesh.flags & M.FREE_SURFACE) != 0
    ip, ix = neighbours(mesh)
    for e in np.nonzero(bound[mesh.conn].sum(axis=0) == d)[0]:
        nodes = mesh.conn[:, e]
        b = bound[nodes]
        out = int(nodes[~b][0])
        fac = nodes[b]
        P = pos[:, fac].T
        normal = np.zeros(d)
        if d == 2:
            if P[0, 0] == P[1, 0]:
                normal[0] = 1
                dist = abs(P[0, 0] - pos[0, out])
            elif P[0, 1] == P[1, 1]:
                normal[1] = 1
                dist = abs(P[0, 1] - pos[1, out])
            else:
                normal = np.linalg.lstsq(P, -np.ones(2), rcond=None)[0]
                dist = abs(normal @ pos[:, out] + 1) / np.linalg.norm(normal)
        else:
            if P[0, 0] == P[1, 0] and P[1, 0] == P[2, 0]:
                normal[0] = 1
                dist = abs(P[0, 0] - pos[0, out])
            elif P[0, 1] == P[1, 1] and P[1, 1] == P[2, 1]:
                normal[1] = 1
                dist = abs(P[0, 1] - pos[1, out])
            elif P[0, 2] == P[1, 2] and P[1, 1] == P[2, 2]:  # the reference compares y with z here
                normal[2] = 1
                dist = abs(P[0, 2] - pos[2, out])
            else:
                normal = np.linalg.lstsq(P, -np.ones(3), rcond=None)[0]
                dist = abs(normal @ pos[:, out] + 1) / np.linalg.norm(normal)
        if dist > h / 3:
            continue
        if fs[out]:
            n = normal / np.linalg.norm(normal)
            if n @ (pos[:, out] - P[0]) < 0:
                n = -n
            pos[:, out] += h / 3 * n
        else:
            nb = ix[ip[out]:ip[out + 1]]
            pos[:, out] = pos[:, nb].mean(axis=1)


def add_nodes(mesh, pos, states, params):
    """`Mesh::addNodes` (`Mesh.cpp:27-147`): a node at the centroid of every element larger
    than omega h^d (skipping free-surface elements unless addOnFS), with the mean state of the
    element's nodes.  Returns (pos, flags, states) with the new nodes appended."""
    d = mesh.dim
    refsize = 0.5 if d == 2 else 1.0 / 6.0
    X = pos[:, mesh.conn]                       # (d, d+1, E)
    J = X[:, 1:, :] - X[:, :1, :]
    size = np.linalg.det(np.moveaxis(J, 2, 0)) * refsize
    fs = (mesh.flags & M.FREE_SURFACE) != 0
    on_fs = fs[mesh.conn].any(axis=0)
    grow = size > params.omega * params.hchar ** d
    if not params.add_on_fs:
        grow &= ~on_fs
    sel = np.nonzero(grow)[0]
    if sel.size == 0:
        return pos, mesh.flags.copy(), states
    newpos = X[:, :, sel].mean(axis=1)
    N = mesh.n_nodes
    nf = len(states) // N
    S = states.reshape(nf, N)
    newst = S[:, mesh.conn[:, sel]].mean(axis=1)
    pos = np.concatenate([pos, newpos], axis=1)
    flags = np.concatenate([mesh.flags, np.zeros(sel.size, np.uint8)])
    states = np.concatenate([S, newst], axis=1).ravel()
    return pos, flags, states


def remove_nodes(mesh, pos, flags, params):
    """`Mesh::removeNodes` (`Mesh.cpp:928-1017`): of two nodes closer than gamma h (half that
    on the free surface), one is deleted, never a bound node.  Returns the keep mask over the
    nodes of `mesh` (nodes appended after it are kept)."""
    N = mesh.n_nodes
    ip, ix = neighbours(mesh)
    bound = (flags[:N] & M.BOUND) != 0
    fs = (flags[:N] & M.FREE_SURFACE) != 0
    free = mesh.is_free()
    limit = params.gamma * params.hchar
    rows = np.repeat(np.arange(N), np.diff(ip))
    dist = np.linalg.norm(pos[:, rows] - pos[:, ix], axis=0)
    close = dist <= np.where(fs[rows] & fs[ix], 0.5, 1.0) * limit
    touched = np.zeros(N, bool)
    delete = np.zeros(N, bool)
    for i in np.unique(rows[close]):   # only nodes with a too-close neighbour can change anything
        if delete[i] or free[i]:
            continue
        for k in range(ip[i], ip[i + 1]):
            j = ix[k]
            if close[k]:
                if touched[j]:
                    if bound[i] or (fs[i] and not fs[j]):
                        continue
                    delete[i] = True
                else:
                    if bound[j] or (fs[j] and not fs[i]):
                        continue
                    touched[i] = True
                    delete[j] = True
    return ~delete


def check_bounding_box(pos, bbox, dim):
    """`Mesh::checkBoundingBox` (`Mesh.cpp:149-207`): keep mask of the nodes inside
    [xmin, ymin(, zmin)] x [xmax, ymax(, zmax)]."""
    if bbox is None:
        return np.ones(pos.shape[1], bool)
    lo = np.asarray(bbox[:dim])[:, None]
    hi = np.asarray(bbox[dim:])[:, None]
    return ((pos >= lo) & (pos <= hi)).all(axis=0)


def remesh_map(mesh, params: RemeshParams):
    """One `Mesh::remesh` of `mesh` (positions already moved) without the states: returns the new
    HostMesh and, per new node, the old nodes its states come from, (n_new, dim + 1) int32 padded
    with -1: one old node for a node that survived, the element's dim + 1 nodes for a node added
    at a centroid (their mean, `Mesh.cpp:59-67`).  `pfg_upload_mesh_remap` applies it on the
    device; `apply_origin` on the host."""
    d = mesh.dim
    N = mesh.n_nodes
    pos = mesh.pos.copy()
    if params.laplacian_smoothing_boundaries:
        laplacian_smoothing_boundaries(mesh, pos)
    ident = np.full((N, d + 1), -1, np.int32)
    ident[:, 0] = np.arange(N)
    # add_nodes with the "state" of a node being its own index row
    pos2, flags, _ = add_nodes(mesh, pos, np.zeros(N), params)
    n_add = pos2.shape[1] - N
    origin = ident
    if n_add:
        X = pos[:, mesh.conn]
        J = X[:, 1:, :] - X[:, :1, :]
        size = np.linalg.det(np.moveaxis(J, 2, 0)) * (0.5 if d == 2 else 1.0 / 6.0)
        fs = (mesh.flags & M.FREE_SURFACE) != 0
        grow = size > params.omega * params.hchar ** d
        if not params.add_on_fs:
            grow &= ~fs[mesh.conn].any(axis=0)
        sel = np.nonzero(grow)[0]
        assert sel.size == n_add
        origin = np.concatenate([ident, mesh.conn[:, sel].T.astype(np.int32)])
    keep = np.ones(pos2.shape[1], bool)
    keep[:N] = remove_nodes(mesh, pos2, flags, params)
    keep &= check_bounding_box(pos2, params.bounding_box, d)
    idx = np.nonzero(keep)[0]
    new = M.alpha_shape(pos2[:, idx], flags[idx], params.hchar, params.alpha,
                        delete_flying_nodes=params.delete_flying_nodes)
    return new, np.ascontiguousarray(origin[idx][new.node_origin])


def apply_origin(states, origin, n_old):
    """Field-major states of the new nodes from an origin table of `remesh_map`: a copy for one
    source, the mean in source order for dim + 1 sources (as numpy's mean in `add_nodes`)."""
    S = np.asarray(states, float).reshape(-1, n_old)
    single = origin[:, 1] < 0
    out = np.empty((S.shape[0], origin.shape[0]))
    out[:, single] = S[:, origin[single, 0]]
    multi = ~single
    if multi.any():
        out[:, multi] = S[:, origin[multi]].mean(axis=2)
    return out.ravel()


def remesh(mesh, states, params: RemeshParams):
    """One `Mesh::remesh` of `mesh` (positions already moved) carrying the field-major node
    `states` along.  Returns (new HostMesh, new states)."""
    d = mesh.dim
    N = mesh.n_nodes
    nf = len(states) // N
    pos = mesh.pos.copy()
    if params.laplacian_smoothing_boundaries:
        laplacian_smoothing_boundaries(mesh, pos)
    pos, flags, st = add_nodes(mesh, pos, states, params)
    keep = np.ones(pos.shape[1], bool)
    keep[:N] = remove_nodes(mesh, pos, flags, params)
    keep &= check_bounding_box(pos, params.bounding_box, d)
    idx = np.nonzero(keep)[0]
    pos, flags = pos[:, idx], flags[idx]
    st = st.reshape(nf, -1)[:, idx]
    new = M.alpha_shape(pos, flags, params.hchar, params.alpha, delete_flying_nodes=params.delete_flying_nodes)
    st = st[:, new.node_origin].ravel()
    return new, np.ascontiguousarray(st)
