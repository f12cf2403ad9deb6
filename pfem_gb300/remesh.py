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

import ctypes as C
import math
import os
import threading
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
    native: bool = False                # remesh_map through the C++ library libpfemremesh.so


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


def qr_basic_solve(A, b):
    """Basic solution of the square system A x = b by Householder QR with column pivoting, the
    way the reference's `colPivHouseholderQr().solve` treats a rank-deficient A (`Mesh.cpp:
    630,681`): the pivots after the remaining columns' squared norms fall below
    (max column norm * eps)^2 (n - k) / n are dropped, their unknowns set to 0, the rest solved by
    back substitution.  Plain scalar arithmetic in a fixed order; `pfem_remesh.cpp` runs the
    same operations."""
    n = len(b)
    A = [list(map(float, r)) for r in A]
    b = list(map(float, b))
    perm = list(range(n))
    norms = []
    for j in range(n):
        s2 = 0.0
        for i in range(n):
            s2 += A[i][j] * A[i][j]
        norms.append(s2)
    mx = 0.0
    for j in range(n):
        mx = max(mx, math.sqrt(norms[j]))
    thresh = (mx * 2.220446049250313e-16) ** 2 / n
    nz = n
    for k in range(n):
        jb = k
        for j in range(k + 1, n):
            if norms[j] > norms[jb]:
                jb = j
        if nz == n and norms[jb] < thresh * (n - k):
            nz = k
        if jb != k:
            for i in range(n):
                A[i][k], A[i][jb] = A[i][jb], A[i][k]
            perm[k], perm[jb] = perm[jb], perm[k]
            norms[k], norms[jb] = norms[jb], norms[k]
        alpha = A[k][k]
        sigma = 0.0
        for i in range(k + 1, n):
            sigma += A[i][k] * A[i][k]
        if sigma != 0.0:
            nrm = math.sqrt(alpha * alpha + sigma)
            beta = -nrm if alpha >= 0 else nrm
            v = [0.0] * n
            v[k] = 1.0
            for i in range(k + 1, n):
                v[i] = A[i][k] / (alpha - beta)
            tau = (beta - alpha) / beta
            for j in range(k + 1, n):
                w = A[k][j]
                for i in range(k + 1, n):
                    w += v[i] * A[i][j]
                w *= tau
                A[k][j] -= w
                for i in range(k + 1, n):
                    A[i][j] -= w * v[i]
            w = b[k]
            for i in range(k + 1, n):
                w += v[i] * b[i]
            w *= tau
            b[k] -= w
            for i in range(k + 1, n):
                b[i] -= w * v[i]
            A[k][k] = beta
            for i in range(k + 1, n):
                A[i][k] = 0.0
        for j in range(k + 1, n):
            s2 = 0.0
            for i in range(k + 1, n):
                s2 += A[i][j] * A[i][j]
            norms[j] = s2
    c = [0.0] * n
    for k in range(nz - 1, -1, -1):
        s2 = b[k]
        for j in range(k + 1, nz):
            s2 -= A[k][j] * c[j]
        c[k] = s2 / A[k][k]
    x = [0.0] * n
    for k in range(nz):
        x[perm[k]] = c[k]
    return x


def laplacian_smoothing_boundaries(mesh, pos):
    """`Mesh::laplacianSmoothingBoundaries` (`Mesh.cpp:580-760`): for every element touching the
    walls with exactly `dim` bound nodes, a non-bound node closer than h/3 to the wall facet is
    pushed h/3 along the facet normal (free-surface node) or moved to the mean of its
    neighbours.  Elements are visited in order and see earlier moves.  Scalar arithmetic in the
    reference's order (the facet plane n.x = -1 by `qr_basic_solve`, sums left to right)."""
    d, h = mesh.dim, mesh.hchar
    bound = (mesh.flags & M.BOUND) != 0
    fs = (mesh.flags & M.FREE_SURFACE) != 0
    ip, ix = neighbours(mesh)
    for e in np.nonzero(bound[mesh.conn].sum(axis=0) == d)[0]:
        nodes = mesh.conn[:, e]
        b = bound[nodes]
        out = int(nodes[~b][0])
        fac = nodes[b]
        P = [[float(pos[c, f]) for c in range(d)] for f in fac]
        x = [float(pos[c, out]) for c in range(d)]
        normal = [0.0] * d
        axis = True
        if d == 2:
            if P[0][0] == P[1][0]:
                normal[0] = 1.0
                dist = abs(P[0][0] - x[0])
            elif P[0][1] == P[1][1]:
                normal[1] = 1.0
                dist = abs(P[0][1] - x[1])
            else:
                axis = False
        else:
            if P[0][0] == P[1][0] and P[1][0] == P[2][0]:
                normal[0] = 1.0
                dist = abs(P[0][0] - x[0])
            elif P[0][1] == P[1][1] and P[1][1] == P[2][1]:
                normal[1] = 1.0
                dist = abs(P[0][1] - x[1])
            elif P[0][2] == P[1][2] and P[1][1] == P[2][2]:  # the reference compares y with z here
                normal[2] = 1.0
                dist = abs(P[0][2] - x[2])
            else:
                axis = False
        if not axis:
            normal = qr_basic_solve(P, [-1.0] * d)
            dot, nn = 0.0, 0.0
            for c in range(d):
                dot += normal[c] * x[c]
                nn += normal[c] * normal[c]
            dist = abs(dot + 1) / math.sqrt(nn)
        if dist > h / 3:
            continue
        if fs[out]:
            if d == 2:  # sign with the raw normal, then normalised (Mesh.cpp:697-715)
                side = normal[0] * (x[0] - P[0][0]) + normal[1] * (x[1] - P[0][1])
                if side < 0:
                    normal = [-normal[0], -normal[1]]
                nn = math.sqrt(normal[0] * normal[0] + normal[1] * normal[1])
                normal = [normal[0] / nn, normal[1] / nn]
            else:  # normalised, then the sign (:716-734)
                nn = math.sqrt(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2])
                normal = [normal[0] / nn, normal[1] / nn, normal[2] / nn]
                side = (x[0] - P[0][0]) * normal[0] + (x[1] - P[0][1]) * normal[1] + (x[2] - P[0][2]) * normal[2]
                if side < 0:
                    normal = [-normal[0], -normal[1], -normal[2]]
            for c in range(d):
                pos[c, out] += h / 3 * normal[c]
        else:
            nb = ix[ip[out]:ip[out + 1]]
            for c in range(d):
                acc = 0.0
                for j in nb:
                    acc += float(pos[c, j])
                pos[c, out] = acc / float(len(nb))


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


def remesh_map(mesh, params: RemeshParams, jitter=None):
    """One `Mesh::remesh` of `mesh` (positions already moved) without the states: returns the new
    HostMesh and, per new node, the old nodes its states come from, (n_new, dim + 1) int32 padded
    with -1: one old node for a node that survived, the element's dim + 1 nodes for a node added
    at a centroid (their mean, `Mesh.cpp:59-67`).  `pfg_upload_mesh_remap` applies it on the
    device; `apply_origin` on the host.  With `params.native` the C++ library computes it
    (`remesh_map_native`); `jitter` is the triangulation's perturbation (see `M.alpha_shape`)."""
    if params.native:
        return remesh_map_native(mesh, params)
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
                        delete_flying_nodes=params.delete_flying_nodes, jitter=jitter)
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


# --------------------------------------------------------------------------------------
# The C++ remesh (include/pfem_remesh.h, pfem_gb300/host/pfem_remesh.cpp)
# --------------------------------------------------------------------------------------

class _PfrParams(C.Structure):
    _fields_ = [("dim", C.c_int32), ("add_on_fs", C.c_int32), ("delete_flying_nodes", C.c_int32),
                ("laplacian_smoothing_boundaries", C.c_int32), ("hchar", C.c_double), ("alpha", C.c_double),
                ("omega", C.c_double), ("gamma", C.c_double), ("jitter", C.c_double),
                ("has_bounding_box", C.c_int32), ("single_triangulation", C.c_int32),
                ("bounding_box", C.c_double * 6)]


REMESH_EXPORTED = ("pfr_default_params", "pfr_remesh", "pfr_alpha_shape", "pfr_mesh_counts", "pfr_mesh_read",
                   "pfr_mesh_free", "pfr_last_error")
_LIB = None
_LIB_LOCK = threading.Lock()


def native_lib():
    """libpfemremesh.so, built by `build.build_remesh` (raises when it is missing)."""
    global _LIB
    with _LIB_LOCK:
        if _LIB is None:
            path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libpfemremesh.so")
            if not os.path.exists(path):
                raise RuntimeError(f"{path} is missing: run pfem_gb300.build.build_remesh()")
            L = C.CDLL(path)
            vp, dp, u8p, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_uint8), C.POINTER(C.c_int32)
            L.pfr_default_params.argtypes = [C.c_int32, C.c_double, C.POINTER(_PfrParams)]
            L.pfr_remesh.argtypes = [C.POINTER(_PfrParams), C.c_int32, dp, u8p, C.c_int32, ip, C.POINTER(vp)]
            L.pfr_alpha_shape.argtypes = [C.POINTER(_PfrParams), C.c_int32, dp, u8p, C.POINTER(vp)]
            L.pfr_mesh_counts.argtypes = [vp, ip, ip, ip]
            L.pfr_mesh_read.argtypes = [vp, dp, u8p, ip, ip, ip, ip, ip]
            L.pfr_mesh_free.argtypes = [vp]
            L.pfr_mesh_free.restype = None
            L.pfr_last_error.restype = C.c_char_p
            _LIB = L
        return _LIB


def jitter_field(n, dim, amplitude):
    """The perturbation the C++ triangulation applies, (dim, n): coordinate c of node i moves by
    amplitude * (2 u - 1), u = the top 53 bits of SplitMix64's output function applied to
    (i dim + c + 1) * 0x9E3779B97F4A7C15 (mod 2^64), over 2^53."""
    k = np.arange(n * dim, dtype=np.uint64) + np.uint64(1)
    z = k * np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    u = 2.0 * (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53 - 1.0
    return np.ascontiguousarray((u * amplitude).reshape(n, dim).T)


def _native_params(dim, params: RemeshParams, jitter=None):
    p = _PfrParams()
    L = native_lib()
    if L.pfr_default_params(dim, float(params.hchar), C.byref(p)) != 0:
        raise ValueError("bad remesh parameters")
    p.add_on_fs = int(params.add_on_fs)
    p.delete_flying_nodes = int(params.delete_flying_nodes)
    p.laplacian_smoothing_boundaries = int(params.laplacian_smoothing_boundaries)
    p.alpha, p.omega, p.gamma = float(params.alpha), float(params.omega), float(params.gamma)
    if jitter is not None:
        p.jitter = float(jitter)
    if params.bounding_box is not None:
        p.has_bounding_box = 1
        for i, v in enumerate(params.bounding_box):
            p.bounding_box[i] = float(v)
    return p


def _read_native(h, dim, hchar, alpha):
    L = native_lib()
    n, e, f = C.c_int32(), C.c_int32(), C.c_int32()
    L.pfr_mesh_counts(h, C.byref(n), C.byref(e), C.byref(f))
    n, e, f = n.value, e.value, f.value
    pos = np.empty((dim, n))
    flags = np.empty(n, np.uint8)
    conn = np.empty((dim + 1, e), np.int32)
    facets = np.empty((dim, f), np.int32)
    felm = np.empty(f, np.int32)
    fout = np.empty(f, np.int32)
    origin = np.empty((n, dim + 1), np.int32)
    ptr = lambda a, t: a.ctypes.data_as(C.POINTER(t))  # noqa: E731
    L.pfr_mesh_read(h, ptr(pos, C.c_double), ptr(flags, C.c_uint8), ptr(conn, C.c_int32), ptr(facets, C.c_int32),
                    ptr(felm, C.c_int32), ptr(fout, C.c_int32), ptr(origin, C.c_int32))
    L.pfr_mesh_free(h)
    mesh = M.HostMesh(dim, pos, flags, conn, facets, felm, fout, hchar, alpha)
    mesh.node_origin = origin[:, 0].copy()
    return mesh, origin


def alpha_shape_native(pos, flags, hchar, alpha=1.2, delete_flying_nodes=False, jitter=None, single=False):
    """`M.alpha_shape` through the C++ library; `jitter` is its perturbation amplitude relative
    to hchar (default 1e-6 in 3D, 0 in 2D); `single` forces one triangulation (large 3D clouds
    are otherwise triangulated in cells in parallel).  The result carries `node_origin`."""
    dim, n = pos.shape
    prm = RemeshParams(hchar=hchar, alpha=alpha, delete_flying_nodes=delete_flying_nodes)
    p = _native_params(dim, prm, jitter)
    p.single_triangulation = int(single)
    L = native_lib()
    P = np.ascontiguousarray(pos, float)
    F = np.ascontiguousarray(flags, np.uint8)
    h = C.c_void_p()
    rc = L.pfr_alpha_shape(C.byref(p), n, P.ctypes.data_as(C.POINTER(C.c_double)),
                           F.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(h))
    if rc != 0:
        raise RuntimeError(f"pfr_alpha_shape failed ({rc}): {L.pfr_last_error().decode()}")
    return _read_native(h, dim, hchar, alpha)[0]


def remesh_map_native(mesh, params: RemeshParams, jitter=None):
    """`remesh_map` through the C++ library (`pfr_remesh`): the same steps and rules, the
    Delaunay triangulation its own (exact predicates) instead of Qhull."""
    d = mesh.dim
    p = _native_params(d, params, jitter)
    L = native_lib()
    P = np.ascontiguousarray(mesh.pos, float)
    F = np.ascontiguousarray(mesh.flags, np.uint8)
    K = np.ascontiguousarray(mesh.conn, np.int32)
    h = C.c_void_p()
    rc = L.pfr_remesh(C.byref(p), mesh.n_nodes, P.ctypes.data_as(C.POINTER(C.c_double)),
                      F.ctypes.data_as(C.POINTER(C.c_uint8)), mesh.n_elems, K.ctypes.data_as(C.POINTER(C.c_int32)),
                      C.byref(h))
    if rc != 0:
        raise RuntimeError(f"pfr_remesh failed ({rc}): {L.pfr_last_error().decode()}")
    return _read_native(h, d, params.hchar, params.alpha)
