"""The C++ host remesh (include/pfem_remesh.h, libpfemremesh.so) against the Python host remesh.

* Alpha shape of the initial node clouds (2D and 3D dam breaks, the sloshing tank), both
  triangulating the same perturbed points: the same elements, facets, flags and node origins.
* One remesh of a moved mesh: positions, flags and state origins bit for bit (the smoothing,
  node addition and removal run the same arithmetic); elements equal except where Qhull's
  triangulation is not exactly Delaunay, which an exact in-sphere test shows.
* A square lattice (every cell co-circular) without perturbation: exact predicates give a
  triangulation with two positive triangles per cell and no lattice point inside any
  circumcircle (integer arithmetic).
* Errors: bad parameters and out-of-range connectivity return error codes with a message.
"""
import ctypes as C
from fractions import Fraction

import numpy as np
import pytest

from pfem_gb300 import build
from pfem_gb300 import mesh as M
from pfem_gb300 import remesh as R


@pytest.fixture(scope="module", autouse=True)
def lib():
    build.build_remesh()
    return R.native_lib()


def canon_elems(m):
    return set(map(tuple, np.sort(m.conn, axis=0).T.tolist()))


def canon_facets(m):
    return set(zip(map(tuple, np.sort(m.facets, axis=0).T.tolist()), m.facet_out.tolist()))


def same_mesh(a, b):
    assert a.n_nodes == b.n_nodes
    assert np.array_equal(a.pos, b.pos)
    assert np.array_equal(a.flags, b.flags)
    assert np.array_equal(a.node_origin, b.node_origin)
    assert canon_elems(a) == canon_elems(b)
    assert canon_facets(a) == canon_facets(b)


def positive(m):
    X = m.pos[:, m.conn]
    J = X[:, 1:, :] - X[:, :1, :]
    return np.linalg.det(np.moveaxis(J, 2, 0)).min() > 0


CLOUDS = {
    "dam 2d h0.05": lambda: (M.dam_break_nodes_2d(0.05), 0.05),
    "dam 2d h0.02": lambda: (M.dam_break_nodes_2d(0.02), 0.02),
    "sloshing 2d": lambda: (M.sloshing_nodes_2d(0.02), 0.02),
    "dam 3d h0.05": lambda: (M.dam_break_nodes_3d(0.05, tank=(0.6, 0.3, 0.5), column=(0.2, 0.3, 0.3)), 0.05),
    "dam 3d h0.03": lambda: (M.dam_break_nodes_3d(0.03, tank=(0.6, 0.3, 0.5), column=(0.2, 0.3, 0.3)), 0.03),
}


@pytest.mark.parametrize("case", sorted(CLOUDS))
def test_alpha_shape_equals_python(case):
    (pos, flags), h = CLOUDS[case]()
    dim = pos.shape[0]
    jit = lambda n: R.jitter_field(n, dim, 1e-6 * h)  # noqa: E731
    py = M.alpha_shape(pos, flags, h, 1.2, True, jitter=jit)
    cc = R.alpha_shape_native(pos, flags, h, 1.2, True, jitter=1e-6)
    same_mesh(py, cc)
    assert positive(cc)
    # every facet node belongs to its element, and the opposite node is the element's other node
    for f in range(cc.facets.shape[1]):
        el = set(cc.conn[:, cc.facet_elm[f]].tolist())
        assert set(cc.facets[:, f].tolist()) | {int(cc.facet_out[f])} == el


def _insphere_exact(P, t, q):
    """Sign of the in-sphere determinant of point q against simplex t (rows of P), with the
    orientation folded in: > 0 when q is strictly inside the circumsphere."""
    pts = [[Fraction(float(x)) for x in P[i]] for i in t]
    qq = [Fraction(float(x)) for x in P[q]]
    d = len(qq)
    A = [[p[c] - pts[0][c] for c in range(d)] for p in pts[1:]]

    def det(m):
        if len(m) == 1:
            return m[0][0]
        return sum((-1) ** j * m[0][j] * det([r[:j] + r[j + 1:] for r in m[1:]]) for j in range(len(m)))

    o = det(A)
    rows = [[p[c] - qq[c] for c in range(d)] + [sum((p[c] - qq[c]) ** 2 for c in range(d))] for p in pts]
    s = det(rows)
    # det[[p_k - q, |p_k - q|^2]] has the sign (-1)^d of "inside" for a positive simplex
    return s * o * (1 if d == 2 else -1)


@pytest.mark.parametrize("dim", [2, 3])
def test_remesh_map_equals_python(dim):
    if dim == 2:
        h = 0.03
        m = M.dam_break_2d(h)
    else:
        h = 0.04
        m = M.dam_break_3d(h, tank=(0.8, 0.4, 0.6), column=(0.3, 0.4, 0.4))
    rng = np.random.default_rng(5)
    free = (m.flags & M.BOUND) == 0
    m.pos = m.pos + rng.uniform(-0.3, 0.3, m.pos.shape) * h * free
    prm = R.RemeshParams(hchar=h, omega=0.5, gamma=0.3)
    amp = 1e-6 * h
    a, oa = R.remesh_map(m, prm, jitter=lambda n: R.jitter_field(n, dim, amp))
    prm.native = True
    b, ob = R.remesh_map_native(m, prm, jitter=1e-6)
    assert a.n_nodes == b.n_nodes
    assert np.array_equal(a.pos, b.pos)
    assert np.array_equal(a.flags, b.flags)
    assert np.array_equal(oa, ob)
    assert positive(b)
    ea, eb = canon_elems(a), canon_elems(b)
    diff_a, diff_b = ea - eb, eb - ea
    assert len(diff_a) + len(diff_b) <= 1e-3 * len(ea)
    if diff_a:
        # where they differ, Qhull's simplex has a node of the C++ simplex on or inside its
        # circumsphere in the perturbed points; the C++ simplices have none inside
        jt = R.jitter_field(int(b.node_origin.max()) + 1, dim, amp)
        Q = (b.pos + jt[:, b.node_origin]).T
        nodes_b = {n for t in diff_b for n in t}
        for t in diff_a:
            assert any(_insphere_exact(Q, t, q) >= 0 for q in nodes_b - set(t)), t
        nodes_a = {n for t in diff_a for n in t}
        for t in diff_b:
            assert all(_insphere_exact(Q, t, q) <= 0 for q in nodes_a - set(t)), t


def test_square_lattice_without_perturbation():
    n = 12
    gx, gy = np.meshgrid(np.arange(n + 1, dtype=float), np.arange(n + 1, dtype=float), indexing="ij")
    pos = np.stack([gx.ravel(), gy.ravel()])
    flags = np.zeros(pos.shape[1], np.uint8)
    m = R.alpha_shape_native(pos, flags, 1.0, alpha=10.0, delete_flying_nodes=False, jitter=0.0)
    assert m.n_elems == 2 * n * n
    assert positive(m)
    P = [(int(x), int(y)) for x, y in pos.T]
    for e in range(m.n_elems):
        (ax, ay), (bx, by), (cx, cy) = (P[i] for i in m.conn[:, e])
        for (dx, dy) in P:
            rows = [(ax - dx, ay - dy), (bx - dx, by - dy), (cx - dx, cy - dy)]
            L = [x * x + y * y for x, y in rows]
            det = sum(L[k] * (rows[(k + 1) % 3][0] * rows[(k + 2) % 3][1] - rows[(k + 1) % 3][1] * rows[(k + 2) % 3][0])
                      for k in range(3))
            assert det <= 0


def test_errors(lib):
    p = R._PfrParams()
    assert lib.pfr_default_params(4, 0.1, C.byref(p)) != 0
    assert lib.pfr_default_params(2, -1.0, C.byref(p)) != 0
    assert lib.pfr_default_params(2, 0.1, C.byref(p)) == 0 and p.alpha == 1.2 and p.jitter == 0.0
    pos = np.zeros((2, 3))
    pos[0, 1] = pos[1, 2] = 1.0
    flags = np.zeros(3, np.uint8)
    conn = np.array([[0], [1], [5]], np.int32)
    h = C.c_void_p()
    rc = lib.pfr_remesh(C.byref(p), 3, pos.ctypes.data_as(C.POINTER(C.c_double)),
                        flags.ctypes.data_as(C.POINTER(C.c_uint8)), 1, conn.ctypes.data_as(C.POINTER(C.c_int32)),
                        C.byref(h))
    assert rc == -1 and not h.value
    assert b"out of range" in lib.pfr_last_error()
    p.hchar = 0.0
    assert lib.pfr_alpha_shape(C.byref(p), 3, pos.ctypes.data_as(C.POINTER(C.c_double)),
                               flags.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(h)) == -1


def test_cells_equal_one_triangulation():
    """A 3D cloud above the cell threshold (50k nodes) triangulated in cells on several threads
    gives the simplices, facets, flags and node origins of one triangulation, fresh and moved."""
    h = (0.25 / 3e4) ** (1 / 3)
    pos, flags = M.dam_break_nodes_3d(h, seed=1)
    assert pos.shape[1] >= 16384
    rng = np.random.default_rng(3)
    for p in (pos, pos + rng.uniform(-0.3, 0.3, pos.shape) * h * ((flags & M.BOUND) == 0)):
        one = R.alpha_shape_native(p, flags, h, 1.2, True, single=True)
        cells = R.alpha_shape_native(p, flags, h, 1.2, True)
        assert canon_elems(one) == canon_elems(cells)
        assert canon_facets(one) == canon_facets(cells)
        assert np.array_equal(one.flags, cells.flags) and np.array_equal(one.node_origin, cells.node_origin)
        assert positive(cells)
