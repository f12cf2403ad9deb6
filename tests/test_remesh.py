"""Host remeshing (Mesh::remesh restated in pfem_gb300/remesh.py): node addition, removal,
bounding box, boundary smoothing and the state remap through node_origin.  CPU only."""
import numpy as np

from pfem_gb300 import mesh as M
from pfem_gb300 import remesh as R


def _square_mesh():
    # four bound corners and one interior node: 4 triangles
    pos = np.array([[0.0, 1.0, 1.0, 0.0, 0.5], [0.0, 0.0, 1.0, 1.0, 0.5]])
    flags = np.array([M.BOUND] * 4 + [0], np.uint8)
    conn = np.array([[0, 1, 2, 3], [1, 2, 3, 0], [4, 4, 4, 4]], np.int32)
    return M.HostMesh(2, pos, flags, conn, hchar=1.0)


def test_add_nodes_centroid_and_mean_state():
    m = _square_mesh()
    st = np.arange(3 * 5, dtype=float)
    prm = R.RemeshParams(hchar=1.0, omega=0.2)           # every triangle (area 1/4) is too big
    pos, flags, st2 = R.add_nodes(m, m.pos.copy(), st, prm)
    assert pos.shape[1] == 9 and flags[5:].tolist() == [0, 0, 0, 0]
    assert np.allclose(pos[:, 5], m.pos[:, m.conn[:, 0]].mean(axis=1))
    S = st.reshape(3, 5)
    assert np.allclose(st2.reshape(3, 9)[:, 5], S[:, m.conn[:, 0]].mean(axis=1))


def test_add_nodes_skips_free_surface_unless_asked():
    m = _square_mesh()
    m.flags[4] |= M.FREE_SURFACE
    st = np.zeros(15)
    pos, _, _ = R.add_nodes(m, m.pos.copy(), st, R.RemeshParams(hchar=1.0, omega=0.2, add_on_fs=False))
    assert pos.shape[1] == 5
    pos, _, _ = R.add_nodes(m, m.pos.copy(), st, R.RemeshParams(hchar=1.0, omega=0.2, add_on_fs=True))
    assert pos.shape[1] == 9


def test_remove_nodes_keeps_bound_nodes():
    m = _square_mesh()
    m.pos[:, 4] = [0.05, 0.05]                           # interior node next to a bound corner
    keep = R.remove_nodes(m, m.pos, m.flags, R.RemeshParams(hchar=1.0, gamma=0.2))
    assert keep.tolist() == [True, True, True, True, False]


def test_bounding_box():
    pos = np.array([[0.0, 2.0, -1.0], [0.0, 0.5, 0.5]])
    assert R.check_bounding_box(pos, (-0.5, -0.5, 1.5, 1.5), 2).tolist() == [True, False, False]


def test_laplacian_smoothing_moves_interior_node_off_the_wall():
    m = _square_mesh()
    m.pos[:, 4] = [0.5, 0.1]                             # within h/3 of the bottom wall
    pos = m.pos.copy()
    R.laplacian_smoothing_boundaries(m, pos)
    assert np.allclose(pos[:, 4], m.pos[:, :4].mean(axis=1))


def test_remesh_carries_states_with_nodes():
    m = M.dam_break_2d(0.1)
    q = M.incomp_initial_states(m)
    rng = np.random.default_rng(0)
    m.pos[:, ~((m.flags & M.BOUND) != 0)] += rng.uniform(-0.01, 0.01, (2, int((~((m.flags & M.BOUND) != 0)).sum())))
    new, q2 = R.remesh(m, q, R.RemeshParams(hchar=0.1, bounding_box=(-0.01, -1, 4.01, 100)))
    assert len(q2) == 3 * new.n_nodes
    # every kept node carries its own pressure: match nodes by position
    key = {tuple(np.round(m.pos[:, i], 12)): i for i in range(m.n_nodes)}
    N2 = new.n_nodes
    for j in range(N2):
        i = key.get(tuple(np.round(new.pos[:, j], 12)))
        if i is not None:
            assert q2[2 * N2 + j] == q[2 * m.n_nodes + i]
    assert new.n_elems > 0 and not new.is_free()[(new.flags & M.BOUND) == 0].any()


def test_remesh_map_reproduces_the_host_remap():
    """`remesh_map` + `apply_origin` (the table `pfg_upload_mesh_remap` applies on the device)
    give the host remap's mesh and states bitwise, added centroid nodes included."""
    mesh = M.dam_break_2d(0.1)
    rng = np.random.default_rng(7)
    prm = R.RemeshParams(hchar=0.1, omega=0.7, gamma=0.2, bounding_box=(-0.01, -1.0, 4.01, 100.0))
    cur = mesh.copy()
    cur.pos = mesh.pos + 0.02 * rng.standard_normal(mesh.pos.shape) * ((mesh.flags & M.BOUND) == 0)
    states = rng.standard_normal(4 * mesh.n_nodes)  # three flow fields and a temperature
    new, st = R.remesh(cur, states, prm)
    new2, origin = R.remesh_map(cur, prm)
    assert np.array_equal(new.conn, new2.conn) and np.array_equal(new.pos, new2.pos)
    assert origin.shape == (new.n_nodes, 3) and (origin[:, 1] >= 0).any()
    assert np.array_equal(R.apply_origin(states, origin, mesh.n_nodes), st)


def test_flux_at_gauss_points_uses_reference_positions():
    from pfem_gb300 import heat as H

    mesh = M.dam_break_2d(0.1)
    q = H.flux_at_gauss_points(mesh.pos, mesh.facets, lambda x, t: np.array([x[0] + t, 2 * x[1]]), 0.5)
    xs = H.facet_gauss_positions(mesh.pos, mesh.facets)
    assert q.shape == (mesh.facets.shape[1], 3, 2)
    assert np.allclose(q[..., 0], xs[..., 0] + 0.5) and np.allclose(q[..., 1], 2 * xs[..., 1])
    # 2D: the middle point sits on the facet's first node (half-edge Jacobian on [-1, 1])
    assert np.array_equal(xs[:, 1, :], mesh.pos[:, mesh.facets[0]].T)
