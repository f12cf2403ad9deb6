"""Output on the host (pfem_gb300/output.py): the writable quantities of the reference's
problems and the GMSH file layout (MSH 2.2 ASCII), read back.  CPU only."""
import numpy as np

from pfem_gb300 import api
from pfem_gb300 import mesh as M
from pfem_gb300 import output as OUT


def _read_msh(path):
    lines = open(path).read().split("\n")
    out, i = {"data": {}}, 0
    while i < len(lines):
        tag = lines[i]
        if tag == "$Nodes":
            n = int(lines[i + 1])
            out["nodes"] = np.array([[float(x) for x in lines[i + 2 + k].split()[1:]] for k in range(n)])
            i += n + 2
        elif tag == "$Elements":
            n = int(lines[i + 1])
            out["elements"] = [list(map(int, lines[i + 2 + k].split())) for k in range(n)]
            i += n + 2
        elif tag == "$NodeData":
            name = lines[i + 2].strip('"')
            nc, n = int(lines[i + 7]), int(lines[i + 8])
            out["data"][name] = np.array([[float(x) for x in lines[i + 9 + k].split()[1:]] for k in range(n)])
            assert out["data"][name].shape == (n, nc)
            i += n + 9
        else:
            i += 1
    return out


def test_writable_data_incompressible_and_wc():
    m = M.dam_break_2d(0.1)
    N = m.n_nodes
    rng = np.random.default_rng(0)
    q = rng.normal(size=3 * N)
    d = OUT.writable_data(api.KIND_INCOMP_PSPG, 2, q, N)
    assert np.allclose(d["ke"][:, 0], 0.5 * (q[:N] ** 2 + q[N:2 * N] ** 2))
    assert np.allclose(d["velocity"][:, 2], 0) and np.allclose(d["p"][:, 0], q[2 * N:])
    w = rng.normal(size=6 * N)
    d = OUT.writable_data(api.KIND_WC_CDS_DPDT, 2, w, N)
    assert np.allclose(d["rho"][:, 0], w[3 * N:4 * N]) and np.allclose(d["ay"][:, 0], w[5 * N:])


def test_write_msh_round_trip(tmp_path):
    m = M.dam_break_2d(0.1)
    N, E = m.n_nodes, m.n_elems
    q = M.incomp_initial_states(m)
    path = str(tmp_path / "out.msh")
    OUT.write_msh(path, m, m.pos, q, api.KIND_INCOMP_PSPG, 0.25, step=7, what=("p", "velocity"))
    r = _read_msh(path)
    assert np.allclose(r["nodes"][:, :2], m.pos.T) and np.allclose(r["nodes"][:, 2], 0)
    tris = [e for e in r["elements"] if e[1] == 2]
    pts = [e for e in r["elements"] if e[1] == 15]
    assert len(tris) == E and len(pts) == N
    assert np.array_equal(np.array([t[-3:] for t in tris]) - 1, m.conn.T)
    assert np.allclose(r["data"]["p"][:, 0], q[2 * N:]) and r["data"]["velocity"].shape == (N, 3)
