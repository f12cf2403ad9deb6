"""Generate the known-answer fixtures in tests/golden/.

The reference ships no tests or golden vectors, so the fixtures here are derived
independently from closed forms of the P1 element integrals (not from the oracle):

* kat_elements.npz: for one right triangle and one right tetrahedron, the PSPG element
  matrix Ae and vector be of m_buildAbPSPG (MomContEquationPSPG.inl:26-53) written out from
  the exact integrals of linear shape functions:
      int N_i N_j   = |e| (1 + d_ij) / ((d+1)(d+2))
      int N_i       = |e| / (d+1)
      strain-rate energy with Ddev = diag(2,..,2,1,..,1) -> mu |e| [d_f1f2 gradN_i.gradN_j
                                                               + dN_i/dx_f2 dN_j/dx_f1]
  and tau of m_computeTauPSPG (:237-259).  Rerun with `python tests/golden/make_golden.py`.
"""
import os

import numpy as np

OUT = os.path.dirname(os.path.abspath(__file__))


def p1_element(X, rho, mu, dt, g, v_iter, v_prev):
    """X: (d+1, d) node coordinates.  v_iter/v_prev: (d+1, d) nodal velocities."""
    d = X.shape[1]
    npe = d + 1
    J = (X[1:] - X[0]).T                      # columns x_i - x_0
    detJ = np.linalg.det(J)
    ref = 0.5 if d == 2 else 1.0 / 6.0
    vol = detJ * ref
    invJ = np.linalg.inv(J)
    Gref = np.hstack([-np.ones((d, 1)), np.eye(d)])  # dN/dxi
    G = invJ.T @ Gref                          # (d, npe): dN_i/dx_f
    M = rho * vol * (np.ones((npe, npe)) + np.eye(npe)) / ((d + 1) * (d + 2))
    s = np.full(npe, 1.0 / (d + 1))
    nv = d * npe
    K = np.zeros((nv, nv))
    for i in range(npe):
        for j in range(npe):
            dot = G[:, i] @ G[:, j]
            for f1 in range(d):
                for f2 in range(d):
                    K[f1 * npe + i, f2 * npe + j] = mu * vol * ((f1 == f2) * dot + G[f2, i] * G[f1, j])
    D = np.zeros((npe, nv))
    C = np.zeros((npe, nv))
    for i in range(npe):
        for j in range(npe):
            for f in range(d):
                D[i, f * npe + j] = vol * s[i] * G[f, j]
                C[i, f * npe + j] = vol * G[f, i] * s[j]
    L = vol / rho * G.T @ G
    F = np.array([rho * vol * g[f] * s[i] for f in range(d) for i in range(npe)])
    H = vol * (G.T @ np.asarray(g[:d]))
    h = np.sqrt(ref * detJ / np.pi)
    U = np.mean(np.linalg.norm(v_iter, axis=1))
    tau = 1 / np.sqrt((2 / dt) ** 2 + (2 * U / h) ** 2 + 9 * (4 * mu / (h * h * rho)) ** 2)
    Mb = np.kron(np.eye(d), M / dt)
    Ae = np.block([[Mb + K, -D.T], [tau / dt * C + D, tau * L]])
    vp = v_prev.T.reshape(-1)                  # field-major element vector
    be = np.concatenate([F + Mb @ vp, tau * H + tau / dt * C @ vp])
    return Ae, be, detJ, tau


def main():
    rng = np.random.default_rng(7)
    cases = {}
    params = dict(rho=1000.0, mu=1e-3, dt=1e-3)
    g2 = np.array([0.0, -9.81, 0.0])
    tri = np.array([[0.0, 0.0], [0.05, 0.0], [0.0, 0.05]])
    tri_skew = np.array([[0.1, 0.2], [0.16, 0.21], [0.12, 0.27]])
    tet = np.array([[0.0, 0.0, 0.0], [0.01, 0.0, 0.0], [0.0, 0.01, 0.0], [0.0, 0.0, 0.01]])
    tet_skew = np.array([[0.3, 0.1, 0.2], [0.312, 0.101, 0.198], [0.303, 0.113, 0.2], [0.301, 0.104, 0.211]])
    g3 = np.array([0.0, 0.0, -9.81])
    for name, X, g in (("tri", tri, g2), ("tri_skew", tri_skew, g2), ("tet", tet, g3), ("tet_skew", tet_skew, g3)):
        d = X.shape[1]
        vi = rng.uniform(-1, 1, size=(d + 1, d))
        vp = rng.uniform(-1, 1, size=(d + 1, d))
        Ae, be, detJ, tau = p1_element(X, params["rho"], params["mu"], params["dt"], g, vi, vp)
        cases[f"{name}_X"] = X
        cases[f"{name}_viter"] = vi
        cases[f"{name}_vprev"] = vp
        cases[f"{name}_Ae"] = Ae
        cases[f"{name}_be"] = be
        cases[f"{name}_detJ"] = np.array(detJ)
        cases[f"{name}_tau"] = np.array(tau)
    cases["params"] = np.array([params["rho"], params["mu"], params["dt"]])
    np.savez_compressed(os.path.join(OUT, "kat_elements.npz"), **cases)
    print("wrote", os.path.join(OUT, "kat_elements.npz"))


if __name__ == "__main__":
    main()
