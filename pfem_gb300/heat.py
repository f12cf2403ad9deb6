"""Host helpers of the heat equation (problems "Conduction" and "Boussinesq").

The library takes the heat boundary conditions as arrays (`Context.heat_set_bc`,
`Context.heat_set_flux`); the reference evaluates its Lua BC functions at the node positions
(Dirichlet "T", `HeatEquation.inl:384-389`) and at the facet Gauss points (flux "Q",
`HeatEquation.inl:78-88` through `MatrixBuilder::getQN`, `MatricesBuilder.inl:246-272`).  These
helpers give the caller the same evaluation points.
"""
from __future__ import annotations

import numpy as np

# three-point facet rule of the heat equation (nGPLD = 3, HeatEquation.inl:13-22), the points of
# Mesh::getGaussPoints(dim - 1, 3) (Mesh.cpp:342-413)
_GP_1D = np.array([[-np.sqrt(3.0 / 5.0), 0.0], [0.0, 0.0], [np.sqrt(3.0 / 5.0), 0.0]])
_GP_2D = np.array([[1.0 / 6.0, 1.0 / 6.0], [1.0 / 6.0, 2.0 / 3.0], [2.0 / 3.0, 1.0 / 6.0]])


def facet_gauss_positions(pos, facets):
    """Facet::getPosFromGP (Facet.cpp:227-237) at the three heat Gauss points of every facet.

    pos: (dim, N) node positions; facets: (dim, F) facet nodes.  Returns (F, 3, dim):
    x = J xi + x_0 with J the facet Jacobian of Facet::computeJ (Facet.cpp:15-58).  In 2D the
    Jacobian is half the edge while the points lie in [-1, 1], so, as in the reference, the
    points are centred on the facet's first node rather than on its midpoint."""
    pos = np.asarray(pos, np.float64)
    facets = np.asarray(facets, np.int64)
    dim = pos.shape[0]
    x0 = pos[:, facets[0]].T                                    # (F, dim)
    if dim == 2:
        j0 = (pos[:, facets[1]].T - x0) / 2
        return x0[:, None, :] + _GP_1D[None, :, 0, None] * j0[:, None, :]
    j0 = pos[:, facets[1]].T - x0
    j1 = pos[:, facets[2]].T - x0
    return x0[:, None, :] + _GP_2D[None, :, 0, None] * j0[:, None, :] + _GP_2D[None, :, 1, None] * j1[:, None, :]


def flux_at_gauss_points(pos, facets, q, t):
    """Evaluate a flux function q(x, t) -> (dim,) at every facet Gauss point: (F, 3, dim)."""
    xs = facet_gauss_positions(pos, facets)
    out = np.empty_like(xs)
    for f in range(xs.shape[0]):
        for g in range(3):
            out[f, g] = q(xs[f, g], t)
    return out
