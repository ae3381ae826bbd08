"""Ansatz spaces known to the GB300 kernels.

``fem_iso_line_quad_brick`` marks the isoparametric Lagrange space of AutoPDEx
(spaces.py:302-12190); the kernels implement its Q1 members: 2-node lines, 4-node quads
and 8-node bricks, with the physical-gradient rule of its custom JVP
(spaces.py:12162-12190).  Calling it evaluates the Q1 interpolation on the host.
"""
import numpy as np

_SIGNS = {
    1: np.array([[-1.0], [1.0]]),
    2: np.array([[-1.0, -1.0], [1.0, -1.0], [1.0, 1.0], [-1.0, 1.0]]),
    3: np.array([[-1.0, -1.0, -1.0], [1.0, -1.0, -1.0], [1.0, 1.0, -1.0], [-1.0, 1.0, -1.0],
                 [-1.0, -1.0, 1.0], [1.0, -1.0, 1.0], [1.0, 1.0, 1.0], [-1.0, 1.0, 1.0]]),
}


def q1_shape_functions(xi, n_dim):
    """N_a(xi) of the Q1 element of dimension ``n_dim`` in AutoPDEx's node order."""
    s = _SIGNS[n_dim]
    xi = np.atleast_1d(np.asarray(xi, dtype=np.float64))
    return np.prod((1 + s * xi[None, :]) / 2, axis=1)


def fem_iso_line_quad_brick(x, xI, fI, settings, overwrite_diff, n_dim):
    """Q1 interpolation sum_a N_a(x) fI[a] at the reference point ``x`` (host only)."""
    xI = np.asarray(xI)
    if xI.shape[0] != 2 ** n_dim:
        raise NotImplementedError("the gb300 backend implements the Q1 members of this space")
    return np.tensordot(q1_shape_functions(x, n_dim), np.asarray(fI, dtype=np.float64), axes=(0, 0))


def simplex_shape_functions(xi, n_dim, n_nodes):
    """N_a(xi) of the simplex members of fem_iso_line_tri_tet (spaces.py:12193): linear and
    quadratic triangles (corners, then mid-sides 0-1, 1-2, 2-0) and tetrahedra (corners, then
    edges 0-1, 1-2, 0-2, 0-3, 1-3, 2-3)."""
    xi = np.asarray(xi, dtype=np.float64)
    if n_dim == 2 and n_nodes == 3:
        return np.array([1 - xi[0] - xi[1], xi[0], xi[1]])
    if n_dim == 2 and n_nodes == 6:
        L = np.array([1 - xi[0] - xi[1], xi[0], xi[1]])
        return np.array([L[0] * (2 * L[0] - 1), L[1] * (2 * L[1] - 1), L[2] * (2 * L[2] - 1),
                         4 * L[0] * L[1], 4 * L[1] * L[2], 4 * L[2] * L[0]])
    if n_dim == 3 and n_nodes == 4:
        return np.array([1 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]])
    if n_dim == 3 and n_nodes == 10:  # corners, then edges 0-1, 1-2, 0-2, 0-3, 1-3, 2-3
        L = np.array([1 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]])
        edges = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
        return np.concatenate([L * (2 * L - 1), [4 * L[i] * L[j] for i, j in edges]])
    raise NotImplementedError("the gb300 backend implements 3- and 6-node triangles and 4- and 10-node tetrahedra")


def fem_iso_line_tri_tet(x, xI, fI, settings, overwrite_diff, n_dim):
    """Simplex interpolation sum_a N_a(x) fI[a] at the reference point ``x`` (host only); the
    kernels implement the 3- and 6-node triangles and the 4- and 10-node tetrahedra."""
    N = simplex_shape_functions(x, n_dim, np.asarray(xI).shape[0])
    return np.tensordot(N, np.asarray(fI, dtype=np.float64), axes=(0, 0))
