"""Ansatz spaces known to the GB300 kernels.

``fem_iso_line_quad_brick`` marks the isoparametric Lagrange space of AutoPDEx
(spaces.py:302-12190); the kernels implement its 2- and 3-node lines, 4- and 9-node quads
and 8- and 27-node bricks, with the physical-gradient rule of its custom JVP
(spaces.py:12162-12190).  ``fem_iso_line_tri_tet`` marks its simplex counterpart.  Calling
either evaluates the interpolation on the host.
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


# 1-D quadratic basis index (0: -1, 1: 0, 2: +1) per node and direction: the 9-node quad
# (corners, mid-sides bottom, right, top, left, centre) and the 27-node brick (corners,
# bottom-face edges, top-face edges, vertical edges, face centres x-, x+, y-, y+, z-, z+,
# centre), the node orders of spaces.py:1924-1950 and :12083-12154
_Q2_NODES = {
    2: [(0, 0), (2, 0), (2, 2), (0, 2), (1, 0), (2, 1), (1, 2), (0, 1), (1, 1)],
    3: [(0, 0, 0), (2, 0, 0), (2, 2, 0), (0, 2, 0), (0, 0, 2), (2, 0, 2), (2, 2, 2), (0, 2, 2),
        (1, 0, 0), (2, 1, 0), (1, 2, 0), (0, 1, 0), (1, 0, 2), (2, 1, 2), (1, 2, 2), (0, 1, 2),
        (0, 0, 1), (2, 0, 1), (2, 2, 1), (0, 2, 1), (0, 1, 1), (2, 1, 1), (1, 0, 1), (1, 2, 1),
        (1, 1, 0), (1, 1, 2), (1, 1, 1)],
}


def q2_shape_functions(xi, n_dim):
    """N_a(xi) of the 9-node quad (n_dim 2) or the 27-node brick (n_dim 3) in AutoPDEx's order."""
    xi = np.atleast_1d(np.asarray(xi, dtype=np.float64))
    l = [np.array([0.5 * t * (t - 1), 1 - t * t, 0.5 * t * (t + 1)]) for t in xi]
    return np.array([np.prod([l[d][k] for d, k in enumerate(node)]) for node in _Q2_NODES[n_dim]])


def fem_iso_line_quad_brick(x, xI, fI, settings, overwrite_diff, n_dim):
    """Q1/Q2 interpolation sum_a N_a(x) fI[a] at the reference point ``x`` (host only); the
    kernels implement 2-node lines, 4- and 9-node quads and 8- and 27-node bricks."""
    xI = np.asarray(xI)
    if xI.shape[0] == 2 ** n_dim:
        N = q1_shape_functions(x, n_dim)
    elif n_dim in (2, 3) and xI.shape[0] == 3 ** n_dim:
        N = q2_shape_functions(x, n_dim)
    else:
        raise NotImplementedError("the gb300 backend implements the Q1 and Q2 members of this space")
    return np.tensordot(N, np.asarray(fI, dtype=np.float64), axes=(0, 0))


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
