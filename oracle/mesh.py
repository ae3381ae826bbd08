"""Oracle: meshes, quadrature, shape functions and boundary selectors (float64 NumPy).

Test infrastructure only (see ``oracle/__init__.py``).  Each function restates the
AutoPDEx function named in its docstring.
"""
import numpy as np


# ----------------------------------------------------------------------------------
# mesher.structured_mesh  (autopdex/mesher.py:29-205)
# ----------------------------------------------------------------------------------
def structured_mesh(n_elements, vertices, element_type):
    """Structured quad/brick mesh of a bilinearly/trilinearly mapped square/cube.

    Node numbering ``i*(ny+1)+j`` (2-D) and ``i*(ny+1)*(nz+1)+j*(nz+1)+k`` (3-D);
    element node order as mesher.py:88-94 (quad) and mesher.py:150-160 (brick).
    """
    v = np.asarray(vertices, dtype=np.float64)
    dim = v.shape[1]
    if dim == 2:
        assert element_type == "quad"
        nx, ny = n_elements
        s = np.linspace(-1.0, 1.0, nx + 1)
        t = np.linspace(-1.0, 1.0, ny + 1)
        S, T = np.meshgrid(s, t, indexing="ij")
        S = S.ravel()[:, None]
        T = T.ravel()[:, None]
        coords = ((1 - S) * (1 - T) * v[0] + (1 + S) * (1 - T) * v[1]
                  + (1 + S) * (1 + T) * v[2] + (1 - S) * (1 + T) * v[3]) / 4
        I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        I = I.ravel()
        J = J.ravel()
        elems = np.stack([I * (ny + 1) + J, I * (ny + 1) + J + 1,
                          (I + 1) * (ny + 1) + J + 1, (I + 1) * (ny + 1) + J], axis=1)
        return coords, elems.astype(np.int64)
    if dim == 3:
        assert element_type == "brick"
        nx, ny, nz = n_elements
        s = np.linspace(-1.0, 1.0, nx + 1)
        t = np.linspace(-1.0, 1.0, ny + 1)
        u = np.linspace(-1.0, 1.0, nz + 1)
        S, T, U = np.meshgrid(s, t, u, indexing="ij")
        S = S.ravel()[:, None]
        T = T.ravel()[:, None]
        U = U.ravel()[:, None]
        coords = ((1 - S) * (1 - T) * (1 - U) * v[0] + (1 + S) * (1 - T) * (1 - U) * v[1]
                  + (1 + S) * (1 + T) * (1 - U) * v[2] + (1 - S) * (1 + T) * (1 - U) * v[3]
                  + (1 - S) * (1 - T) * (1 + U) * v[4] + (1 + S) * (1 - T) * (1 + U) * v[5]
                  + (1 + S) * (1 + T) * (1 + U) * v[6] + (1 - S) * (1 + T) * (1 + U) * v[7]) / 8
        I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        I = I.ravel()
        J = J.ravel()
        K = K.ravel()
        a = (ny + 1) * (nz + 1)
        b = nz + 1
        n = lambda i, j, k: i * a + j * b + k
        elems = np.stack([n(I, J, K), n(I + 1, J, K), n(I + 1, J + 1, K), n(I, J + 1, K),
                          n(I, J, K + 1), n(I + 1, J, K + 1), n(I + 1, J + 1, K + 1),
                          n(I, J + 1, K + 1)], axis=1)
        return coords, elems.astype(np.int64)
    raise NotImplementedError(dim)


# ----------------------------------------------------------------------------------
# seeder.gauss_legendre_nd / tensor_product_rule  (autopdex/seeder.py:303-386, :1046-1062)
# ----------------------------------------------------------------------------------
_GL01 = {
    2: (np.array([0.21132486540518713, 0.7886751345948129]), np.array([0.5, 0.5])),
    3: (np.array([0.21132486540518713, 0.7886751345948129]), np.array([0.5, 0.5])),
    4: (np.array([0.1127016653792583, 0.5, 0.8872983346207417]),
        np.array([0.2777777777777777, 0.44444444444444453, 0.2777777777777777])),
    5: (np.array([0.1127016653792583, 0.5, 0.8872983346207417]),
        np.array([0.2777777777777777, 0.44444444444444453, 0.2777777777777777])),
}


def _tensor2(xi, yi):
    """seeder.tensor_product_two_coordinate_arrays (seeder.py:303-321): first index fastest."""
    return np.tile(xi, yi.shape[0]), np.tile(yi, xi.shape[0]).reshape(xi.shape[0], yi.shape[0]).T.ravel()


def gauss_legendre_nd(dimension, order):
    """Points on [-1,1]^d and weights (x fastest), as seeder.py:1046-1062 + :324-367."""
    p, w = _GL01[order]
    p = 2 * p - 1
    w = 2 * w
    if dimension == 1:
        return p.copy(), w.copy()
    if dimension == 2:
        xi, yi = _tensor2(p, p)
        return np.stack([xi, yi], axis=1), np.outer(w, w).ravel()
    if dimension == 3:
        xi2, yi2 = _tensor2(p, p)
        xi, zi = _tensor2(xi2, p)
        yi, _ = _tensor2(yi2, p)
        w2 = np.outer(w, w).ravel()
        return np.stack([xi, yi, zi], axis=1), np.outer(w2, w).ravel()
    raise NotImplementedError(dimension)


# ----------------------------------------------------------------------------------
# spaces.fem_iso_line_quad_brick shape functions (autopdex/spaces.py:356-366, :1913-1950,
# :12057-12081).  Written from the Lagrange tensor-product definitions; node order as there.
# ----------------------------------------------------------------------------------
# 27-node brick: per node the 1-D basis index (0: -1, 1: 0, 2: +1) in x, y, z, in the node order
# of spaces.py:12083-12154 -- corners as the 8-node brick, mid-edges of the bottom face
# (0-1, 1-2, 2-3, 3-0), of the top face, the vertical edges (0-4, 1-5, 2-6, 3-7), the face
# centres x-, x+, y-, y+, z-, z+, and the centre
HEX27_NODES = [(0, 0, 0), (2, 0, 0), (2, 2, 0), (0, 2, 0), (0, 0, 2), (2, 0, 2), (2, 2, 2), (0, 2, 2),
               (1, 0, 0), (2, 1, 0), (1, 2, 0), (0, 1, 0), (1, 0, 2), (2, 1, 2), (1, 2, 2), (0, 1, 2),
               (0, 0, 1), (2, 0, 1), (2, 2, 1), (0, 2, 1), (0, 1, 1), (2, 1, 1), (1, 0, 1), (1, 2, 1),
               (1, 1, 0), (1, 1, 2), (1, 1, 1)]


def shape_functions(xi, n_dim, n_nodes, xp=np):
    """N_a(xi) for line (2, 3 nodes), quad (4, 9 nodes), triangle (3, 6 nodes), brick (8, 27
    nodes) and tetrahedron (4, 10 nodes) elements.

    ``xi`` is a scalar (line) or a vector of length ``n_dim``; ``xp`` is ``numpy`` or
    ``torch`` so that the same definition serves the AD-based element routines.
    """
    stack = xp.stack
    if n_dim == 1:
        if n_nodes == 2:
            return stack([0.5 * (1 - xi), 0.5 * (1 + xi)])
        if n_nodes == 3:  # nodes at -1, 1, 0
            return stack([0.5 * xi * (xi - 1), 0.5 * xi * (xi + 1), 1 - xi * xi])
    if n_dim == 2:
        x, y = xi[0], xi[1]
        if n_nodes == 4:  # (-1,-1), (1,-1), (1,1), (-1,1)
            return stack([(1 - x) * (1 - y), (1 + x) * (1 - y), (1 + x) * (1 + y), (1 - x) * (1 + y)]) / 4
        if n_nodes == 9:  # corners, then mid-sides (bottom, right, top, left), then centre
            lx = [0.5 * x * (x - 1), 1 - x * x, 0.5 * x * (x + 1)]
            ly = [0.5 * y * (y - 1), 1 - y * y, 0.5 * y * (y + 1)]
            order = [(0, 0), (2, 0), (2, 2), (0, 2), (1, 0), (2, 1), (1, 2), (0, 1), (1, 1)]
            return stack([lx[i] * ly[j] for i, j in order])
    if n_dim == 2 and n_nodes == 3:  # fem_iso_line_tri_tet, n_dim 2, 3 nodes (spaces.py:13748-13752)
        return stack([1 - xi[0] - xi[1], xi[0], xi[1]])
    if n_dim == 2 and n_nodes == 6:  # the 6-node case (spaces.py:13753-13757), expanded as written there
        x, y = xi[0], xi[1]
        x0 = 4 * x
        x1 = x0 * y
        x2 = -x - y + 1
        return stack([x1 + 2 * x ** 2 - 3 * x + 2 * y ** 2 - 3 * y + 1, x * (2 * x - 1), y * (2 * y - 1),
                      x0 * x2, x1, 4 * x2 * y])
    if n_dim == 3 and n_nodes == 4:  # n_dim 3, 4 nodes (spaces.py:14625-14630)
        return stack([1 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]])
    if n_dim == 3 and n_nodes == 10:  # the 10-node case (spaces.py:14632-14640), expanded as written there
        x, y, z = xi[0], xi[1], xi[2]
        x0 = 4 * x
        x1 = x0 * y
        x2 = x0 * z
        x3 = 4 * y
        x4 = x3 * z
        x5 = -x - y - z + 1
        return stack([x1 + x2 + x4 + 2 * x ** 2 - 3 * x + 2 * y ** 2 - 3 * y + 2 * z ** 2 - 3 * z + 1,
                      x * (2 * x - 1), y * (2 * y - 1), z * (2 * z - 1), x0 * x5, x1, x3 * x5, 4 * x5 * z, x2, x4])
    if n_dim == 3 and n_nodes == 27:  # spaces.py:12083-12154: tensor products of the 1-D quadratic basis
        x, y, z = xi[0], xi[1], xi[2]
        lx = [0.5 * x * (x - 1), 1 - x * x, 0.5 * x * (x + 1)]
        ly = [0.5 * y * (y - 1), 1 - y * y, 0.5 * y * (y + 1)]
        lz = [0.5 * z * (z - 1), 1 - z * z, 0.5 * z * (z + 1)]
        return stack([lx[i] * ly[j] * lz[k] for i, j, k in HEX27_NODES])
    if n_dim == 3 and n_nodes == 8:
        x, y, z = xi[0], xi[1], xi[2]
        sgn = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1),
               (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]
        return stack([(1 + a * x) * (1 + b * y) * (1 + c * z) / 8 for a, b, c in sgn])
    raise NotImplementedError((n_dim, n_nodes))


# ----------------------------------------------------------------------------------
# geometry.psdf_polygon / in_sdfs / in_planes / select_elements_in_plane
# (autopdex/geometry.py:33-45, :78-90, :123-157, :185-201, :462-484, :672-694, :850-922, :1048-1067)
# ----------------------------------------------------------------------------------
def _sdf_infinite_line(x, p1, p2):
    L = np.linalg.norm(p2 - p1)
    return ((x[:, 0] - p1[0]) * (p2[1] - p1[1]) - (x[:, 1] - p1[1]) * (p2[0] - p1[0])) / L


def _sdf_sphere(x, xc, r):
    d = x - xc
    return (r ** 2 - np.sum(d * d, axis=1)) / (2 * r)


def _r_trimming(o, t):
    return np.sqrt(o ** 2 + (np.sqrt(t ** 2 + o ** 4) - t) ** 2 / 4)


def _psdf_trimmed_line(x, p1, p2):
    omega = _sdf_infinite_line(x, p1, p2)
    xc = (p1 + p2) / 2
    trim = _sdf_sphere(x, xc, np.linalg.norm(p2 - p1) / 2)
    return _r_trimming(omega, trim)


def psdf_polygon(x, pts):
    """Positive smooth distance to a polygon boundary, combined by R-equivalence.

    The combination o1*o2/(o1+o2) is NaN where two edges both vanish (the polygon's
    corners), exactly as in geometry.py:33-45 + :672-694, so ``in_sdfs`` does not
    select corner nodes.
    """
    x = np.atleast_2d(np.asarray(x, dtype=np.float64))
    p = np.asarray(pts, dtype=np.float64)
    n = p.shape[0]
    with np.errstate(invalid="ignore", divide="ignore"):
        d = _psdf_trimmed_line(x, p[0], p[1])
        for i in range(n - 1):
            di = _psdf_trimmed_line(x, p[-i], p[-(i + 1)])
            d = d * di / (d + di)
    return d


def in_sdfs(x, pts, tol=1e-6):
    """Nodes on the polygon boundary: ``isclose(psdf, 0, atol=tol)`` (geometry.py:850-871)."""
    d = psdf_polygon(x, pts)
    with np.errstate(invalid="ignore"):
        return np.abs(d) <= tol


def in_planes(x, p1, normal, tol=1e-6):
    """Nodes in the plane through ``p1`` with ``normal`` (geometry.py:185-201, :909-922)."""
    x = np.asarray(x, dtype=np.float64)
    d = (x - np.asarray(p1, dtype=np.float64)) @ np.asarray(normal, dtype=np.float64)
    return np.abs(d) <= tol


def select_elements_in_plane(x, surface_elements, p1, normal, tol=1e-6):
    """Surface elements whose nodes all lie in the plane (geometry.py:1048-1067)."""
    on = in_planes(x, p1, normal, tol)
    return np.all(on[np.asarray(surface_elements)], axis=1)


def dof_select(dirichlet_nodes, selected_fields):
    """utility.dof_select (utility.py:448-462)."""
    if isinstance(selected_fields, bool):
        return dirichlet_nodes * selected_fields
    return np.outer(dirichlet_nodes, np.asarray(selected_fields))
