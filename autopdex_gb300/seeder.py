"""Gauss-Legendre rules with AutoPDEx's point order (seeder.py:303-386, :1046-1062).

Host-side set-up: the returned arrays are what ``models.*`` builders receive; the kernels
hard-code the 2-point rule and the builders check that this is the rule passed.
"""
import numpy as np

_RULES01 = {
    1: (np.array([0.5]), np.array([1.0])),
    2: (np.array([0.21132486540518713, 0.7886751345948129]), np.array([0.5, 0.5])),
    3: (np.array([0.21132486540518713, 0.7886751345948129]), np.array([0.5, 0.5])),
    4: (np.array([0.1127016653792583, 0.5, 0.8872983346207417]),
        np.array([0.2777777777777777, 0.44444444444444453, 0.2777777777777777])),
    5: (np.array([0.1127016653792583, 0.5, 0.8872983346207417]),
        np.array([0.2777777777777777, 0.44444444444444453, 0.2777777777777777])),
}


def gauss_legendre_1d(order):
    """Points and weights on [0, 1], exact for polynomials up to ``order``."""
    if order not in _RULES01:
        raise NotImplementedError("Quadrature order not implemented")
    p, w = _RULES01[order]
    return p.copy(), w.copy()


def _pair(a, b):
    # first array varies fastest, as tensor_product_two_coordinate_arrays
    return np.tile(a, b.shape[0]), np.repeat(b, a.shape[0])


def gauss_legendre_nd(dimension, order):
    """Tensor-product rule on [-1, 1]^dimension, first coordinate fastest."""
    p, w = gauss_legendre_1d(order)
    p = 2 * p - 1
    w = 2 * w
    if dimension == 1:
        return p, w
    if dimension == 2:
        x, y = _pair(p, p)
        return np.stack([x, y], axis=1), np.outer(w, w).reshape(-1)
    if dimension == 3:
        x2, y2 = _pair(p, p)
        x, z = _pair(x2, p)
        y, _ = _pair(y2, p)
        w2 = np.outer(w, w).reshape(-1)
        return np.stack([x, y, z], axis=1), np.outer(w2, w).reshape(-1)
    raise NotImplementedError("Not implemented for this dimensionality!")


def int_pts_ref_tri(order):
    """Points (n, 2) and weights on the reference triangle (0,0) (1,0) (0,1), exact for
    polynomials of degree ``order`` (1 to 4), in the point order of seeder.py:1813-1880:
    the centroid; the three-point rule with points at 1/6 and 2/3; the symmetric six-point
    rule of Dunavant (Int. J. Numer. Meth. Eng. 21, 1985) for degrees 3 and 4."""
    if order == 1:
        return np.array([[1.0 / 3.0, 1.0 / 3.0]]), np.array([0.5])
    if order == 2:
        a, b = 1.0 / 6.0, 2.0 / 3.0
        return np.array([[a, b], [a, a], [b, a]]), np.full(3, 1.0 / 6.0)
    if order in (3, 4):
        a1, w1 = 0.445948490915965, 0.223381589678011
        a2, w2 = 0.091576213509771, 0.109951743655322
        x = [a1, a1, 1 - 2 * a1, a2, a2, 1 - 2 * a2]
        y = [1 - 2 * a1, a1, a1, 1 - 2 * a2, a2, a2]
        return np.stack([x, y], axis=1), 0.5 * np.array([w1, w1, w1, w2, w2, w2])
    raise NotImplementedError("triangle rules of degree 1 to 4 are implemented")


def int_pts_ref_tet(order):
    """Points (n, 3) and weights on the reference tetrahedron, exact for polynomials of
    degree ``order`` (1 or 2): the centroid, and the symmetric four-point rule with points
    at (5 - sqrt 5)/20 and (5 + 3 sqrt 5)/20.  (seeder.py:2288-2330 uses a non-symmetric
    four-point rule of the same degree for order 2; both integrate quadratics exactly, so
    P1 tetrahedra get the same matrices to rounding.)"""
    if order == 1:
        return np.array([[0.25, 0.25, 0.25]]), np.array([1.0 / 6.0])
    if order == 2:
        a = (5.0 - np.sqrt(5.0)) / 20.0
        b = (5.0 + 3.0 * np.sqrt(5.0)) / 20.0
        pts = np.array([[a, a, a], [b, a, a], [a, b, a], [a, a, b]])
        return pts, np.full(4, 1.0 / 24.0)
    raise NotImplementedError("tetrahedron rules of degree 1 and 2 are implemented")
