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
