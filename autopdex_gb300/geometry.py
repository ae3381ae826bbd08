"""Boundary selection helpers with AutoPDEx's semantics (geometry.py).

Host-side set-up, run once per mesh.  ``in_sdfs(x, psdf_polygon)`` keeps the reference's
behaviour at polygon corners: two vanishing edge distances combine to 0/0 = NaN under
R-equivalence (geometry.py:33-45, :672-694), so corner nodes are not selected.
"""
import numpy as np


def _psdf_segment(x, p1, p2):
    L = np.linalg.norm(p2 - p1)
    omega = ((x[:, 0] - p1[0]) * (p2[1] - p1[1]) - (x[:, 1] - p1[1]) * (p2[0] - p1[0])) / L
    c = (p1 + p2) / 2
    r = L / 2
    d = x - c
    trim = (r * r - np.sum(d * d, axis=1)) / (2 * r)
    return np.sqrt(omega ** 2 + (np.sqrt(trim ** 2 + omega ** 4) - trim) ** 2 / 4)


def psdf_polygon(x, pts):
    """Positive smooth distance to a polygon boundary (geometry.py:672-694)."""
    x = np.atleast_2d(np.asarray(x, dtype=np.float64))
    p = np.asarray(pts, dtype=np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):
        d = _psdf_segment(x, p[0], p[1])
        for i in range(p.shape[0] - 1):
            di = _psdf_segment(x, p[-i], p[-(i + 1)])
            d = d * di / (d + di)
    return d


def in_sdfs(x, sdf_fun, tol=1e-6):
    """``isclose(sdf(x), 0, atol=tol)`` per point (geometry.py:858-871).  ``sdf_fun`` maps an
    (n, dim) array to n distances (e.g. ``lambda x: psdf_polygon(x, pts)``)."""
    d = np.asarray(sdf_fun(np.asarray(x, dtype=np.float64)), dtype=np.float64)
    with np.errstate(invalid="ignore"):
        return np.abs(d) <= tol


def in_planes(x, x_p1, normal, tol=1e-6):
    """Points on the plane through ``x_p1`` with ``normal`` (geometry.py:909-922)."""
    d = (np.asarray(x, dtype=np.float64) - np.asarray(x_p1, dtype=np.float64)) @ np.asarray(normal, dtype=np.float64)
    return np.abs(d) <= tol


def select_elements_in_plane(x_nodes, surface_elements, x_p1, normal):
    """Surface elements with all nodes in the plane (geometry.py:1048-1067)."""
    on = in_planes(x_nodes, x_p1, normal)
    return np.all(on[np.asarray(surface_elements)], axis=1)
