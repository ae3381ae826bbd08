"""Simplex elements on the host: the oracle's triangle and tetrahedron routines against
closed-form stiffness matrices, the simplex rules of seeder against exact monomial integrals,
and the set-up's element-type mapping.  No GPU."""
from math import factorial

import numpy as np
import pytest
import torch

from autopdex_gb300 import _problem, models, seeder, spaces
from autopdex_gb300 import _native as N
from oracle import elements as el


def _stiffness(dim, nen, rule, xI):
    fun = el.user_potential_element(el.heat_potential_integrand(0.0), dim, nen, rule=rule)
    R, K = fun(torch.zeros(nen, dtype=torch.float64), torch.as_tensor(xI, dtype=torch.float64),
               torch.tensor([1.0], dtype=torch.float64))
    return K.numpy()


def test_p1_triangle_and_tetrahedron_stiffness():
    """grad N_a . grad N_b times the volume on the reference simplices (counter-clockwise,
    det J = 1): 1/2 [[2,-1,-1],[-1,1,0],[-1,0,1]] and 1/6 [[3,-1,-1,-1],[-1,1,0,0],...]."""
    K = _stiffness(2, 3, seeder.int_pts_ref_tri(1), [[0., 0.], [1., 0.], [0., 1.]])
    assert np.allclose(K, 0.5 * np.array([[2, -1, -1], [-1, 1, 0], [-1, 0, 1]]), rtol=0, atol=1e-15)
    K = _stiffness(3, 4, seeder.int_pts_ref_tet(1), [[0., 0., 0.], [1., 0., 0.], [0., 1., 0.], [0., 0., 1.]])
    G = np.array([[-1., -1., -1.], [1., 0., 0.], [0., 1., 0.], [0., 0., 1.]])
    assert np.allclose(K, G @ G.T / 6.0, rtol=0, atol=1e-15)


def test_p2_triangle_stiffness_exact():
    """The 6-node triangle with the degree-2 rule (exact for its quadratic integrand) against
    the closed-form matrix, and against a scaled copy of the element (K is scale-free in 2-D)."""
    sp = pytest.importorskip("sympy")
    x, y = sp.symbols("x y")
    L = [1 - x - y, x, y]
    Nf = [L[0] * (2 * L[0] - 1), L[1] * (2 * L[1] - 1), L[2] * (2 * L[2] - 1), 4 * L[0] * L[1], 4 * L[1] * L[2],
          4 * L[2] * L[0]]
    G = [[sp.diff(n, x), sp.diff(n, y)] for n in Nf]
    exact = np.array([[float(sp.integrate(sp.integrate(G[a][0] * G[b][0] + G[a][1] * G[b][1], (y, 0, 1 - x)),
                                          (x, 0, 1))) for b in range(6)] for a in range(6)])
    xI = [[0., 0.], [1., 0.], [0., 1.], [0.5, 0.], [0.5, 0.5], [0., 0.5]]
    K = _stiffness(2, 6, seeder.int_pts_ref_tri(2), xI)
    assert np.allclose(K, exact, rtol=0, atol=1e-14)
    K3 = _stiffness(2, 6, seeder.int_pts_ref_tri(2), 3.0 * np.asarray(xI))
    assert np.allclose(K3, exact, rtol=0, atol=1e-13)


def test_p2_tetrahedron_stiffness_exact():
    """The 10-node tetrahedron with the degree-2 rule against the closed-form matrix."""
    sp = pytest.importorskip("sympy")
    x, y, z = sp.symbols("x y z")
    L = [1 - x - y - z, x, y, z]
    Nf = [l * (2 * l - 1) for l in L] + [4 * L[i] * L[j] for i, j in [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]]
    G = [[sp.diff(n, v) for v in (x, y, z)] for n in Nf]

    def vol(f):
        return float(sp.integrate(sp.integrate(sp.integrate(f, (z, 0, 1 - x - y)), (y, 0, 1 - x)), (x, 0, 1)))
    exact = np.array([[vol(sum(G[a][d] * G[b][d] for d in range(3))) for b in range(10)] for a in range(10)])
    c = np.array([[0., 0., 0.], [1., 0., 0.], [0., 1., 0.], [0., 0., 1.]])
    mids = [0.5 * (c[i] + c[j]) for i, j in [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]]
    K = _stiffness(3, 10, seeder.int_pts_ref_tet(2), np.vstack([c, mids]))
    assert np.allclose(K, exact, rtol=0, atol=1e-14)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_triangle_rules_exact(order):
    p, w = seeder.int_pts_ref_tri(order)
    assert abs(w.sum() - 0.5) < 1e-15
    for a in range(order + 1):
        for b in range(order + 1 - a):
            exact = factorial(a) * factorial(b) / factorial(a + b + 2)
            assert abs(np.sum(w * p[:, 0] ** a * p[:, 1] ** b) - exact) < 1e-14, (a, b)


@pytest.mark.parametrize("order", [1, 2])
def test_tetrahedron_rules_exact(order):
    p, w = seeder.int_pts_ref_tet(order)
    for a in range(order + 1):
        for b in range(order + 1 - a):
            for c in range(order + 1 - a - b):
                exact = factorial(a) * factorial(b) * factorial(c) / factorial(a + b + c + 3)
                assert abs(np.sum(w * p[:, 0] ** a * p[:, 1] ** b * p[:, 2] ** c) - exact) < 1e-15


def test_simplex_set_up():
    assert _problem._elem_type(3, 2) == N.AGX_TRI3 and _problem._elem_type(3, 2, surface=True) == N.AGX_LINE3
    assert _problem._elem_type(6, 2) == N.AGX_TRI6 and _problem._elem_type(4, 3) == N.AGX_TET4
    assert _problem._elem_type(10, 3) == N.AGX_TET10
    assert _problem._elem_type(4, 2) == N.AGX_QUAD4
    with pytest.raises(NotImplementedError):
        _problem._elem_type(20, 3)
    d = models.mixed_reference_domain_potential(models.poisson_sincos_integrand(), {"phi": spaces.fem_iso_line_tri_tet},
                                                *seeder.int_pts_ref_tri(2), "phi")
    assert d.qpoints.shape == (3, 2) and np.isclose(d.qweights.sum(), 0.5)
    weak = models.hyperelastic_steady_state_weak(models.neo_hooke, 1.0, 0.3, "3d")
    d = models.isoparametric_domain_element_galerkin(weak, spaces.fem_iso_line_tri_tet, *seeder.int_pts_ref_tet(2))
    assert d.qpoints.shape == (4, 3)
    assert np.allclose(spaces.fem_iso_line_tri_tet([0.2, 0.3], np.zeros((6, 2)), np.arange(6.0), {}, False, 2),
                       spaces.simplex_shape_functions([0.2, 0.3], 2, 6) @ np.arange(6.0))


def test_q2_brick_oracle():
    """The 27-node brick: N_a is 1 at its own node and 0 at the others, and the stiffness
    with the 3-point rule equals the exact integral over the reference cube, assembled from
    the exact 1-D mass and stiffness matrices of the quadratic basis (the integrand is a
    sum of products of 1-D factors)."""
    from numpy.polynomial import polynomial as P
    from oracle.mesh import HEX27_NODES, shape_functions
    pos = np.array(HEX27_NODES, dtype=float) - 1.0
    V = np.array([shape_functions(p, 3, 27) for p in pos])
    assert np.allclose(V, np.eye(27), rtol=0, atol=1e-15)
    basis = [np.array([0.0, -0.5, 0.5]), np.array([1.0, 0.0, -1.0]), np.array([0.0, 0.5, 0.5])]  # t(t-1)/2, 1-t^2, t(t+1)/2

    def integral(c):
        ci = P.polyint(c)
        return P.polyval(1.0, ci) - P.polyval(-1.0, ci)
    M = np.array([[integral(P.polymul(bi, bj)) for bj in basis] for bi in basis])
    S = np.array([[integral(P.polymul(P.polyder(bi), P.polyder(bj))) for bj in basis] for bi in basis])
    idx = np.array(HEX27_NODES)
    ix, iy, iz = (idx[:, d] for d in range(3))
    exact = (S[np.ix_(ix, ix)] * M[np.ix_(iy, iy)] * M[np.ix_(iz, iz)] + M[np.ix_(ix, ix)] * S[np.ix_(iy, iy)] *
             M[np.ix_(iz, iz)] + M[np.ix_(ix, ix)] * M[np.ix_(iy, iy)] * S[np.ix_(iz, iz)])
    K = _stiffness(3, 27, seeder.gauss_legendre_nd(3, 4), pos)
    assert np.allclose(K, exact, rtol=0, atol=1e-13)
