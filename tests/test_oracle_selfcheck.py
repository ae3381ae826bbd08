"""Self-checks of the CPU oracle on what the reference's own tests do not pin (Q1 bricks,
simplices, convergence): constant-gradient patch tests on distorted meshes, a manufactured
Poisson solution converging at O(h^2), and symmetric tangents from potentials.  No GPU."""
import numpy as np
import pytest
import torch

from autopdex_gb300 import seeder
from oracle import elements as el
from oracle import mesh, newton


def _laplace_element(dim, nen, rule=None, order=2):
    """1/2 |grad u|^2 (no source)."""
    return el.user_potential_element(lambda x, phi, g, p: 0.5 * (g @ g), dim, nen, order=order, rule=rule)


def _solve_linear_patch(coords, conn, fun, boundary):
    a = np.array([0.3, -1.2, 0.7][:coords.shape[1]])
    exact = 0.5 + coords @ a
    s = newton.ElementSet("potential", conn, fun, lambda st: np.zeros((conn.shape[0], 1)), 1)
    prob = newton.Problem([s], coords, coords.shape[0], boundary, exact * boundary)
    sol, info, _ = newton.damped_newton(prob, np.zeros(coords.shape[0]), {}, 1e-12)
    return sol, exact


def _distorted_quads(n):
    coords, conn = mesh.structured_mesh((n, n), [[0., 0.], [1., 0.1], [1.3, 1.0], [-0.1, 0.9]], "quad")
    bnd = np.zeros(coords.shape[0], dtype=bool)
    idx = np.arange(coords.shape[0]).reshape(n + 1, n + 1)
    bnd[idx[0]] = bnd[idx[-1]] = bnd[idx[:, 0]] = bnd[idx[:, -1]] = True
    return coords, conn, bnd


@pytest.mark.parametrize("kind", ["quad4", "tri3", "tri6", "hex8", "tet4"])
def test_patch_linear_field_reproduced(kind):
    """Laplace with Dirichlet data of a linear field: the discrete solution is that field."""
    if kind in ("quad4", "tri3", "tri6"):
        coords, quads, bnd = _distorted_quads(4)
        if kind == "quad4":
            sol, exact = _solve_linear_patch(coords, quads, _laplace_element(2, 4), bnd)
        else:
            tris = np.concatenate([quads[:, [0, 1, 2]], quads[:, [0, 2, 3]]])
            if kind == "tri3":
                sol, exact = _solve_linear_patch(coords, tris, _laplace_element(2, 3, seeder.int_pts_ref_tri(1)), bnd)
            else:
                pts, mid = [c for c in coords], {}

                def node(a, b):
                    k = (min(a, b), max(a, b))
                    if k not in mid:
                        mid[k] = len(pts)
                        pts.append(0.5 * (coords[a] + coords[b]))
                    return mid[k]
                t6 = np.array([[a, b, c, node(a, b), node(b, c), node(c, a)] for a, b, c in tris])
                x6 = np.array(pts)
                # corner nodes on the boundary, and the mid-nodes of boundary edges (the
                # diagonals that split the quads are interior)
                b6 = np.zeros(len(x6), dtype=bool)
                b6[:len(coords)] = bnd
                outer = set(_boundary_edges(quads, bnd))
                for edge, m in mid.items():
                    b6[m] = edge in outer
                sol, exact = _solve_linear_patch(x6, t6, _laplace_element(2, 6, seeder.int_pts_ref_tri(2)), b6)
    else:
        verts = [[0, 0, 0], [1, 0, 0], [1.1, 1, 0], [0, 0.9, 0.1], [0, 0.1, 1], [1, 0, 1.2], [1, 1, 1], [-0.1, 1, 1]]
        coords, hexes = mesh.structured_mesh((3, 3, 3), verts, "brick")
        idx = np.arange(coords.shape[0]).reshape(4, 4, 4)
        bnd = np.zeros(coords.shape[0], dtype=bool)
        for sl in (idx[0], idx[-1], idx[:, 0], idx[:, -1], idx[:, :, 0], idx[:, :, -1]):
            bnd[sl.ravel()] = True
        if kind == "hex8":
            sol, exact = _solve_linear_patch(coords, hexes, _laplace_element(3, 8), bnd)
        else:
            kuhn = [[0, 1, 2, 6], [0, 2, 3, 6], [0, 3, 7, 6], [0, 7, 4, 6], [0, 4, 5, 6], [0, 5, 1, 6]]
            tets = np.concatenate([hexes[:, k] for k in kuhn])
            sol, exact = _solve_linear_patch(coords, tets, _laplace_element(3, 4, seeder.int_pts_ref_tet(1)), bnd)
    assert np.abs(sol - exact).max() <= 1e-10


def _boundary_edges(quads, bnd):
    """Edges of the quads whose both nodes lie on the boundary and that belong to one quad."""
    from collections import Counter
    cnt = Counter()
    for q in quads:
        for i in range(4):
            a, b = q[i], q[(i + 1) % 4]
            cnt[(min(a, b), max(a, b))] += 1
    return [e for e, c in cnt.items() if c == 1 and bnd[e[0]] and bnd[e[1]]]


def test_manufactured_poisson_converges_at_second_order():
    """-lap u = 2 pi^2 sin(pi x) sin(pi y) on the unit square, u = 0 on the boundary: the nodal
    error of the Q1 solution falls by about 4 per halving of h."""
    pi = np.pi

    def integrand(x, phi, g, p):
        f = 2 * pi ** 2 * torch.sin(pi * x[0]) * torch.sin(pi * x[1])
        return 0.5 * (g @ g) - f * phi
    errs = []
    for n in (8, 16, 32):
        coords, conn = mesh.structured_mesh((n, n), [[0., 0.], [1., 0.], [1., 1.], [0., 1.]], "quad")
        bnd = np.isclose(coords[:, 0], 0) | np.isclose(coords[:, 0], 1) | np.isclose(coords[:, 1], 0) | \
            np.isclose(coords[:, 1], 1)
        fun = el.user_potential_element(integrand, 2, 4, order=4)
        s = newton.ElementSet("potential", conn, fun, lambda st: np.zeros((conn.shape[0], 1)), 1)
        prob = newton.Problem([s], coords, coords.shape[0], bnd, np.zeros(coords.shape[0]))
        sol, info, _ = newton.damped_newton(prob, np.zeros(coords.shape[0]), {}, 1e-12)
        errs.append(np.abs(sol - np.sin(pi * coords[:, 0]) * np.sin(pi * coords[:, 1])).max())
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates > 1.8), (errs, rates)


def _t(x):
    return torch.as_tensor(np.asarray(x, dtype=np.float64))


@pytest.mark.parametrize("kind", ["poisson_quad4", "heat_hex8", "neo_hooke_quad4", "neo_hooke_tet4"])
def test_potential_tangents_are_symmetric(kind):
    rng = np.random.default_rng(1)
    if kind == "poisson_quad4":
        fun = el.user_potential_element(el.poisson_sincos_integrand(), 2, 4)
        args = (_t(rng.uniform(-1, 1, 4)), _t([[0., 0.], [1., 0.1], [1.2, 1.], [0., 0.8]]),
                torch.zeros(1))
    elif kind == "heat_hex8":
        fun = el.user_potential_element(el.heat_potential_integrand(1.0), 3, 8)
        x = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]],
                     dtype=float) * 0.5 + rng.uniform(-0.05, 0.05, (8, 3))
        args = (_t(rng.uniform(-1, 1, 8)), _t(x), _t([2.5]))
    elif kind == "neo_hooke_quad4":
        fun = el.hyperelastic_element(2, 4, 2, "plain strain")
        args = (_t(rng.uniform(-0.05, 0.05, (4, 2))), _t([[0., 0.], [1., 0.1], [1.2, 1.], [0., 0.8]]),
                _t([100.0, 0.3]))
    else:
        fun = el.hyperelastic_element(3, 4, 0, "3d", rule=seeder.int_pts_ref_tet(2))
        args = (_t(rng.uniform(-0.05, 0.05, (4, 3))),
                _t([[0., 0., 0.], [1., 0., 0.], [0., 1., 0.], [0., 0., 1.]]),
                _t([100.0, 0.3]))
    R, K = fun(*args)
    K = K.numpy().reshape(R.numel(), R.numel())
    assert np.abs(K - K.T).max() <= 1e-13 * np.abs(K).max()


def test_brick_transfers_are_adjoint_and_interpolate_trilinear_fields():
    """The oracle's 3-D transfers (the learned preconditioner's restriction and prolongation on
    brick grids): restrict3 is the transpose of prolong3 (<P c, r> = <c, P^T r>), and prolong3
    reproduces a trilinear field's nodal values exactly."""
    from oracle import nn as onn
    rng = np.random.default_rng(3)
    for shape, f in (((3, 4, 5), 4), ((5, 5, 2), 2), ((2, 3, 2), 3)):
        c = rng.standard_normal(shape)
        fine = tuple((m - 1) * f + 1 for m in shape)
        r = rng.standard_normal(fine)
        assert abs((onn.prolong3(c, f) * r).sum() - (c * onn.restrict3(r, f, shape)).sum()) <= 1e-12 * np.abs(r).sum()
        I, J, K = np.meshgrid(*(np.arange(m, dtype=float) for m in shape), indexing="ij")
        lin = lambda x, y, z: 1.0 + 0.5 * x - 2.0 * y + 0.25 * z + 0.1 * x * y * z
        fi, fj, fk = np.meshgrid(*(np.arange(m, dtype=float) / f for m in fine), indexing="ij")
        assert np.abs(onn.prolong3(lin(I, J, K), f) - lin(fi, fj, fk)).max() <= 1e-12


def test_unet3d_oracle_shapes_and_linearity_of_the_output_layer():
    """The oracle's 3-D U-Net maps (B, D, H, W, 16) to (B, D, H, W, 16) for extents divisible by 8,
    and its output layer (no ReLU) is affine in its input."""
    from oracle import nn as onn
    g = torch.Generator().manual_seed(1)
    P = {n: (torch.randn(co, c1 + c2, 3, 3, 3, generator=g, dtype=torch.float64) * 0.1,
             torch.randn(co, generator=g, dtype=torch.float64) * 0.1) for n, c1, c2, co, relu in onn.LAYERS3}
    x = torch.randn(2, 8, 16, 8, 16, generator=g, dtype=torch.float64)
    y = onn.unet3d(x, P)
    assert y.shape == x.shape
    w, b = P["out"]
    a = torch.randn(1, 8, 8, 8, 16, generator=g, dtype=torch.float64)
    c = torch.randn(1, 8, 8, 8, 16, generator=g, dtype=torch.float64)
    lhs = onn.conv3d(a + c, w, b, 0)
    rhs = onn.conv3d(a, w, b, 0) + onn.conv3d(c, w, torch.zeros_like(b), 0)
    assert (lhs - rhs).abs().max() <= 1e-12 * lhs.abs().max()
