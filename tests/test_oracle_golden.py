"""The CPU oracle against the golden values of the reference's own tests, plus
finite-difference checks of its AD-derived tangents (no GPU)."""
import json
import os

import numpy as np
import pytest
import torch

from oracle import elements as el
from oracle import mesh, newton

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "golden.json")) as _fh:
    GOLDEN = json.load(_fh)


def test_golden_poisson_5x5():
    """tests/test_dicts_as_dofs_user_potential.py:63 -> sum(phi) = 1.9066412530282952."""
    pts = [[0., 0.], [1., 0.], [1., 1.], [0., 1.]]
    coords, elems = mesh.structured_mesh((5, 5), pts, "quad")
    dn = mesh.in_sdfs(coords, pts)
    fun = el.user_potential_element(el.poisson_sincos_integrand(), 2, 4)
    s = newton.ElementSet("potential", elems, fun, lambda st: np.zeros((elems.shape[0], 1)), 1)
    prob = newton.Problem([s], coords, coords.shape[0], dn, np.zeros(coords.shape[0]))
    sol, info, _ = newton.damped_newton(prob, np.zeros(coords.shape[0]), {})
    assert info[0] == 1 and not info[2]
    g = GOLDEN["poisson_5x5_sum_phi"]["value"]
    assert g == 1.9066412530282952
    assert abs(sol.sum() - g) <= 1e-12 * g


def test_polygon_corners_not_selected():
    """R-equivalence of two vanishing edge distances is 0/0 at a polygon corner, so the
    reference's in_sdfs(psdf_polygon) leaves the 4 corners free (20 boundary nodes -> 16)."""
    pts = [[0., 0.], [1., 0.], [1., 1.], [0., 1.]]
    coords, _ = mesh.structured_mesh((5, 5), pts, "quad")
    dn = mesh.in_sdfs(coords, pts)
    assert dn.sum() == 16
    corners = [0, 5, 30, 35]
    assert not dn[corners].any()


def _q2_test_arrays():
    golden = os.path.join(HERE, "golden", "cook_q2_mesh.npz")
    d = np.load(golden)
    return d["x_nodes"], d["elements"], d["surface_elements"]


@pytest.fixture(scope="module")
def cook_q2():
    """The Q2 Cook membrane of tests/test_user_elem_impl_diff_and_adaptive_load_step.py (Q2
    user element, neo-Hooke plane strain, Neumann traction 20) solved by load stepping to 1."""
    x, E, S = _q2_test_arrays()
    pts = [[0., 0.], [48., 44.], [48., 60.], [0., 44.]]
    dn = mesh.in_planes(x, pts[0], [1., 0.])
    dd = mesh.dof_select(dn, np.array([True, True]))
    NE = S[mesh.select_elements_in_plane(x, S, pts[1], [1., 0.])]
    s1 = newton.ElementSet("element", E, el.hyperelastic_element(2, 9, 4, "plain strain"),
                           lambda st: np.tile([st["E"], st["nu"]], (E.shape[0], 1)), 2)
    s2 = newton.ElementSet("neumann", NE, el.neumann_line_element(3, 4), None, 2,
                           traction=lambda st: np.array([0., st["load"]]))
    n = x.shape[0] * 2
    prob = newton.Problem([s1, s2], x, n, dd, np.zeros(n))
    dofs = np.zeros(n)
    st = {"E": 100., "nu": 0.3}
    for m in [0.2, 0.4, 0.6, 0.8, 1.0]:
        st["load"] = m * 20.0
        dofs, info, _ = newton.damped_newton(prob, dofs, st, 1e-8)
        assert not info[2]
    return prob, dofs, st


_FIRST = (("E", "cook_q2_d_dofs_dot_dofs_d_youngs_modulus"), ("nu", "cook_q2_d_dofs_dot_dofs_d_poisson_ratio"))
_NAME = {"E": "youngs_modulus", "nu": "poisson_ratio"}


def test_golden_q2_cook_neo_hooke(cook_q2):
    """tests/test_user_elem_impl_diff_and_adaptive_load_step.py:153-155 -> dofs.dofs =
    19390.35027108 and its derivatives -216.0310416 (E) and -1859.43760286 (nu)."""
    prob, dofs, st = cook_q2
    g = GOLDEN["cook_q2_dofs_dot_dofs"]["value"]
    assert abs(dofs @ dofs - g) <= 1e-9 * g
    # first derivatives of u.u in E and nu by implicit differentiation at the final state
    # (the golden values carry 10 and 12 significant digits)
    for key, name in _FIRST:
        du = newton.implicit_sensitivity(prob, dofs, st, key)
        ref = GOLDEN[name]["value"]
        assert abs(2.0 * dofs @ du - ref) <= 1e-7 * abs(ref), (key, 2.0 * dofs @ du, ref)


def test_golden_q2_cook_second_order(cook_q2):
    """tests/test_user_elem_impl_diff_and_adaptive_load_step.py:156-159 -> the second
    derivatives of u.u: 4.17157824 (E E), -51.42695148 (E nu and nu E), -45854.7002203
    (nu nu).  d2(u.u)/dp_i dp_j = 2 (u_i . u_j + u . u_ij), with u_ij from
    K u_ij = -D^2 R[(u_i, e_i), (u_j, e_j)] (nested forward-mode AD of the elements)."""
    prob, dofs, st = cook_q2
    du = {k: newton.implicit_sensitivity(prob, dofs, st, k) for k in ("E", "nu")}
    for a, b in (("E", "E"), ("E", "nu"), ("nu", "E"), ("nu", "nu")):
        uab = newton.implicit_second_sensitivity(prob, dofs, st, du[a], a, du[b], b)
        val = 2.0 * (du[a] @ du[b] + dofs @ uab)
        ref = GOLDEN["cook_q2_d2_dofs_dot_dofs_d_%s_%s" % (_NAME[a], _NAME[b])]["value"]
        assert abs(val - ref) <= 1e-8 * abs(ref), (a, b, val, ref)


def test_golden_q2_cook_reverse_mode(cook_q2):
    """Reverse implicit differentiation (implicit_diff_mode 'backward', checked by the
    reference at tests/test_user_elem_impl_diff_and_adaptive_load_step.py:169-170 against
    the forward values): one adjoint solve K^T lam = dJ/du = 2u gives dJ/dp = -lam . dR/dp
    for every p, and the second derivative d2J/dnu2 = 2 u_nu . u_nu - lam . D^2 R[d_nu, d_nu]."""
    prob, dofs, st = cook_q2
    for key, name in _FIRST:
        val = newton.adjoint_sensitivity(prob, dofs, st, 2.0 * dofs, key)
        ref = GOLDEN[name]["value"]
        assert abs(val - ref) <= 1e-7 * abs(ref), (key, val, ref)
    du = newton.implicit_sensitivity(prob, dofs, st, "nu")
    _, coo = newton.assemble(prob.sets, dofs, prob.coords, st, prob.n_dofs)
    lam = newton.linear_solve_scipy((coo[1], coo[0], coo[2]), 2.0 * dofs, prob.n_dofs, ~prob.dirichlet)
    D2 = newton.second_directional_residual(prob, dofs, st, du, "nu", du, "nu")
    free = ~prob.dirichlet
    val = 2.0 * du @ du - lam[free] @ D2[free]
    ref = GOLDEN["cook_q2_d2_dofs_dot_dofs_d_poisson_ratio_poisson_ratio"]["value"]
    assert abs(val - ref) <= 1e-8 * abs(ref), (val, ref)


class _OracleOps:
    """The oracle's residual, tangent product and spsolve in the interface the backend's
    implicit-differentiation algebra (``autopdex_gb300.implicit_diff``) runs on."""

    def __init__(self, prob, u, settings):
        self.prob, self.u, self.settings = prob, u, settings
        self.free = (~prob.dirichlet).astype(np.float64)

    def residual(self, w, settings):
        return self.prob.residual(w, settings)

    def tangent_apply(self, w, settings, v):
        import scipy.sparse
        _, (r, c, d) = newton.assemble(self.prob.sets, w, self.prob.coords, settings, self.prob.n_dofs)
        return scipy.sparse.coo_matrix((d, (r, c)), shape=(self.prob.n_dofs,) * 2).tocsr() @ v

    def solve(self, rhs):
        _, coo = newton.assemble(self.prob.sets, self.u, self.prob.coords, self.settings, self.prob.n_dofs)
        return newton.linear_solve_scipy(coo, rhs, self.prob.n_dofs, ~self.prob.dirichlet)


def test_implicit_diff_algebra_reproduces_golden(cook_q2):
    """The backend's second-order and adjoint algebra (four-point differences of tangent
    products and residuals, ``autopdex_gb300.implicit_diff``), run here on the oracle's
    operations, reproduces the reference's seven golden values of the Q2 Cook case."""
    from autopdex_gb300 import implicit_diff
    prob, dofs, st = cook_q2
    ops = _OracleOps(prob, dofs, st)
    first = implicit_diff.first_order(ops, dofs, st, ["E", "nu"])
    for key, name in _FIRST:
        ref = GOLDEN[name]["value"]
        assert abs(2.0 * dofs @ first[key] - ref) <= 1e-7 * abs(ref)
    second = implicit_diff.second_order(ops, dofs, st, first)
    assert len(second) == 4
    for (a, b), uab in second.items():
        val = 2.0 * (first[a] @ first[b] + dofs @ uab)
        ref = GOLDEN["cook_q2_d2_dofs_dot_dofs_d_%s_%s" % (_NAME[a], _NAME[b])]["value"]
        assert abs(val - ref) <= 1e-8 * abs(ref), (a, b, val, ref)
    adj = implicit_diff.adjoint(ops, dofs, st, ["E", "nu"], 2.0 * dofs)
    for key, name in _FIRST:
        ref = GOLDEN[name]["value"]
        assert abs(adj[key] - ref) <= 1e-7 * abs(ref), (key, adj[key], ref)


def _fd_check(fun, args, idx=0, h=1e-6):
    R, K = fun(*args)
    x = args[idx]
    flat = x.reshape(-1)
    Kfd = torch.zeros_like(K.reshape(flat.numel(), flat.numel()))
    for j in range(flat.numel()):
        d = torch.zeros_like(flat)
        d[j] = h
        a = list(args)
        a[idx] = (flat + d).reshape(x.shape)
        rp = fun(*a)[0].reshape(-1)
        a[idx] = (flat - d).reshape(x.shape)
        rm = fun(*a)[0].reshape(-1)
        Kfd[:, j] = (rp - rm) / (2 * h)
    err = (K.reshape(Kfd.shape) - Kfd).abs().max() / K.abs().max()
    return float(err)


@pytest.mark.parametrize("case", ["poisson_q4", "heat_h8", "neo_q4", "neo_h8", "heat_be_h8"])
def test_oracle_tangent_is_derivative_of_residual(case):
    g = torch.Generator().manual_seed(1)
    D = torch.float64
    if case == "poisson_q4":
        fun = el.user_potential_element(el.poisson_sincos_integrand(), 2, 4)
        xI = torch.tensor([[0., 0.], [1.1, 0.1], [1.0, 0.9], [-0.1, 1.0]], dtype=D)
        args = (torch.rand(4, generator=g, dtype=D), xI, torch.zeros(1, dtype=D))
    elif case == "heat_h8":
        fun = el.user_potential_element(el.heat_potential_integrand(1.0), 3, 8)
        xI = torch.tensor(mesh.structured_mesh((1, 1, 1), [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1],
                                                            [1, 0, 1], [1, 1, 1], [0, 1, 1]], "brick")[0], dtype=D)
        xI = xI[[0, 4, 6, 2, 1, 5, 7, 3]]
        args = (torch.rand(8, generator=g, dtype=D), xI, torch.tensor([2.5], dtype=D))
    elif case == "neo_q4":
        fun = el.hyperelastic_element(2, 4, 2, "plain strain")
        xI = torch.tensor([[0., 0.], [1.1, 0.1], [1.0, 0.9], [-0.1, 1.0]], dtype=D)
        args = (0.05 * torch.rand(4, 2, generator=g, dtype=D), xI, torch.tensor([10.0, 0.45], dtype=D))
    elif case == "neo_h8":
        fun = el.hyperelastic_element(3, 8, 2, "3d")
        c, e = mesh.structured_mesh((1, 1, 1), [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1],
                                                [1, 0, 1], [1, 1, 1], [0, 1, 1]], "brick")
        xI = torch.tensor(c[e[0]], dtype=D)
        args = (0.05 * torch.rand(8, 3, generator=g, dtype=D), xI, torch.tensor([1.0, 0.3], dtype=D))
    else:
        fun0 = el.nonlinear_heat_be_element(3, 8, 2)
        c, e = mesh.structured_mesh((1, 1, 1), [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1],
                                                [1, 0, 1], [1, 1, 1], [0, 1, 1]], "brick")
        xI = torch.tensor(c[e[0]], dtype=D)
        Tn = torch.rand(8, generator=g, dtype=D)
        p = torch.tensor([1.0, 0.5, 1.0, 1e-3], dtype=D)
        fun = lambda T, xI_, p_: fun0(T, Tn, xI_, p_)
        args = (torch.rand(8, generator=g, dtype=D), xI, p)
    assert _fd_check(fun, args) < 1e-7
