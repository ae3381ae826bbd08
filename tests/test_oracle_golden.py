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


def test_golden_q2_cook_neo_hooke():
    """tests/test_user_elem_impl_diff_and_adaptive_load_step.py:153-155 -> dofs.dofs =
    19390.35027108 and its derivatives -216.0310416 (E) and -1859.43760286 (nu) (Q2 user
    element, neo-Hooke plane strain, Neumann traction 20, load stepping to 1)."""
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
    g = GOLDEN["cook_q2_dofs_dot_dofs"]["value"]
    assert abs(dofs @ dofs - g) <= 1e-9 * g
    # first derivatives of u.u in E and nu by implicit differentiation at the final state
    # (the golden values carry 10 and 12 significant digits)
    for key, name in (("E", "cook_q2_d_dofs_dot_dofs_d_youngs_modulus"),
                      ("nu", "cook_q2_d_dofs_dot_dofs_d_poisson_ratio")):
        du = newton.implicit_sensitivity(prob, dofs, st, key)
        ref = GOLDEN[name]["value"]
        assert abs(2.0 * dofs @ du - ref) <= 1e-7 * abs(ref), (key, 2.0 * dofs @ du, ref)


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
