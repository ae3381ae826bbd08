"""The reference's own Q2 golden case through the GPU backend.

tests/test_user_elem_impl_diff_and_adaptive_load_step.py:153-155 of AutoPDEx: a Cook membrane
of 12 nine-node quads (3 x 3 Gauss points) under a 20-unit shear traction on 3-node lines,
neo-Hooke plane strain with E = 100 and nu = 0.3, adaptive load stepping with Newton to 1e-8.
The reference asserts u.u = 19390.35027108 and, by forward implicit differentiation,
d(u.u)/dE = -216.0310416 and d(u.u)/dnu = -1859.43760286.  Here the same settings dicts go
through ``solver.adaptive_load_stepping`` and ``solver.sensitivities`` of this backend; the
tolerances are those of the golden values' printed digits (1e-9 and 1e-7 relative).
"""
import json
import os

import numpy as np
import pytest

from autopdex_gb300 import geometry, models, seeder, solver, spaces, utility

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _cook_golden_setup():
    """Settings dicts of the reference's golden Q2 Cook case, for this backend."""
    d = np.load(os.path.join(HERE, "golden", "cook_q2_mesh.npz"))
    x_nodes, elements, surface = d["x_nodes"], d["elements"], d["surface_elements"]
    pts = [[0., 0.], [48., 44.], [48., 60.], [0., 44.]]
    dirichlet_nodes = geometry.in_planes(x_nodes, pts[0], [1., 0.])
    dirichlet_dofs = utility.dof_select(dirichlet_nodes, np.asarray([True, True]))
    neumann = surface[geometry.select_elements_in_plane(x_nodes, surface, pts[1], [1., 0.])]
    weak = models.hyperelastic_steady_state_weak(models.neo_hooke, lambda x, s: s["youngs modulus"],
                                                 lambda x, s: s["poisson ratio"], "plain strain")
    dom = models.isoparametric_domain_element_galerkin(weak, spaces.fem_iso_line_quad_brick,
                                                       *seeder.gauss_legendre_nd(dimension=2, order=4))
    q0 = 20.0
    trac = models.isoparametric_surface_element_galerkin(
        models.neumann_weak(lambda x, s: np.asarray([0., s["load multiplier"]])), spaces.fem_iso_line_quad_brick,
        *seeder.gauss_legendre_nd(dimension=1, order=4), tangent_contributions=False)

    def multiplier_settings(settings, multiplier):
        settings["load multiplier"] = multiplier * q0
        return settings

    static = {"number of fields": (2, 2), "assembling mode": ("user element", "user element"),
              "solution structure": ("nodal imposition", "nodal imposition"), "model": (dom, trac),
              "solver type": "newton", "solver backend": "gb300", "solver": "lapack", "verbose": -1}
    settings = {"dirichlet dofs": dirichlet_dofs, "connectivity": (elements, neumann), "load multiplier": q0,
                "node coordinates": x_nodes, "dirichlet conditions": np.zeros_like(dirichlet_dofs, dtype=np.float64),
                "youngs modulus": 100., "poisson ratio": 0.3}
    dofs0 = np.zeros((x_nodes.shape[0], 2))
    return static, settings, multiplier_settings, dofs0


def _cook_golden_solution():
    static, settings, multiplier_settings, dofs0 = _cook_golden_setup()
    dofs, mult, *_ = solver.adaptive_load_stepping(dofs0, settings, static, multiplier_settings, False,
                                                   newton_tol=1e-8)
    assert abs(mult - 1.0) < 1e-12
    return static, multiplier_settings(dict(settings), 1.0), dofs


def test_q2_cook_golden_and_sensitivities():
    golden = json.load(open(os.path.join(HERE, "golden", "golden.json")))
    static, settings, dofs = _cook_golden_solution()
    u = np.asarray(dofs).reshape(-1)
    g = golden["cook_q2_dofs_dot_dofs"]["value"]
    assert abs(u @ u - g) <= 1e-9 * g, u @ u
    sens = solver.sensitivities(dofs, settings, static, ["youngs modulus", "poisson ratio"])
    for key, name in (("youngs modulus", "cook_q2_d_dofs_dot_dofs_d_youngs_modulus"),
                      ("poisson ratio", "cook_q2_d_dofs_dot_dofs_d_poisson_ratio")):
        du = np.asarray(sens[key]).reshape(-1)
        ref = golden[name]["value"]
        assert abs(2.0 * u @ du - ref) <= 1e-7 * abs(ref), (key, 2.0 * u @ du, ref)


def test_sensitivity_of_a_linear_problem_is_exact():
    """Heat with a source given by a settings entry s: R = K u - s f, so du/ds = u / s; the
    residual is linear in s and the central difference is exact up to rounding."""
    from autopdex_gb300 import configs
    w = configs.heat_grf(n=48, seed=3)
    integrand = models.heat_conduction_integrand("conductivity", "source")
    model = models.mixed_reference_domain_potential(integrand, {"T": spaces.fem_iso_line_quad_brick},
                                                    *seeder.gauss_legendre_nd(2, 2), "T")
    static = dict(w.static_settings, model=(model,), solver="pcg", precision="float64")
    settings = dict(w.settings, source=2.5)
    sol, info = solver.solver(w.dofs, settings, static, newton_tol=0.0, newton_rtol=1e-12, krylov_tol=1e-13)
    assert not info[2]
    du = solver.sensitivities(sol, settings, static, ["source"])["source"]
    u = np.asarray(sol["T"])
    assert np.abs(np.asarray(du["T"]) - u / 2.5).max() <= 1e-9 * np.abs(u / 2.5).max()


def _q2_problem(kind):
    """The golden Q2 Cook mesh with (a) the neo-Hooke element and traction lines or (b) the
    Poisson user potential; GPU settings and the oracle problem for the same inputs."""
    from oracle import elements as el, newton
    d = np.load(os.path.join(HERE, "golden", "cook_q2_mesh.npz"))
    x, E9, S = d["x_nodes"], d["elements"], d["surface_elements"]
    pts = [[0., 0.], [48., 44.], [48., 60.], [0., 44.]]
    dn = geometry.in_planes(x, pts[0], [1., 0.])
    NE = S[geometry.select_elements_in_plane(x, S, pts[1], [1., 0.])]
    if kind == "neo_hooke":
        weak = models.hyperelastic_steady_state_weak(models.neo_hooke, 100., 0.3, "plain strain")
        dom = models.isoparametric_domain_element_galerkin(weak, spaces.fem_iso_line_quad_brick,
                                                           *seeder.gauss_legendre_nd(2, 4))
        trac = models.isoparametric_surface_element_galerkin(
            models.neumann_weak(lambda x_, s: np.asarray([0., s["load multiplier"]])), spaces.fem_iso_line_quad_brick,
            *seeder.gauss_legendre_nd(1, 4), tangent_contributions=False)
        dd = utility.dof_select(dn, np.asarray([True, True]))
        static = {"assembling mode": ("user element", "user element"),
                  "solution structure": ("nodal imposition", "nodal imposition"), "model": (dom, trac),
                  "solver type": "newton", "solver backend": "gb300", "verbose": -1}
        settings = {"dirichlet dofs": dd, "connectivity": (E9, NE), "node coordinates": x, "load multiplier": 7.0,
                    "dirichlet conditions": np.zeros_like(dd, dtype=np.float64)}
        s1 = newton.ElementSet("element", E9, el.hyperelastic_element(2, 9, 4, "plain strain"),
                               lambda st: np.tile([100., 0.3], (E9.shape[0], 1)), 2)
        s2 = newton.ElementSet("neumann", NE, el.neumann_line_element(3, 4), None, 2,
                               traction=lambda st: np.array([0., st["load multiplier"]]))
        prob = newton.Problem([s1, s2], x, x.shape[0] * 2, dd, np.zeros(x.shape[0] * 2))
        shape = (x.shape[0], 2)
    else:
        pot = models.mixed_reference_domain_potential(models.poisson_sincos_integrand(), {"phi": spaces.fem_iso_line_quad_brick},
                                                      *seeder.gauss_legendre_nd(2, 4), "phi")
        xs = x / 48.0  # the source oscillates on the unit scale
        static = {"assembling mode": ("user potential",), "solution structure": ("nodal imposition",),
                  "model": (pot,), "solver type": "newton", "solver backend": "gb300", "verbose": -1}
        settings = {"dirichlet dofs": {"phi": dn}, "connectivity": ({"phi": E9},), "node coordinates": {"phi": xs},
                    "dirichlet conditions": {"phi": np.zeros(x.shape[0])}}
        fun = el.user_potential_element(el.poisson_sincos_integrand(), 2, 9, order=4)
        s1 = newton.ElementSet("potential", E9, fun, lambda st: np.zeros((E9.shape[0], 1)), 1)
        prob = newton.Problem([s1], xs, x.shape[0], dn, np.zeros(x.shape[0]))
        shape = None
    return static, settings, prob, shape


@pytest.mark.parametrize("kind", ["neo_hooke", "poisson"])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_q2_element_parity(kind, dtype):
    """Nine-node quads and three-node lines with 3-point Gauss rules: float64 residuals to
    1e-12, float64 tangents to 1e-12 and float32 tangents to 2e-6 of the oracle's, at random
    (non-converged) DOFs."""
    from autopdex_gb300 import assembler
    from oracle import newton
    static, settings, prob, shape = _q2_problem(kind)
    u = np.random.default_rng(4).uniform(-0.5, 0.5, prob.n_dofs)
    dofs = u.reshape(shape) if shape else {"phi": u}
    st = {"load multiplier": 7.0}
    R_or, coo = newton.assemble(prob.sets, u, prob.coords, st, prob.n_dofs)
    K_or = newton.scipy_assembling(coo, prob.n_dofs, None)
    if dtype == "float64":
        R = assembler.assemble_residual(dofs, settings, static)
        R = np.asarray(R if shape else R["phi"], dtype=np.float64).reshape(-1)
        assert np.linalg.norm(R - R_or) <= 1e-12 * np.linalg.norm(R_or)
    K = assembler.assemble_tangent(dofs, settings, static, dtype=dtype).to_scipy()
    tol = 1e-12 if dtype == "float64" else 2e-6
    assert abs(K - K_or).max() <= tol * abs(K_or).max()


def test_q2_cook_second_order_and_adjoint():
    """The reference's second-order golden values (lines 156-159: d2(u.u)/dE2 = 4.17157824,
    d2/dE dnu = d2/dnu dE = -51.42695148, d2/dnu2 = -45854.7002203) from
    ``solver.second_order_sensitivities`` -- d2(u.u)/dp dq = 2 (u_p . u_q + u . u_pq) -- and
    the first derivatives again by one adjoint solve (``solver.adjoint_sensitivities`` with
    dJ/du = 2u), which the reference checks in 'backward' mode (lines 169-170).  Tolerance
    1e-6 relative (the reference's own allclose uses 1e-5)."""
    golden = json.load(open(os.path.join(HERE, "golden", "golden.json")))
    static, settings, dofs = _cook_golden_solution()
    keys = ["youngs modulus", "poisson ratio"]
    first, second = solver.second_order_sensitivities(dofs, settings, static, keys)
    u = np.asarray(dofs).reshape(-1)
    du = {k: np.asarray(first[k]).reshape(-1) for k in keys}
    name = {"youngs modulus": "youngs_modulus", "poisson ratio": "poisson_ratio"}
    assert len(second) == 4
    for (a, b), v in second.items():
        val = 2.0 * (du[a] @ du[b] + u @ np.asarray(v).reshape(-1))
        ref = golden["cook_q2_d2_dofs_dot_dofs_d_%s_%s" % (name[a], name[b])]["value"]
        assert abs(val - ref) <= 1e-6 * abs(ref), (a, b, val, ref)
    adj = solver.adjoint_sensitivities(dofs, settings, static, keys, 2.0 * np.asarray(dofs))
    for k in keys:
        ref = golden["cook_q2_d_dofs_dot_dofs_d_" + name[k]]["value"]
        assert abs(adj[k] - ref) <= 1e-7 * abs(ref), (k, adj[k], ref)
