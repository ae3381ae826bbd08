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


def test_q2_cook_golden_and_sensitivities():
    golden = json.load(open(os.path.join(HERE, "golden", "golden.json")))
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
    dofs, mult, *_ = solver.adaptive_load_stepping(dofs0, settings, static, multiplier_settings, False,
                                                   newton_tol=1e-8)
    assert abs(mult - 1.0) < 1e-12
    u = np.asarray(dofs).reshape(-1)
    g = golden["cook_q2_dofs_dot_dofs"]["value"]
    assert abs(u @ u - g) <= 1e-9 * g, u @ u
    settings = multiplier_settings(dict(settings), 1.0)
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
