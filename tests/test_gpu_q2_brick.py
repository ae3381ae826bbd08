"""27-node (Q2) bricks on the GPU against the oracle: the Poisson potential and neo-Hooke on a 2 x 2 x 2
mesh of a trilinearly distorted cube with 3 x 3 x 3 Gauss points, float64 residual and tangent
to 1e-12 and float32 tangent to 5e-6 of the oracle's at random DOFs, and a Newton solve to
the oracle's solution."""
import numpy as np
import pytest

from autopdex_gb300 import assembler, models, seeder, solver, spaces

pytestmark = pytest.mark.gpu


def _mesh(n=2):
    from oracle.mesh import HEX27_NODES
    m = 2 * n + 1
    g = np.linspace(0.0, 1.0, m)
    P, Q, R = np.meshgrid(g, g, g, indexing="ij")
    u = np.stack([P.ravel(), Q.ravel(), R.ravel()], axis=1)
    x = u + 0.08 * u[:, [1]] * u[:, [2]] * np.array([1.0, -0.5, 0.3])  # a non-affine trilinear map
    idx = np.array(HEX27_NODES)
    conn = []
    for i in range(n):
        for j in range(n):
            for k in range(n):
                conn.append(((2 * i + idx[:, 0]) * m + 2 * j + idx[:, 1]) * m + 2 * k + idx[:, 2])
    return x, np.array(conn)


def _problem():
    from oracle import elements as el, newton
    x, conn = _mesh()
    n = x.shape[0]
    fixed = np.abs(x[:, 0]) < 1e-12
    rule = seeder.gauss_legendre_nd(3, 4)
    pot = models.mixed_reference_domain_potential(models.poisson_sincos_integrand(20.0, 10.0, (1.0, 0.5, 0.2)),
                                                  {"phi": spaces.fem_iso_line_quad_brick}, *rule, "phi")
    static = {"assembling mode": ("user potential",), "solution structure": ("nodal imposition",),
              "model": (pot,), "solver type": "newton", "solver backend": "gb300", "solver": "pcg", "verbose": -1}
    settings = {"dirichlet dofs": {"phi": fixed}, "connectivity": ({"phi": conn},), "node coordinates": {"phi": x},
                "dirichlet conditions": {"phi": np.zeros(n)}}
    fun = el.user_potential_element(el.poisson_sincos_integrand(20.0, 10.0, (1.0, 0.5, 0.2)), 3, 27, order=4)
    s1 = newton.ElementSet("potential", conn, fun, lambda st: np.zeros((conn.shape[0], 1)), 1)
    return static, settings, newton.Problem([s1], x, n, fixed, np.zeros(n))


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_q2_brick_parity(dtype):
    from oracle import newton
    static, settings, prob = _problem()
    u = np.random.default_rng(7).uniform(-0.5, 0.5, prob.n_dofs)
    R_or, coo = newton.assemble(prob.sets, u, prob.coords, {}, prob.n_dofs)
    K_or = newton.scipy_assembling(coo, prob.n_dofs, None)
    if dtype == "float64":
        R = np.asarray(assembler.assemble_residual({"phi": u}, settings, static)["phi"]).reshape(-1)
        assert np.linalg.norm(R - R_or) <= 1e-12 * np.linalg.norm(R_or)
    K = assembler.assemble_tangent({"phi": u}, settings, static, dtype=dtype).to_scipy()
    tol = 1e-12 if dtype == "float64" else 5e-6
    assert abs(K - K_or).max() <= tol * abs(K_or).max()


def test_q2_brick_newton_matches_oracle():
    from oracle import newton
    static, settings, prob = _problem()
    sol, (it, res, div) = solver.solver({"phi": np.zeros(prob.n_dofs)}, settings, static, newton_tol=1e-10)
    assert not div
    ref, info, _ = newton.damped_newton(prob, np.zeros(prob.n_dofs), {}, 1e-10)
    u = np.asarray(sol["phi"])
    assert np.abs(u - ref).max() <= 1e-8 * max(1.0, np.abs(ref).max())


def _neo_hooke_problem():
    """Neo-Hooke (E = 1, nu = 0.3) on the same 27-node brick mesh with 3 x 3 x 3 Gauss points,
    x = 0 clamped, u_x = 0.02 prescribed on x = 1."""
    from oracle import elements as el, newton
    x, conn = _mesh()
    n = x.shape[0]
    mask = np.zeros((n, 3), dtype=bool)
    mask[np.abs(x[:, 0]) < 1e-12, :] = True
    right = np.abs(x[:, 0] - x[:, 0].max()) < 1e-12
    mask[right, 0] = True
    vals = np.zeros((n, 3))
    vals[right, 0] = 0.02
    weak = models.hyperelastic_steady_state_weak(models.neo_hooke, 1.0, 0.3, "3d")
    dom = models.isoparametric_domain_element_galerkin(weak, spaces.fem_iso_line_quad_brick,
                                                       *seeder.gauss_legendre_nd(3, 4))
    static = {"assembling mode": ("user element",), "solution structure": ("nodal imposition",), "model": (dom,),
              "solver type": "newton", "solver backend": "gb300", "solver": "pcg", "verbose": -1}
    settings = {"dirichlet dofs": mask, "connectivity": (conn,), "node coordinates": x, "dirichlet conditions": vals}
    fun = el.hyperelastic_element(3, 27, 4, "3d")
    s1 = newton.ElementSet("element", conn, fun, lambda st: np.tile([1.0, 0.3], (conn.shape[0], 1)), 3)
    return static, settings, newton.Problem([s1], x, 3 * n, mask.reshape(-1), vals.reshape(-1))


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_q2_brick_neo_hooke_parity(dtype):
    """The 27-node brick's neo-Hooke residual and tangent (assembled in column chunks) against
    the oracle's AD element at random displacements."""
    from oracle import newton
    static, settings, prob = _neo_hooke_problem()
    u = np.random.default_rng(8).uniform(-0.01, 0.01, prob.n_dofs)
    R_or, coo = newton.assemble(prob.sets, u, prob.coords, {}, prob.n_dofs)
    K_or = newton.scipy_assembling(coo, prob.n_dofs, None)
    if dtype == "float64":
        R = np.asarray(assembler.assemble_residual(u.reshape(-1, 3), settings, static)).reshape(-1)
        assert np.linalg.norm(R - R_or) <= 1e-12 * np.linalg.norm(R_or)
    K = assembler.assemble_tangent(u.reshape(-1, 3), settings, static, dtype=dtype).to_scipy()
    tol = 1e-12 if dtype == "float64" else 5e-6
    assert abs(K - K_or).max() <= tol * abs(K_or).max()


def test_q2_brick_neo_hooke_newton_matches_oracle():
    from oracle import newton
    static, settings, prob = _neo_hooke_problem()
    n = prob.n_dofs // 3
    sol, (it, res, div) = solver.solver(np.zeros((n, 3)), settings, static, newton_tol=1e-10)
    assert not div
    ref, info, _ = newton.damped_newton(prob, np.zeros(prob.n_dofs), {}, 1e-10)
    assert np.abs(np.asarray(sol).reshape(-1) - ref).max() <= 1e-8 * max(1.0, np.abs(ref).max())
