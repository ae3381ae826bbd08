"""GPU kernels against the CPU oracle on the same seeded inputs (parity proper).

Tolerances, written where they are used:
* float64 residuals:   ||R_gpu - R_oracle|| <= 1e-12 ||R_oracle||  (random, non-converged DOFs)
* float64 tangents:    max |K_gpu - K_oracle| <= 1e-12 max |K_oracle|
* float32 tangents:    max |K32 - K_oracle| <= 2e-6 max |K_oracle|
* Newton solutions:    ||u_gpu - u_oracle||_inf <= 1e-8 max(1, ||u_oracle||_inf), both converged
                       to the Newton tolerance (solver.py:899-903 semantics)
"""
import numpy as np
import pytest
import scipy.sparse

from autopdex_gb300 import configs
from oracle import newton
from oracle_setup import oracle_problem, oracle_settings

pytestmark = pytest.mark.gpu


def _flat(d):
    a = next(iter(d.values())) if isinstance(d, dict) else d
    return np.asarray(a, dtype=np.float64).reshape(-1)


def _like(w, flat):
    d = w.dofs
    if isinstance(d, dict):
        k = next(iter(d))
        return {k: flat.reshape(np.shape(d[k]))}
    return flat.reshape(np.shape(d))


def _random_dofs(w, scale, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(-scale, scale, w.n_dofs)


CASES = {
    "poisson": (lambda: configs.poisson(n=12), 1.0),
    "heat": (lambda: configs.heat_grf(n=10, seed=4), 1.0),
    "neo_hooke_3d": (lambda: configs.neo_hooke_cube(n=3, n_steps=2), 0.02),
    "cook": (lambda: configs.cook_membrane(n=6, n_steps=2), 0.05),
    "heat_be": (lambda: configs.heat_transient(n=3, n_steps=1), 1.0),
}


@pytest.mark.parametrize("case", list(CASES))
def test_residual_parity(case):
    from autopdex_gb300 import assembler
    make, scale = CASES[case]
    w = make()
    if case == "cook":
        w.settings["load multiplier"] = 0.03
    u = _random_dofs(w, scale)
    R_gpu = _flat(assembler.assemble_residual(_like(w, u), w.settings, w.static_settings))
    prob = oracle_problem(w)
    R_or = newton.assemble(prob.sets, u, prob.coords, oracle_settings(w), prob.n_dofs, tangent=False)[0]
    assert np.linalg.norm(R_gpu - R_or) <= 1e-12 * np.linalg.norm(R_or)


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_tangent_parity(case, dtype):
    from autopdex_gb300 import assembler
    make, scale = CASES[case]
    w = make()
    u = _random_dofs(w, scale, seed=1)
    K = assembler.assemble_tangent(_like(w, u), w.settings, w.static_settings, dtype=dtype).to_scipy()
    prob = oracle_problem(w)
    _, coo = newton.assemble(prob.sets, u, prob.coords, oracle_settings(w), prob.n_dofs)
    K_or = newton.scipy_assembling(coo, prob.n_dofs, None)
    diff = abs(K - K_or).max()
    tol = 1e-12 if dtype == "float64" else 2e-6
    assert diff <= tol * abs(K_or).max()


def test_dirichlet_elimination_matches_row_column_deletion():
    """Free-free block equals scipy_assembling's reduced matrix (solver.py:1214-1217);
    prescribed rows/columns are identity."""
    from autopdex_gb300 import assembler
    w = configs.cook_membrane(n=5, n_steps=2)
    u = _random_dofs(w, 0.05, seed=2)
    K = assembler.assemble_tangent(_like(w, u), w.settings, w.static_settings, eliminate_dirichlet=True).to_scipy()
    prob = oracle_problem(w)
    _, coo = newton.assemble(prob.sets, u, prob.coords, oracle_settings(w), prob.n_dofs)
    free = ~prob.dirichlet
    K_red = newton.scipy_assembling(coo, prob.n_dofs, free)
    assert abs(K[free][:, free] - K_red).max() <= 1e-12 * abs(K_red).max()
    d = prob.dirichlet
    Kd = K[d]
    assert np.array_equal(Kd.toarray(), scipy.sparse.eye(prob.n_dofs, format="csr")[d].toarray())


def test_golden_poisson_5x5_through_backend():
    """The reference's golden test (test_dicts_as_dofs_user_potential.py:63) with
    'solver backend': 'gb300'."""
    from autopdex_gb300 import solver
    w = configs.poisson(n=5, solver="lapack")
    sol, (it, res, div) = solver.solver(w.dofs, w.settings, w.static_settings)
    assert not div
    assert abs(sol["phi"].sum() - 1.9066412530282952) <= 1e-10 * 1.9066412530282952


@pytest.mark.parametrize("case", ["poisson", "heat"])
@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_linear_solve_matches_oracle(case, precision):
    from autopdex_gb300 import solver
    w = configs.poisson(n=40, precision=precision) if case == "poisson" else configs.heat_grf(n=32, seed=7,
                                                                                             precision=precision)
    sol, (it, res, div) = solver.solver(w.dofs, w.settings, w.static_settings, newton_tol=1e-10,
                                        newton_rtol=1e-12)
    assert not div
    prob = oracle_problem(w)
    ref, info, _ = newton.damped_newton(prob, np.zeros(w.n_dofs), oracle_settings(w), 1e-10)
    u = _flat(sol)
    assert np.abs(u - ref).max() <= 1e-8 * max(1.0, np.abs(ref).max())
    if precision == "mixed":
        assert it >= 2  # float32 inner solves refined by float64 Newton residuals


@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_neo_hooke_cube_load_steps_match_oracle(precision):
    from autopdex_gb300 import solver
    w = configs.neo_hooke_cube(n=3, n_steps=2, precision=precision)
    prob = oracle_problem(w)
    u_gpu = w.dofs
    u_or = np.zeros(w.n_dofs)
    for step in w.steps:
        w.settings = step(w.settings)
        prob.values = np.asarray(w.settings["dirichlet conditions"]).reshape(-1)
        u_gpu, (it, res, div) = solver.solver(u_gpu, w.settings, w.static_settings, newton_tol=1e-9)
        assert not div and res <= 1e-9
        u_or, info, _ = newton.damped_newton(prob, u_or, oracle_settings(w), 1e-9)
    assert np.abs(_flat(u_gpu) - u_or).max() <= 1e-8 * max(1.0, np.abs(u_or).max())


@pytest.mark.parametrize("precision", ["float64", "mixed"])
def test_cook_load_steps_match_oracle(precision):
    """Nearly incompressible (nu = 0.4999): the float64 residual floor is ~2e-9 here (the
    oracle stalls there too), so the reference's default tolerance 1e-8 is used."""
    from autopdex_gb300 import solver
    w = configs.cook_membrane(n=6, n_steps=2, precision=precision)
    prob = oracle_problem(w)
    u_gpu = w.dofs
    u_or = np.zeros(w.n_dofs)
    for step in w.steps:
        w.settings = step(w.settings)
        u_gpu, (it, res, div) = solver.solver(u_gpu, w.settings, w.static_settings, newton_tol=1e-8)
        assert not div and res <= 1e-8
        u_or, info, _ = newton.damped_newton(prob, u_or, oracle_settings(w), 1e-8)
    assert np.abs(_flat(u_gpu) - u_or).max() <= 1e-8 * max(1.0, np.abs(u_or).max())


def test_heat_backward_euler_step_matches_oracle():
    from autopdex_gb300 import solver
    w = configs.heat_transient(n=4, n_steps=1)
    prob = oracle_problem(w)
    sol, (it, res, div) = solver.solver(w.dofs, w.settings, w.static_settings, newton_tol=1e-10)
    assert not div
    ref, info, _ = newton.damped_newton(prob, w.raw["T0"].copy(), oracle_settings(w), 1e-10)
    assert np.abs(_flat(sol) - ref).max() <= 1e-8


def test_newton_reports_divergence_on_nan_input():
    """NaN DOFs (injected on the host) give the reference's diverged flag, no exception."""
    from autopdex_gb300 import solver
    w = configs.neo_hooke_cube(n=2, n_steps=1)
    w.settings = w.steps[0](w.settings)
    u = np.zeros((w.n_dofs // 3, 3))
    u[5, 1] = np.nan
    sol, (it, res, div) = solver.solver(u, w.settings, w.static_settings, maxiter=3)
    assert div


def test_newton_maxiter_stop():
    from autopdex_gb300 import solver
    w = configs.neo_hooke_cube(n=2, n_steps=1)
    w.settings = w.steps[0](w.settings)
    sol, (it, res, div) = solver.solver(w.dofs, w.settings, w.static_settings, newton_tol=1e-300, maxiter=1)
    assert it == 2 and div  # maxiter + 1 passes, then the forced stop (solver.py:926-930)


def test_all_dofs_prescribed():
    from autopdex_gb300 import solver
    w = configs.poisson(n=3)
    w.settings["dirichlet dofs"] = {"phi": np.ones(16, dtype=bool)}
    w.settings["dirichlet conditions"] = {"phi": np.arange(16.0)}
    sol, (it, res, div) = solver.solver(w.dofs, w.settings, w.static_settings)
    assert np.array_equal(sol["phi"], np.arange(16.0)) and res == 0.0 and not div


class _Foreign:
    """A minimal array of another framework: it exports DLPack and nothing torch knows."""

    def __init__(self, t):
        self._t = t
        self.shape = tuple(t.shape)

    def __dlpack__(self, stream=None, **kw):
        return self._t.__dlpack__()

    def __dlpack_device__(self):
        return self._t.__dlpack_device__()


def test_dlpack_inputs_match_numpy_path():
    """DOFs and Dirichlet values handed over as foreign DLPack arrays on the device give the
    same Newton solution as NumPy inputs; the result is a device tensor of the DOFs' shape
    and the caller's array is left unchanged."""
    import torch
    from autopdex_gb300 import solver
    w = configs.neo_hooke_cube(n=3, n_steps=2)
    w.settings = w.steps[0](w.settings)
    ref, (it0, res0, div0) = solver.solver(w.dofs, w.settings, w.static_settings, newton_tol=1e-10)
    d0 = torch.as_tensor(np.asarray(w.dofs), device="cuda")
    settings = dict(w.settings)
    settings["dirichlet conditions"] = _Foreign(torch.as_tensor(np.asarray(w.settings["dirichlet conditions"]),
                                                                device="cuda"))
    sol, (it, res, div) = solver.solver(_Foreign(d0), settings, w.static_settings, newton_tol=1e-10)
    assert not div and not div0 and it == it0
    assert isinstance(sol, torch.Tensor) and sol.is_cuda and tuple(sol.shape) == np.shape(w.dofs)
    assert np.abs(sol.cpu().numpy() - np.asarray(ref)).max() <= 1e-12 * max(1.0, np.abs(ref).max())
    assert torch.count_nonzero(d0) == 0


def _sheared_brick_heat_be(shape=(6, 5, 4), seed=3):
    """The 128^3 backward-Euler heat workload's model (configs.heat_transient) on a sheared,
    non-cubic brick grid: a parallelepiped lattice, so the assembly takes the uniform brick
    grid's kernels with a full (non-diagonal) Jacobian."""
    from autopdex_gb300 import mesher, models, seeder, spaces
    from autopdex_gb300.configs import Workload
    e1, e2, e3 = np.array([1.2, 0.1, 0.0]), np.array([0.3, 0.9, 0.2]), np.array([0.1, 0.2, 0.8])
    verts = np.array([0 * e1, e1, e1 + e2, e2, e3, e1 + e3, e1 + e2 + e3, e2 + e3])
    coords, elems = mesher.structured_mesh(shape, verts, "brick")
    nx, ny, nz = shape
    idx = np.arange(coords.shape[0])
    i, j, k = idx // ((ny + 1) * (nz + 1)), (idx // (nz + 1)) % (ny + 1), idx % (nz + 1)
    bnd = (i == 0) | (i == nx) | (j == 0) | (j == ny) | (k == 0) | (k == nz)
    rng = np.random.default_rng(seed)
    T0 = rng.uniform(0.0, 1.0, coords.shape[0])
    T0[bnd] = 0.0
    dt = 1e-3
    integrand = models.heat_backward_euler_integrand(1.0, 0.5, 1.0, "time increment", "dofs n")
    model = models.mixed_reference_domain_residual(integrand, {"T": spaces.fem_iso_line_quad_brick},
                                                   *seeder.gauss_legendre_nd(3, 2), "T")
    static = {"assembling mode": ("user residual",), "solution structure": ("nodal imposition",),
              "model": (model,), "solver type": "newton", "solver backend": "gb300", "solver": "pcg",
              "precision": "mixed", "verbose": -1}
    settings = {"connectivity": ({"T": elems},), "dirichlet dofs": {"T": bnd}, "node coordinates": {"T": coords},
                "dirichlet conditions": {"T": np.zeros(coords.shape[0])}, "dofs n": {"T": T0.copy()},
                "time increment": dt}
    raw = dict(coords=coords, conns=[elems], dirichlet=bnd, values=np.zeros(coords.shape[0]), T0=T0, dt=dt,
               kind="heat_be", n_steps=1)
    return Workload("heat_be_sheared_brick", {"T": T0.copy()}, settings, static, raw)


def test_sheared_brick_grid_residual_and_float32_tangent_match_oracle():
    """The uniform brick grid's float64 residual (sum-factorised) and float32 row-gathered
    tangent against the oracle at random DOFs; tolerances as above (1e-12 and 2e-6)."""
    from autopdex_gb300 import assembler
    w = _sheared_brick_heat_be()
    u = _random_dofs(w, 1.0, seed=5)
    R_gpu = _flat(assembler.assemble_residual(_like(w, u), w.settings, w.static_settings))
    prob = oracle_problem(w)
    R_or, coo = newton.assemble(prob.sets, u, prob.coords, oracle_settings(w), prob.n_dofs)
    assert np.linalg.norm(R_gpu - R_or) <= 1e-12 * np.linalg.norm(R_or)
    K = assembler.assemble_tangent(_like(w, u), w.settings, w.static_settings, dtype="float32").to_scipy()
    K_or = newton.scipy_assembling(coo, prob.n_dofs, None)
    assert abs(K - K_or).max() <= 2e-6 * abs(K_or).max()
    Kd = assembler.assemble_tangent(_like(w, u), w.settings, w.static_settings, dtype="float32",
                                    eliminate_dirichlet=True).to_scipy()
    free = ~prob.dirichlet
    K_red = newton.scipy_assembling(coo, prob.n_dofs, free)
    assert abs(Kd[free][:, free] - K_red).max() <= 2e-6 * abs(K_red).max()
    assert np.array_equal(Kd[prob.dirichlet].toarray(),
                          scipy.sparse.eye(prob.n_dofs, format="csr")[prob.dirichlet].toarray())
