"""The other entry points of the solve path against the CPU oracle: the 'linear' solver type
(solver.py:544-659), assemble_tangent_diagonal (assembler.py:639-680) and time stepping
through the manager (dae.py:1734-2283) stepped like the oracle's Newton solve.

Tolerances, written where they are used:
* linear solve:     ||u_gpu - u_oracle||_inf <= 1e-9 max(1, ||u_oracle||_inf) (Krylov to 1e-13
                    against SciPy's spsolve)
* tangent diagonal: max |d_gpu - d_oracle| <= 1e-12 max |d_oracle| (float64), 2e-6 (float32)
* trajectories:     max |T_gpu - T_oracle| <= 1e-8 after three steps, both Newton solves to
                    1e-10
"""
import numpy as np
import pytest

from autopdex_gb300 import configs
from oracle import newton
from oracle_setup import oracle_problem, oracle_settings

pytestmark = pytest.mark.gpu

CASES = {
    "poisson": (lambda: configs.poisson(n=12), 1.0),
    "heat": (lambda: configs.heat_grf(n=10, seed=4), 1.0),
    "neo_hooke_3d": (lambda: configs.neo_hooke_cube(n=3, n_steps=2), 0.02),
    "cook": (lambda: configs.cook_membrane(n=6, n_steps=2), 0.05),
    "heat_be": (lambda: configs.heat_transient(n=3, n_steps=1), 1.0),
}


def _flat(d):
    a = next(iter(d.values())) if isinstance(d, dict) else d
    return np.asarray(a, dtype=np.float64).reshape(-1)


def _like(w, flat):
    d = w.dofs
    if isinstance(d, dict):
        k = next(iter(d))
        return {k: flat.reshape(np.shape(d[k]))}
    return flat.reshape(np.shape(d))


@pytest.mark.parametrize("case", ["poisson", "neo_hooke_3d", "cook"])
def test_solver_type_linear_matches_oracle(case):
    """'solver type': 'linear' returns the increment on free DOFs and the prescribed values on
    Dirichlet DOFs (solver.py:612-659), from a non-zero state for the nonlinear models."""
    from autopdex_gb300 import solver
    make, scale = CASES[case]
    w = make()
    if w.steps:
        w.settings = w.steps[-1](w.settings)
    static = dict(w.static_settings, **{"solver type": "linear", "solver": "lapack"})
    # small states for the nearly incompressible membrane: far from equilibrium its tangent is
    # indefinite (lam / mu = 5000) and the direct solve, a Cholesky factorization, refuses it
    u0 = np.random.default_rng(3).uniform(-scale, scale, w.n_dofs) * {"poisson": 0.0, "neo_hooke_3d": 0.2,
                                                                       "cook": 2e-4}[case]
    sol, info = solver.solver(_like(w, u0), w.settings, static, krylov_tol=1e-13)
    assert info is None
    prob = oracle_problem(w)
    prob.values = _flat(w.settings["dirichlet conditions"]) if w.settings.get("dirichlet conditions") is not None \
        else prob.values
    ref = prob.solve_linear(u0.copy(), oracle_settings(w))
    u = _flat(sol)
    assert np.abs(u - ref).max() <= 1e-9 * max(1.0, np.abs(ref).max())
    d = prob.dirichlet
    assert np.array_equal(u[d], prob.values[d])


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_assemble_tangent_diagonal_matches_oracle(case, dtype):
    from autopdex_gb300 import assembler
    make, scale = CASES[case]
    w = make()
    if case == "cook":
        w.settings["load multiplier"] = 0.03
    u = np.random.default_rng(5).uniform(-scale, scale, w.n_dofs)
    d = np.asarray(assembler.assemble_tangent_diagonal(_like(w, u), w.settings, w.static_settings, dtype=dtype))
    prob = oracle_problem(w)
    _, coo = newton.assemble(prob.sets, u, prob.coords, oracle_settings(w), prob.n_dofs)
    d_or = newton.scipy_assembling(coo, prob.n_dofs, None).diagonal()
    assert d.shape == (w.n_dofs,)
    tol = 1e-12 if dtype == "float64" else 2e-6
    assert np.abs(d - d_or).max() <= tol * np.abs(d_or).max()


def _oracle_steps(w, k_steps, n_steps, dt):
    """The oracle's damped Newton stepped as a k-step BDF in backward-Euler form:
    (q - q*) / (dt / c_0) with q* = -sum_i c_i q_(n+1-i) / c_0, the history started from the
    initial state (dae.py:537-587)."""
    from autopdex_gb300 import dae
    c = dae.BackwardDiffFormula(k_steps).coeffs if k_steps > 1 else (1.0, -1.0)
    prob = oracle_problem(w)
    st = oracle_settings(w)
    hist = [w.raw["T0"].copy()] * k_steps
    for _ in range(n_steps):
        q_star = -sum(c[i + 1] * hist[i] for i in range(k_steps)) / c[0]
        st["dofs n"] = q_star
        st["time increment"] = dt / c[0]
        T, info, _ = newton.damped_newton(prob, hist[0].copy(), st, 1e-10)
        assert not info[2]
        hist = [T] + hist[:-1]
    return hist[0]


@pytest.mark.parametrize("k_steps", [1, 2])
def test_time_stepping_trajectory_matches_oracle(k_steps):
    """Backward Euler and BDF2 through dae.TimeSteppingManager on the 3-D nonlinear heat
    problem (8^3 bricks, three steps) against the oracle's Newton solves of the same steps."""
    from autopdex_gb300 import dae
    w = configs.heat_transient(n=8, n_steps=3, dt=1e-3)
    dt = w.raw["dt"]
    integ = dae.BackwardEuler() if k_steps == 1 else dae.BackwardDiffFormula(k_steps)
    static = dict(w.static_settings, **{"time integrators": {"T": integ}})
    st = dae.TimeSteppingManager(static, newton_tol=1e-10).run({"T": w.raw["T0"].copy()}, dt, 3 * dt, 5,
                                                              settings=dict(w.settings))
    assert st.num_accepted == 3 and st.num_rejected == 0
    ref = _oracle_steps(w, k_steps, 3, dt)
    assert np.abs(np.asarray(st.q["T"]) - ref).max() <= 1e-8
