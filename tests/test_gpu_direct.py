"""The direct-solver names ('lapack', 'umfpack', 'direct', 'cholesky') run the GPU banded
Cholesky factorization of the float64 tangent: the role of spsolve in linear_solve_scipy
(solver.py:1493-1539).  Checked against SciPy's spsolve on the reduced matrix and against the
oracle's Newton solve, which uses spsolve.

Tolerances, written where they are used:
* linear solves:    ||x_gpu - x_spsolve||_inf <= 1e-11 ||x_spsolve||_inf, relative residual
                    <= 1e-13 after refinement
* Newton solutions: ||u_gpu - u_oracle||_inf <= 1e-10 max(1, ||u_oracle||_inf)
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from autopdex_gb300 import configs
from oracle import newton
from oracle_setup import oracle_problem, oracle_settings

pytestmark = pytest.mark.gpu


def _flat(d):
    a = next(iter(d.values())) if isinstance(d, dict) else d
    return np.asarray(a, dtype=np.float64).reshape(-1)


@pytest.mark.parametrize("case", ["poisson", "cook", "neo_hooke_3d"])
def test_direct_solve_matches_spsolve(case):
    """agx_solve with AGX_CHOL_BAND on the eliminated float64 tangent at a random state,
    against spsolve on scipy_assembling's reduced matrix (solver.py:1180-1222)."""
    import torch
    from autopdex_gb300 import _native as N
    from autopdex_gb300._problem import get_problem
    w = {"poisson": lambda: configs.poisson(n=30), "cook": lambda: configs.cook_membrane(n=12, n_steps=2),
         "neo_hooke_3d": lambda: configs.neo_hooke_cube(n=4, n_steps=2)}[case]()
    # small random states: with lam / mu = 5000 (Cook, nu = 0.4999) larger ones make the tangent
    # indefinite (pressure stiffness of a far-from-equilibrium state), and Cholesky rightly fails
    scale = {"poisson": 1.0, "cook": 1e-5, "neo_hooke_3d": 0.005}[case]
    rng = np.random.default_rng(11)
    u = rng.uniform(-scale, scale, w.n_dofs)
    if case == "cook":
        w.settings["load multiplier"] = 0.03
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    x_dev = torch.as_tensor(u, device=prob.device)
    prob._call("agx_assemble", N.C.c_void_p(x_dev.data_ptr()), None, N.AGX_F64)
    b = rng.standard_normal(w.n_dofs)
    free = ~prob.mask.astype(bool)
    b[~free] = 0.0
    b_dev = torch.as_tensor(b, device=prob.device)
    x = torch.empty_like(b_dev)
    opts = N.SolveOpts()
    # the membrane's condition number (~1e8 at nu = 0.4999) bounds the attainable float64
    # relative residual near 1e-11 and the agreement of two backward-stable solvers near 1e-8
    rtol, xtol = {"poisson": (1e-13, 1e-11), "cook": (1e-10, 1e-7), "neo_hooke_3d": (1e-13, 1e-11)}[case]
    opts.method, opts.rtol, opts.atol, opts.maxiter, opts.check_every = N.AGX_CHOL_BAND, rtol, 0.0, 10, 1
    info = N.SolveInfo()
    rc = prob._call("agx_solve", N.C.c_void_p(b_dev.data_ptr()), N.C.c_void_p(x.data_ptr()), N.C.byref(opts),
                    N.C.byref(info))
    assert rc == N.AGX_OK and info.status == N.AGX_OK and info.rel_residual <= rtol, (rc, info.rel_residual)
    op = oracle_problem(w)
    _, coo = newton.assemble(op.sets, u, op.coords, oracle_settings(w), op.n_dofs)
    A = newton.scipy_assembling(coo, op.n_dofs, free)
    ref = spla.spsolve(A.tocsc(), b[free])
    got = x.cpu().numpy()
    rel_sp = np.linalg.norm(A @ ref - b[free]) / np.linalg.norm(b[free])
    assert info.rel_residual <= max(rtol, 10.0 * rel_sp)
    assert np.abs(got[free] - ref).max() <= xtol * np.abs(ref).max()
    assert np.all(got[~free] == 0.0)


@pytest.mark.parametrize("name", ["lapack", "umfpack"])
def test_poisson_one_newton_step_direct(name):
    """The 200^2-style Poisson workload (here 60^2) with a direct solver name: one Newton step
    reaches the solution of the oracle's spsolve-based Newton."""
    from autopdex_gb300 import solver
    w = configs.poisson(n=60, solver=name)
    sol, (it, res, div) = solver.solver(w.dofs, w.settings, w.static_settings, newton_tol=1e-10)
    assert not div and it == 1
    ref, info, _ = newton.damped_newton(oracle_problem(w), np.zeros(w.n_dofs), oracle_settings(w), 1e-10)
    assert np.abs(_flat(sol) - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())


def test_cook_load_step_direct_matches_oracle():
    """Nearly incompressible membrane (nu = 0.4999), load step 1 of 2, Newton with the direct
    solve against the oracle's Newton with spsolve (both to the reference's default 1e-8)."""
    from autopdex_gb300 import solver
    w = configs.cook_membrane(n=16, n_steps=2, solver="lapack")
    w.settings = w.steps[0](w.settings)
    sol, (it, res, div) = solver.solver(w.dofs, w.settings, w.static_settings, newton_tol=1e-8)
    assert not div and res <= 1e-8
    ref, info, _ = newton.damped_newton(oracle_problem(w), np.zeros(w.n_dofs), oracle_settings(w), 1e-8)
    assert np.abs(_flat(sol) - ref).max() <= 1e-8 * max(1.0, np.abs(ref).max())


def test_indefinite_tangent_reports_breakdown():
    """A far-from-equilibrium state of the nearly incompressible membrane has an indefinite
    tangent: the factorization reports AGX_DIVERGED (no exception, no garbage solution
    claimed as converged)."""
    import torch
    from autopdex_gb300 import _native as N
    from autopdex_gb300._problem import get_problem
    w = configs.cook_membrane(n=12, n_steps=2)
    u = np.random.default_rng(11).uniform(-0.05, 0.05, w.n_dofs)
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    x_dev = torch.as_tensor(u, device=prob.device)
    prob._call("agx_assemble", N.C.c_void_p(x_dev.data_ptr()), None, N.AGX_F64)
    b = torch.ones(w.n_dofs, dtype=torch.float64, device=prob.device)
    x = torch.empty_like(b)
    opts = N.SolveOpts()
    opts.method, opts.rtol, opts.atol, opts.maxiter, opts.check_every = N.AGX_CHOL_BAND, 1e-13, 0.0, 10, 1
    info = N.SolveInfo()
    rc = prob._call("agx_solve", N.C.c_void_p(b.data_ptr()), N.C.c_void_p(x.data_ptr()), N.C.byref(opts),
                    N.C.byref(info))
    assert rc == N.AGX_DIVERGED and info.status == N.AGX_DIVERGED


def test_newton_with_direct_solve_stops_on_indefinite_tangent():
    """From a far-from-equilibrium start the membrane's tangent is indefinite: Newton with a
    direct-solver name stops with the diverged flag instead of stepping with a failed factor."""
    from autopdex_gb300 import solver
    w = configs.cook_membrane(n=12, n_steps=2, solver="lapack")
    w.settings = w.steps[0](w.settings)
    u0 = np.random.default_rng(11).uniform(-0.05, 0.05, w.n_dofs).reshape(-1, 2)
    sol, (it, res, div) = solver.solver(u0, w.settings, w.static_settings, newton_tol=1e-8)
    assert div and it == 1
