"""Parity at the workloads' own sizes: the GPU path against the oracle's C restatement
(oracle/c/orc.c, itself checked against the AD oracle in test_oracle_c.py) on the full
200^2 Poisson, 64^3 neo-Hooke cube, 512^2 Cook membrane, 1024^2 heat and 128^3 backward-Euler
heat problems.

Tolerances, written where they are used:
* float64 residuals at random non-converged states: ||R_gpu - R_oracle|| <= 1e-12 ||R_oracle||
* float64 tangents: max |K_gpu - K_oracle| <= 1e-12 max |K_oracle|; float32: 2e-6
* converged GPU solutions: the oracle's float64 residual of the GPU solution <= 2x the Newton
  tolerance of the solve (relative to the step's first residual), and ||u_gpu - u_oracle||_inf
  <= 1e-8 max |u_oracle| where the oracle solves too
"""
import numpy as np
import pytest
import scipy.sparse as sps
import scipy.sparse.linalg as spla

from autopdex_gb300 import configs
from oracle import corc

pytestmark = pytest.mark.gpu


def _flat(d):
    a = next(iter(d.values())) if isinstance(d, dict) else d
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.asarray(a, dtype=np.float64).reshape(-1)


def _like(w, flat):
    d = w.dofs
    if isinstance(d, dict):
        k = next(iter(d))
        return {k: flat.reshape(np.shape(d[k]))}
    return flat.reshape(np.shape(d))


def _residual(w, u, settings):
    """The oracle's float64 residual of workload w (C elements, element-order scatter)."""
    r = w.raw
    kind, coords = r["kind"], r["coords"]
    n = coords.shape[0]
    if kind == "poisson":
        Re, _ = corc.q1_elements("poisson", r["conns"][0], coords, u, [20.0, 10.0, 1.0, 0.5], tangent=False)
        return corc.scatter(r["conns"][0], 1, Re, n)
    if kind == "heat":
        Re, _ = corc.q1_elements("heat", r["conns"][0], coords, u, [1.0], elem_field=r["k"], tangent=False)
        return corc.scatter(r["conns"][0], 1, Re, n)
    if kind == "neo_hooke_3d":
        Re, _ = corc.q1_elements("neo_hooke", r["conns"][0], coords, u, [r["E"], r["nu"]], accurate=True,
                                 tangent=False)
        return corc.scatter(r["conns"][0], 3, Re, 3 * n)
    if kind == "cook":
        Re, _ = corc.q1_elements("neo_hooke", r["conns"][0], coords, u, [r["E"], r["nu"]], accurate=True,
                                 tangent=False)
        R = corc.scatter(r["conns"][0], 2, Re, 2 * n)
        Rl = corc.neumann_lines(r["conns"][1], coords, (0.0, float(settings["load multiplier"])))
        return R + corc.scatter(r["conns"][1], 2, Rl, 2 * n)
    if kind == "heat_be":
        Re, _ = corc.q1_elements("heat_be", r["conns"][0], coords, u, [1.0, 0.5, 1.0, float(settings["time increment"])],
                                 node_field=_flat(settings["dofs n"]), tangent=False)
        return corc.scatter(r["conns"][0], 1, Re, n)
    raise ValueError(kind)


def _residual_parity(w, scale, seed=0, settings=None):
    from autopdex_gb300 import assembler
    st = settings if settings is not None else w.settings
    u = np.random.default_rng(seed).uniform(-scale, scale, w.n_dofs)
    R_gpu = _flat(assembler.assemble_residual(_like(w, u), st, w.static_settings))
    R_or = _residual(w, u, st)
    return float(np.linalg.norm(R_gpu - R_or) / np.linalg.norm(R_or))


def test_poisson_200_direct_solution_and_residual():
    """200^2 Poisson, one Newton step with the direct solve, against the oracle's C elements,
    SciPy COO->CSR and spsolve (solver.py:1180-1222, :1520)."""
    from autopdex_gb300 import solver
    w = configs.poisson(n=200, solver="lapack")
    assert _residual_parity(w, 1.0) <= 1e-12
    sol, (it, res, div) = solver.solver(w.dofs, w.settings, w.static_settings, newton_tol=1e-10)
    assert not div and it == 1
    r = w.raw
    free = ~r["dirichlet"]
    n = r["coords"].shape[0]
    Re, Ke = corc.q1_elements("poisson", r["conns"][0], r["coords"], np.zeros(n), [20.0, 10.0, 1.0, 0.5])
    R = corc.scatter(r["conns"][0], 1, Re, n)
    c = r["conns"][0]
    A = sps.coo_matrix((Ke.ravel(), (np.repeat(c, 4, axis=1).ravel(), np.tile(c, (1, 4)).ravel())),
                       shape=(n, n)).tocsr()[:, free][free]
    u_or = np.zeros(n)
    u_or[free] = spla.spsolve(A.tocsc(), -R[free])
    u = _flat(sol)
    assert np.abs(u - u_or).max() <= 1e-8 * np.abs(u_or).max()
    assert np.linalg.norm(_residual(w, u, w.settings)[free]) <= 2e-10 * np.linalg.norm(R[free])


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_heat_1024_residual_and_tangent(dtype):
    """1024^2 random-conductivity heat: residual and tangent at random DOFs against the C
    oracle's element tangents summed by SciPy."""
    from autopdex_gb300 import assembler
    w = configs.heat_grf(n=1024, seed=10000)
    if dtype == "float64":
        assert _residual_parity(w, 1.0, seed=3) <= 1e-12
    u = np.random.default_rng(4).uniform(-1.0, 1.0, w.n_dofs)
    K = assembler.assemble_tangent(_like(w, u), w.settings, w.static_settings, dtype=dtype).to_scipy()
    r = w.raw
    n = r["coords"].shape[0]
    _, Ke = corc.q1_elements("heat", r["conns"][0], r["coords"], u, [1.0], elem_field=r["k"])
    c = r["conns"][0]
    K_or = sps.coo_matrix((Ke.ravel(), (np.repeat(c, 4, axis=1).ravel(), np.tile(c, (1, 4)).ravel())),
                          shape=(n, n)).tocsr()
    tol = 1e-12 if dtype == "float64" else 2e-6
    assert abs(K - K_or).max() <= tol * abs(K_or).max()


def test_neo_hooke_64cube_load_step_1():
    """64^3 neo-Hooke cube, load step 1 (mixed precision): the oracle's float64 residual of the
    GPU solution, and residual parity at a random state."""
    from autopdex_gb300 import solver
    w = configs.neo_hooke_cube(n=64, n_steps=10, precision="mixed")
    assert _residual_parity(w, 0.003, seed=5) <= 1e-12
    st = w.steps[0](dict(w.settings))
    x0 = np.zeros((w.n_dofs // 3, 3))
    x0[:, 0] = w.raw["stretch"] / w.raw["n_steps"] * w.raw["coords"][:, 0]
    sol, (it, res, div) = solver.solver(x0, st, w.static_settings, newton_tol=0.0, newton_rtol=1e-10, maxiter=30)
    assert not div
    res0 = solver.last_info.res0
    free = ~w.raw["dirichlet"]
    R = _residual(w, _flat(sol), st)
    assert np.linalg.norm(R[free]) <= 2e-10 * res0


def test_neo_hooke_32cube_solution_matches_oracle_newton():
    """The same load step at 32^3 against the oracle's own Newton solve (C elements, SciPy
    COO->CSR, C Jacobi-PCG to 1e-12 per step, solution updates as solver.py:879-892)."""
    from autopdex_gb300 import solver
    w = configs.neo_hooke_cube(n=32, n_steps=10)
    st = w.steps[0](dict(w.settings))
    r = w.raw
    x0 = np.zeros((w.n_dofs // 3, 3))
    x0[:, 0] = r["stretch"] / r["n_steps"] * r["coords"][:, 0]
    sol, (it, res, div) = solver.solver(x0, st, w.static_settings, newton_tol=0.0, newton_rtol=1e-10, maxiter=30)
    assert not div
    free = ~r["dirichlet"]
    vals = np.asarray(st["dirichlet conditions"]).reshape(-1)
    u = np.where(free, x0.reshape(-1), vals)
    c = r["conns"][0]
    ed = (c[:, :, None] * 3 + np.arange(3)).reshape(c.shape[0], -1)
    res0 = None
    for _ in range(30):
        Re, Ke = corc.q1_elements("neo_hooke", c, r["coords"], u, [r["E"], r["nu"]], accurate=True)
        R = corc.scatter(c, 3, Re, w.n_dofs)
        nr = np.linalg.norm(R[free])
        res0 = nr if res0 is None else res0
        if nr <= 1e-10 * res0:
            break
        A = sps.coo_matrix((Ke.ravel(), (np.repeat(ed, 24, axis=1).ravel(), np.tile(ed, (1, 24)).ravel())),
                           shape=(w.n_dofs, w.n_dofs)).tocsr()[:, free][free].tocsr()
        du, _, _ = corc.pcg_csr_tol(A, -R[free], 1e-12, 100000)
        u[free] += du
    assert np.abs(_flat(sol) - u).max() <= 1e-8 * np.abs(u).max()


def test_cook_512_residual_parity_and_direct_solution():
    """512^2 Cook membrane (nu = 0.4999): residual parity at a small random state, and the
    oracle's float64 residual of the GPU's direct-solve Newton solution of load step 1 within
    twice the 1e-7 tolerance (the float64 floor of this problem is near 4e-8)."""
    from autopdex_gb300 import solver
    w = configs.cook_membrane(n=512, solver="lapack")
    st = w.steps[0](dict(w.settings))
    assert _residual_parity(w, 1e-5, seed=6, settings=st) <= 1e-12
    sol, (it, res, div) = solver.solver(w.dofs, st, w.static_settings, newton_tol=0.0, newton_rtol=1e-7, maxiter=12)
    assert not div
    res0 = solver.last_info.res0
    free = ~w.raw["dirichlet"]
    assert np.linalg.norm(_residual(w, _flat(sol), st)[free]) <= 2e-7 * res0


def test_heat_be_128cube_first_time_step():
    """128^3 backward-Euler heat, the first time step (mixed Jacobi-PCG in the float64 Newton
    loop): residual parity at a random state and the oracle's residual of the GPU solution."""
    from autopdex_gb300 import solver
    w = configs.heat_transient(n=128, solver="pcg", precision="mixed")
    assert _residual_parity(w, 1.0, seed=7) <= 1e-12
    sol, (it, res, div) = solver.solver(w.dofs, w.settings, w.static_settings, newton_tol=0.0, newton_rtol=1e-10,
                                        maxiter=30)
    assert not div
    res0 = solver.last_info.res0
    free = ~w.raw["dirichlet"]
    assert np.linalg.norm(_residual(w, _flat(sol), w.settings)[free]) <= 2e-10 * res0
