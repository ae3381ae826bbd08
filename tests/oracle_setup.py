"""Builds the CPU-oracle problem matching an ``autopdex_gb300.configs`` workload."""
import numpy as np

from oracle import elements as el
from oracle import newton


def oracle_problem(w, settings=None):
    r = w.raw
    coords = r["coords"]
    kind = r["kind"]
    settings = settings if settings is not None else w.settings
    if kind == "poisson":
        fun = el.user_potential_element(el.poisson_sincos_integrand(), 2, 4)
        conn = r["conns"][0]
        sets = [newton.ElementSet("potential", conn, fun, lambda st, n=conn.shape[0]: np.zeros((n, 1)), 1)]
        n = coords.shape[0]
    elif kind == "heat":
        fun = el.user_potential_element(el.heat_potential_integrand(1.0), 2, 4)
        conn = r["conns"][0]
        k = r["k"]
        sets = [newton.ElementSet("potential", conn, fun, lambda st: k.reshape(-1, 1), 1)]
        n = coords.shape[0]
    elif kind == "neo_hooke_3d":
        fun = el.hyperelastic_element(3, 8, 2, "3d")
        conn = r["conns"][0]
        sets = [newton.ElementSet("element", conn, fun,
                                  lambda st, n=conn.shape[0]: np.tile([r["E"], r["nu"]], (n, 1)), 3)]
        n = coords.shape[0] * 3
    elif kind == "cook":
        fun = el.hyperelastic_element(2, 4, 2, "plain strain")
        conn, lines = r["conns"]
        nfun = el.neumann_line_element(2, 2)
        sets = [newton.ElementSet("element", conn, fun,
                                  lambda st, n=conn.shape[0]: np.tile([r["E"], r["nu"]], (n, 1)), 2),
                newton.ElementSet("neumann", lines, nfun, None, 2,
                                  traction=lambda st: np.array([0.0, st["load multiplier"]]))]
        n = coords.shape[0] * 2
    elif kind == "heat_be":
        fun = el.nonlinear_heat_be_element(3, 8, 2)
        conn = r["conns"][0]
        sets = [newton.ElementSet("residual", conn, fun,
                                  lambda st, n=conn.shape[0]: np.tile([1.0, 0.5, 1.0, st["time increment"]], (n, 1)),
                                  1)]
        n = coords.shape[0]
    else:
        raise ValueError(kind)
    return newton.Problem(sets, coords, n, r["dirichlet"], r["values"])


def oracle_settings(w):
    """Plain-dict settings for the oracle (flattened 'dofs n')."""
    st = dict(w.settings)
    if "dofs n" in st:
        v = st["dofs n"]
        st["dofs n"] = np.asarray(next(iter(v.values())) if isinstance(v, dict) else v).reshape(-1)
    return st
