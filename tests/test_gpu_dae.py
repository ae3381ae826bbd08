"""Backward-Euler time stepping through the manager equals the same steps taken by hand with
solver.solver (the 3-D nonlinear heat problem on an 8^3 brick mesh, 3 steps)."""
import numpy as np
import pytest

from autopdex_gb300 import configs, dae, solver

pytestmark = pytest.mark.gpu


def test_manager_matches_manual_steps():
    w = configs.heat_transient(n=8, n_steps=3, dt=1e-3)
    dt = w.raw["dt"]
    q = {"T": w.raw["T0"].copy()}
    settings = dict(w.settings)
    for _ in range(3):
        settings["dofs n"] = q
        settings["time increment"] = dt
        q, info = solver.solver(q, settings, w.static_settings, newton_tol=1e-10)
        assert not info[2]
    static = dict(w.static_settings, **{"time integrators": {"T": dae.BackwardEuler()}})
    m = dae.TimeSteppingManager(static, save_policy=dae.SaveAllPolicy(), newton_tol=1e-10)
    st = m.run({"T": w.raw["T0"].copy()}, dt, 3 * dt, 5, settings=dict(w.settings))
    assert st.num_accepted == 3 and st.num_rejected == 0
    assert np.abs(np.asarray(st.q["T"]) - np.asarray(q["T"])).max() <= 1e-12
    assert np.allclose(st.history.t[:4], dt * np.arange(4))


def test_bdf2_manager_matches_manual_steps():
    """BackwardDiffFormula(2) through the manager equals BDF2 steps taken by hand: each step
    solves the backward-Euler form with q* = (2 T_n - T_(n-1) / 2) / (3/2) and dt / (3/2), the
    history starting from (T0, T0)."""
    w = configs.heat_transient(n=8, n_steps=3, dt=1e-3)
    dt = w.raw["dt"]
    hist = [w.raw["T0"].copy(), w.raw["T0"].copy()]
    settings = dict(w.settings)
    for _ in range(3):
        settings["dofs n"] = {"T": (2.0 * hist[0] - 0.5 * hist[1]) / 1.5}
        settings["time increment"] = dt / 1.5
        q, info = solver.solver({"T": hist[0]}, settings, w.static_settings, newton_tol=1e-10)
        assert not info[2]
        hist = [np.asarray(q["T"]), hist[0]]
    static = dict(w.static_settings, **{"time integrators": {"T": dae.BackwardDiffFormula(2)}})
    m = dae.TimeSteppingManager(static, newton_tol=1e-10)
    st = m.run({"T": w.raw["T0"].copy()}, dt, 3 * dt, 5, settings=dict(w.settings))
    assert st.num_accepted == 3 and st.num_rejected == 0
    assert np.abs(np.asarray(st.q["T"]) - hist[0]).max() <= 1e-12
