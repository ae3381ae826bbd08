"""The time-stepping manager's control flow (dae.py:2087-2283) with a fake root solve on the
host: backward Euler of T' = -lam T, where the fake solve returns T_n / (1 + lam dt) and an
iteration count / divergence chosen by the test.  No GPU."""
import numpy as np
import pytest

from autopdex_gb300 import dae, models, seeder, spaces
from autopdex_gb300 import solver as S

LAM = 2.0


def _static():
    integrand = models.heat_backward_euler_integrand(1.0, 0.5, 1.0, "time increment", "dofs n")
    model = models.mixed_reference_domain_residual(integrand, {"T": spaces.fem_iso_line_quad_brick},
                                                   *seeder.gauss_legendre_nd(3, 2), "T")
    return {"assembling mode": ("user residual",), "model": (model,), "time integrators": {"T": dae.BackwardEuler()},
            "verbose": -1}


def _fake(monkeypatch, iters=lambda dt: 3, diverge=lambda dt: False, log=None):
    def solve(dofs, settings, static_settings, **kw):
        dt = settings["time increment"]
        assert settings["dofs n"] is dofs  # the previous state goes to the model's entry
        if log is not None:
            log.append(dt)
        out = {"T": np.asarray(dofs["T"]) / (1.0 + LAM * dt)}
        return out, (iters(dt), 0.0, diverge(dt))
    monkeypatch.setattr(S, "solver", solve)


def test_constant_steps_and_history(monkeypatch):
    _fake(monkeypatch)
    m = dae.TimeSteppingManager(_static(), save_policy=dae.SaveAllPolicy())
    st = m.run({"T": np.ones(4)}, 0.1, 0.5, 10)
    assert st.num_accepted == 5 and st.num_rejected == 0 and st.num_steps == 5
    assert np.allclose(st.q["T"], 1.2 ** -5)
    assert np.allclose(st.history.t[:6], np.linspace(0, 0.5, 6))
    assert np.allclose(st.history.q["T"][:6, 0], 1.2 ** -np.arange(6.0))
    assert np.all(np.isnan(st.history.t[6:]))
    assert np.isclose(st.settings["current time"], 0.5)


def test_root_iteration_controller_grows_and_clips(monkeypatch):
    log = []
    _fake(monkeypatch, iters=lambda dt: 3, log=log)
    ctrl = dae.RootIterationController(target_niters=6, gamma=0.5)
    st = dae.TimeSteppingManager(_static(), step_size_controller=ctrl).run({"T": np.ones(2)}, 0.1, 0.5, 20)
    # 3 iterations against a target of 6: dt grows by 1 + 0.5 (6 - 3) / 6 = 1.25 per step, the
    # last step is cut at t_max
    expect = [0.1, 0.125, 0.15625]
    expect.append(0.5 - sum(expect))
    assert np.allclose(log, expect) and st.num_accepted == 4


def test_failed_solve_halves_the_step(monkeypatch):
    log = []
    _fake(monkeypatch, iters=lambda dt: 6, diverge=lambda dt: dt > 0.15, log=log)
    st = dae.TimeSteppingManager(_static(), step_size_controller=dae.RootIterationController()).run(
        {"T": np.ones(2)}, 0.2, 0.2, 10)
    assert np.allclose(log, [0.2, 0.1, 0.1]) and st.num_rejected == 1 and st.num_accepted == 2
    assert np.allclose(st.q["T"], 1.2 ** -2)


def test_constant_controller_interrupts(monkeypatch):
    _fake(monkeypatch, diverge=lambda dt: True)
    st = dae.TimeSteppingManager(_static()).run({"T": np.ones(3)}, 0.1, 1.0, 10)
    assert st.num_rejected == 1 and st.num_accepted == 0 and np.all(np.isnan(st.q["T"]))


def test_equidistant_saving(monkeypatch):
    _fake(monkeypatch)
    st = dae.TimeSteppingManager(_static(), save_policy=dae.SaveEquidistantPolicy(num_points=2)).run(
        {"T": np.ones(1)}, 0.1, 1.0, 20)
    assert np.allclose(st.history.t, [0.0, 0.5, 1.0])


def test_only_backward_euler_and_bdf():
    st = _static()
    st["time integrators"] = {"T": object()}
    with pytest.raises(NotImplementedError):
        dae.TimeSteppingManager(st)
    with pytest.raises(ValueError):
        dae.BackwardDiffFormula(7)


def _fake_be_form(monkeypatch, log):
    """Root solve of T' = -lam T in the backward-Euler form the model reads:
    (T - T*) / dt_eff = -lam T."""
    def solve(dofs, settings, static_settings, **kw):
        q_star, dt_eff = settings["dofs n"], settings["time increment"]
        log.append((np.asarray(q_star["T"]).copy(), dt_eff))
        return {"T": np.asarray(q_star["T"]) / (1.0 + LAM * dt_eff)}, (3, 0.0, False)
    monkeypatch.setattr(S, "solver", solve)


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6])
def test_bdf_steps_equal_the_multistep_recurrence(monkeypatch, k):
    """BackwardDiffFormula(k) through the manager equals the k-step recurrence
    (c_0 T_(n+1) + sum_i c_i T_(n+1-i)) / dt = -lam T_(n+1) with the reference's constant-step
    coefficients and a history started from the initial state (dae.py:537-587, :1799-1806)."""
    log = []
    _fake_be_form(monkeypatch, log)
    static = _static()
    static["time integrators"] = {"T": dae.BackwardDiffFormula(k)}
    dt, n = 0.05, 12
    st = dae.TimeSteppingManager(static, save_policy=dae.SaveAllPolicy()).run({"T": np.ones(3)}, dt, n * dt, 20)
    assert st.num_accepted == n
    c = dae.BackwardDiffFormula(k).coeffs
    hist = [1.0] * k
    for _ in range(n):
        T = -sum(ci * h for ci, h in zip(c[1:], hist)) / (c[0] + LAM * dt)
        hist = [T] + hist[:-1]
    assert abs(st.q["T"][0] - hist[0]) <= 1e-14 * abs(hist[0])
    assert np.allclose(log[0][1], dt / c[0]) and np.allclose(log[0][0], 1.0)
    assert np.allclose(st.history.q["T"][n, :], hist[0], rtol=1e-14, atol=0)


def test_bdf_startup_history_and_order(monkeypatch):
    """BDF2 keeps two states and the first step reads (T0, T0) as its history.  That start
    (the reference's: a history filled with the initial state) is a first-order step, so on
    T' = -lam T the error at t = 1 of BDF2 and BDF3 through the manager halves with dt."""
    log = []
    _fake_be_form(monkeypatch, log)
    static = _static()
    static["time integrators"] = {"T": dae.BackwardDiffFormula(2)}
    dae.TimeSteppingManager(static).run({"T": np.ones(1)}, 0.1, 0.3, 3)
    # step 1: q* = (2 T0 - T0 / 2) / (3/2) = T0; step 2: q* = (2 T1 - T0 / 2) / (3/2)
    T1 = 1.0 / (1.0 + LAM * 0.1 / 1.5)
    assert np.isclose(log[0][0][0], 1.0) and np.isclose(log[1][0][0], (2.0 * T1 - 0.5) / 1.5)
    for k in (2, 3):
        static["time integrators"] = {"T": dae.BackwardDiffFormula(k)}
        errs = []
        for dt in (0.02, 0.01, 0.005):
            st = dae.TimeSteppingManager(static).run({"T": np.ones(1)}, dt, 1.0, 400)
            errs.append(abs(st.q["T"][0] - np.exp(-LAM)))
        assert 1.9 < errs[0] / errs[1] < 2.1 and 1.9 < errs[1] / errs[2] < 2.1, errs


def test_callbacks_see_the_real_step_and_state(monkeypatch):
    """For a k-step BDF the root solve reads (q*, dt / c_0); postprocessing and post-step
    callbacks see the real step and the accepted state instead."""
    log, seen = [], []
    _fake_be_form(monkeypatch, log)
    static = _static()
    static["time integrators"] = {"T": dae.BackwardDiffFormula(2)}

    def post(q_fun, t, settings):
        seen.append((t, settings["time increment"], np.asarray(settings["dofs n"]["T"]).copy(),
                     np.asarray(q_fun(t)["T"]).copy()))
        return settings
    dae.TimeSteppingManager(static, post_step_updates=post).run({"T": np.ones(1)}, 0.1, 0.3, 3)
    assert len(seen) == 3
    c0 = dae.BackwardDiffFormula(2).coeffs[0]
    for (t, dt, qn, q), (q_star, dt_eff) in zip(seen, log):
        assert np.isclose(dt, 0.1) and np.isclose(dt_eff, 0.1 / c0)
        assert np.array_equal(qn, q)  # the accepted state, not the synthetic q*
