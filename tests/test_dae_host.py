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


def test_only_backward_euler():
    st = _static()
    st["time integrators"] = {"T": object()}
    with pytest.raises(NotImplementedError):
        dae.TimeSteppingManager(st)
