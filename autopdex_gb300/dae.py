"""Time stepping over the GB300 Newton solve: the backward-Euler / BDF subset of AutoPDEx's
``dae.TimeSteppingManager`` (dae.py:1734-2283).

The reference manager runs multi-stage integrators on 'user residual' forms written in
q and q_t, with its own dense root solver.  Here the residual form is the backend's
backward-Euler heat descriptor (``models.heat_backward_euler_integrand``), which reads the
previous state and the step from two settings entries; the manager fills those entries
every step and calls ``solver.solver`` (the GPU Newton solve) as the root solver.  The step
loop follows dae.py:2141-2250: t = min(t_n + dt, t_max), pre-step update, solve, step size
controller (scaler, accept, interrupt), on acceptance the post-processing, post-step update
and save policy, dt scaled either way; an interrupt ends the run with NaN states.

A k-step backward differentiation formula, q_t = (c_0 q + sum_k c_k q_(n+1-k)) / dt, is the
backward-Euler form c_0 (q - q*) / dt with q* = -sum_k c_k q_(n+1-k) / c_0, so the same kernel
integrates it: the manager passes q* as the previous state and dt / c_0 as the step.  Like
the reference it uses the constant-step coefficients whatever the step history and starts
from a history filled with the initial state (dae.py:1799-1806).
Integrators other than ``BackwardEuler`` and ``BackwardDiffFormula`` and controllers that need
error estimates (``PIDController``) are not implemented.
"""
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import solver as _solver


# ---- integrators -----------------------------------------------------------------------
class BackwardEuler:
    """Implicit Euler (dae.py:288-318): one stage at t_(n+1), q_t = (q - q_n) / dt, order 1."""
    num_stages = 1
    num_steps = 1
    num_derivs = 1
    order = 1
    stage_positions = np.array([1.0])
    stage_list = [0]
    coeffs = (1.0, -1.0)


class BackwardDiffFormula:
    """BDF of 1 to 6 steps (dae.py:537-587): q_t = (c_0 q + sum_k c_k q_(n+1-k)) / dt with the
    constant-step coefficients of order ``num_steps``; one implicit stage."""
    _COEFFS = {
        1: (1.0, -1.0),
        2: (3.0 / 2.0, -2.0, 1.0 / 2.0),
        3: (11.0 / 6.0, -3.0, 3.0 / 2.0, -1.0 / 3.0),
        4: (25.0 / 12.0, -4.0, 3.0, -4.0 / 3.0, 1.0 / 4.0),
        5: (137.0 / 60.0, -5.0, 5.0, -10.0 / 3.0, 5.0 / 4.0, -1.0 / 5.0),
        6: (49.0 / 20.0, -6.0, 15.0 / 2.0, -20.0 / 3.0, 15.0 / 4.0, -6.0 / 5.0, 1.0 / 6.0),
    }
    num_stages = 1
    num_derivs = 1
    stage_positions = np.array([1.0])
    stage_list = [0]

    def __init__(self, num_steps):
        if num_steps not in self._COEFFS:
            raise ValueError("Order of BDF method not supported. Supported orders: 1 to 6. "
                             "From 7 on the BDF method is not stable.")
        self.num_steps = num_steps
        self.order = num_steps
        self.coeffs = self._COEFFS[num_steps]


# ---- step size controllers (dae.py:1314-1573) -------------------------------------------
@dataclass
class ControllerState:
    step_scaler: float = 1.0
    dt: float = 1.0
    accept: bool = True
    interrupt: bool = False


class ConstantStepSizeController:
    """Keeps dt; a step is accepted when the root solve converged, and a failed solve
    interrupts the run (the step cannot be reduced), as dae.py:1474-1497."""

    def initialize(self, initial_error):
        return ControllerState()

    def compute_scaler(self, error, q, q_n, state, order, converged, num_iterations, dt, verbose):
        return state

    def check_accept(self, state, converged, verbose):
        interrupt = state.interrupt or not converged
        if not converged and not state.interrupt and verbose >= 0:
            print("Root solver did not converge, but stepsize controller can not reduce step size!")
        return ControllerState(state.step_scaler, state.dt, converged, interrupt)


class RootIterationController:
    """Aims at ``target_niters`` Newton iterations per step (dae.py:1509-1573): dt is scaled by
    1 + gamma (target - iterations) / target, halved after a failed solve, and clipped to
    [min_step_size, max_step_size]; a failed solve at the minimum step interrupts."""

    def __init__(self, target_niters=6, gamma=0.5, max_step_size=1e20, min_step_size=1e-6):
        self.target_niters = target_niters
        self.gamma = gamma
        self.max_step_size = max_step_size
        self.min_step_size = min_step_size

    def initialize(self, initial_error):
        return ControllerState()

    def compute_scaler(self, error, q, q_n, state, order, converged, num_iterations, dt, verbose):
        correction = 1 + self.gamma * (self.target_niters - num_iterations) / self.target_niters if converged else 0.5
        new_dt = float(np.clip(dt * correction, self.min_step_size, self.max_step_size))
        return ControllerState(new_dt / dt, new_dt, state.accept, state.interrupt)

    def check_accept(self, state, converged, verbose):
        stuck = not converged and np.isclose(state.dt, self.min_step_size) and not state.interrupt
        if stuck and verbose >= 0:
            print("Root solver did not converge, but minimum step_size is reached!")
        return ControllerState(state.step_scaler, state.dt, converged, state.interrupt or stuck)


# ---- save policies (dae.py:1099-1312) -----------------------------------------------------
@dataclass
class HistoryState:
    t: np.ndarray
    q: dict
    user: Any = field(default_factory=dict)


class SaveNothingPolicy:
    def initialize(self, q, t_max, num_time_steps, user_data={}):
        return None

    def save_step(self, state, t, q, user_data={}):
        return None

    def finalize(self, state):
        return None


class SaveAllPolicy:
    """Every accepted step (and the initial state) into arrays pre-filled with NaN."""

    def initialize(self, q, t_max, max_steps, user_data={}):
        return {"t": np.full(max_steps + 1, np.nan),
                "q": {k: np.full((max_steps + 1,) + np.shape(v), np.nan) for k, v in q.items()},
                "user": {k: np.full((max_steps + 1,) + np.shape(v), np.nan) for k, v in user_data.items()},
                "idx": 0, "max": max_steps}

    def save_step(self, state, t, q, user_data={}):
        i = state["idx"]
        state["t"][i] = t
        for k in state["q"]:
            state["q"][k][i] = _host(q[k])
        for k in state["user"]:
            state["user"][k][i] = _host(user_data[k])
        state["idx"] = min(i + 1, state["max"])
        return state

    def finalize(self, state):
        return HistoryState(state["t"], state["q"], state["user"])


class SaveEquidistantPolicy(SaveAllPolicy):
    """At (about) ``num_points`` + 1 equidistant times: a step is saved once it reaches the next
    target time minus ``tol``."""

    def __init__(self, num_points=None, tol=1e-6):
        self.num_points = num_points
        self.tol = tol

    def initialize(self, q, t_max, max_steps, user_data={}):
        n = self.num_points if self.num_points is not None else max_steps
        state = super().initialize(q, t_max, n, user_data)
        state["targets"] = np.linspace(0.0, t_max, n + 1)
        return state

    def save_step(self, state, t, q, user_data={}):
        if t >= state["targets"][state["idx"]] - self.tol:
            return super().save_step(state, t, q, user_data)
        return state


def _host(a):
    return a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)


@dataclass
class TimeSteppingManagerState:
    q: Any
    settings: dict
    history: Any
    num_steps: int
    num_accepted: int
    num_rejected: int


class TimeSteppingManager:
    """Backward-Euler time stepping of a 'user residual' model through the GB300 Newton solve.

    ``static_settings['time integrators']`` maps every DOF field to ``BackwardEuler()``; the
    model's integrand names the settings entries of the previous state and of the step
    (``heat_backward_euler_integrand(..., time_increment=..., dofs_n=...)``).  ``solver_kwargs``
    go to ``solver.solver`` (newton_tol, maxiter, ...)."""

    def __init__(self, static_settings, settings={"current time": 0.0}, root_solver=None, save_policy=None,
                 step_size_controller=None, postprocessing_fun=lambda q_fun, t, settings: {},
                 pre_step_updates=None, post_step_updates=None, **solver_kwargs):
        self.integrators = static_settings["time integrators"]
        if not all(isinstance(i, (BackwardEuler, BackwardDiffFormula)) for i in self.integrators.values()):
            raise NotImplementedError("the gb300 time stepping implements BackwardEuler and BackwardDiffFormula")
        coeffs = {tuple(i.coeffs) for i in self.integrators.values()}
        if len(coeffs) != 1:
            raise NotImplementedError("all fields must use the same integrator (one previous-state entry)")
        self.coeffs = coeffs.pop()
        self.num_steps = len(self.coeffs) - 1
        if root_solver is not None:
            raise NotImplementedError("the root solver is the gb300 Newton solve (solver.solver)")
        keys = set()
        for m in static_settings["model"]:
            p = getattr(getattr(m, "integrand", None), "params", None)
            if not p or "time_increment" not in p:
                raise NotImplementedError("time stepping needs a backward-Euler 'user residual' model "
                                          "(models.heat_backward_euler_integrand)")
            keys.add((p["time_increment"], p["dofs_n"]))
        if len(keys) != 1:
            raise NotImplementedError("all models must read the same step and previous-state entries")
        self.dt_key, self.qn_key = keys.pop()
        self.static_settings = static_settings
        self.save_policy = save_policy
        self.step_size_controller = step_size_controller or ConstantStepSizeController()
        self.postprocessing_fun = postprocessing_fun
        self.pre_step_updates = pre_step_updates or self._set_time
        self.post_step_updates = post_step_updates or (lambda q_fun, t, settings: settings)
        self.verbose = static_settings.get("verbose", 0)
        self.solver_kwargs = solver_kwargs

    @staticmethod
    def _set_time(t, settings):
        settings["current time"] = t
        return settings

    def _backward_euler_form(self, history, dt):
        """(q*, dt / c_0) of the step: the previous state and step the backward-Euler model
        reads.  ``history[0]`` is the latest accepted state."""
        if self.num_steps == 1:
            return history[0], dt
        c = self.coeffs
        q_star = {k: sum(history[i][k] * c[i + 1] for i in range(self.num_steps)) * (-1.0 / c[0])
                  for k in history[0]}
        return q_star, dt / c[0]

    def run(self, dofs, dt0, t_max, num_time_steps, settings={"current time": 0.0}):
        """Steps from t = 0 until t_max or ``num_time_steps`` attempted steps (dae.py:2087-2283)."""
        if list(dofs.keys()) != sorted(dofs.keys()):
            raise ValueError("The keys of the DOFs must be alphabetically sorted.")
        settings = dict(settings)
        t_n, dt = 0.0, float(dt0)
        q_n = dict(dofs)
        ctrl = self.step_size_controller.initialize(0.0)
        user = self.postprocessing_fun(lambda t: q_n, t_n, settings)
        hist = self.save_policy.initialize(q_n, t_max, num_time_steps, user) if self.save_policy else None
        hist = self.save_policy.save_step(hist, t_n, q_n, user) if self.save_policy else hist
        n_acc = n_rej = 0
        q = q_n
        history = [q_n] * self.num_steps
        for _ in range(num_time_steps):
            if not t_n < t_max or ctrl.interrupt:
                break
            t = min(t_n + dt, t_max)
            dt = t - t_n
            settings = self.pre_step_updates(t, settings)
            # the root solve reads the backward-Euler form of the step (q*, dt / c_0); user
            # callbacks keep the real step and the latest accepted state
            solve_settings = dict(settings)
            solve_settings[self.qn_key], solve_settings[self.dt_key] = self._backward_euler_form(history, dt)
            settings[self.qn_key], settings[self.dt_key] = q_n, dt
            q, (n_it, res, diverged) = _solver.solver(q_n, solve_settings, self.static_settings, **self.solver_kwargs)
            converged = not bool(diverged)
            order = min(i.order for i in self.integrators.values())
            ctrl = self.step_size_controller.compute_scaler(None, q, q_n, ctrl, order, converged, int(n_it), dt,
                                                            self.verbose)
            ctrl = self.step_size_controller.check_accept(ctrl, converged, self.verbose)
            if ctrl.accept and not ctrl.interrupt:
                q_n = q
                history = [q] + history[:-1]
                settings[self.qn_key] = q
                user = self.postprocessing_fun(lambda tt: q, t, settings)
                settings = self.post_step_updates(lambda tt: q, t, settings)
                hist = self.save_policy.save_step(hist, t, q, user) if self.save_policy else hist
                t_n = t
                n_acc += 1
            else:
                n_rej += 1
            dt = ctrl.step_scaler * dt
            if self.verbose >= 0:
                print(f"Time: {t:.2e}, accepted step: {ctrl.accept}, dt: {dt:.2e}, iterations: {int(n_it)}")
        if ctrl.interrupt:
            q_n = {k: np.full(np.shape(v), np.nan) for k, v in q_n.items()}
        elif self.verbose >= 0 and not np.isclose(t_n, t_max):
            print("Maximum number of steps reached before t_max!")
        hist = self.save_policy.finalize(hist) if self.save_policy else hist
        return TimeSteppingManagerState(q=q_n, settings=settings, history=hist, num_steps=n_acc + n_rej,
                                        num_accepted=n_acc, num_rejected=n_rej)
