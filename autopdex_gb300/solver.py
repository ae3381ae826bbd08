"""``solver.solver`` of AutoPDEx, run by the GB300 backend.

Drop-in for ``autopdex.solver.solver(dofs, settings, static_settings, **kwargs)``
(solver.py:41-137) when ``static_settings['solver backend'] == 'gb300'``: same dicts, same
DOF pytree in and out, same ``infos = (n_iter, res_norm, diverged)`` of the Newton solvers
(solver.py:740-948).  Assembly, the sparse pattern, the Dirichlet elimination, the Krylov
solve and the Newton loop run on the GPU through libautopdex_gb300.

Keys read from ``static_settings`` (besides AutoPDEx's own):

* ``'solver'``: ``'pcg'`` / ``'cg'`` (Jacobi-PCG, default), ``'bicgstab'`` (non-symmetric
  tangents), ``'fcg'`` (flexible CG for the learned preconditioner); the direct-solver names
  ``'lapack'`` / ``'umfpack'`` / ``'direct'`` / ``'cholesky'`` factor the float64 tangent
  (banded Cholesky on the GPU, refined to a relative residual of 1e-13) -- the role of
  spsolve in linear_solve_scipy (solver.py:1493-1539) -- for symmetric tangents (potentials,
  hyperelastic elements) on meshes with a narrow band; the non-symmetric backward-Euler
  residual model runs float64 BiCGStab to 1e-13 instead.
* ``'precision'``: ``'float64'`` (default) or ``'mixed'`` (float32 tangent and Krylov
  iterations inside the float64 Newton / refinement loop).
* ``'type of preconditioner'``: ``'jacobi'`` (default) or ``'learned'`` (the network set with
  :func:`set_learned_preconditioner`; Jacobi when none is set): flexible CG in float32 with
  ``'precision': 'mixed'``, in float64 with the preconditioner in float32 / bf16 with
  ``'precision': 'float64'``.

Extra keyword arguments: ``newton_tol``, ``maxiter`` (Newton), ``newton_rtol`` (stop also at
``||R|| <= newton_rtol ||R_0||``), ``krylov_tol``, ``krylov_maxiter``, ``reuse_tangent``.

:func:`sensitivities` gives the forward implicit derivatives of a converged solution with
respect to scalar settings (what adaptive_load_stepping's implicit_diff_mode='forward'
differentiates), :func:`second_order_sensitivities` the second ones and
:func:`adjoint_sensitivities` the reverse-mode gradient of a scalar function of the solution.
"""
import numpy as np
import torch

from . import _native as N
from ._problem import get_problem, flatten, _np, is_foreign

last_info = None


def _method(static_settings, kwargs):
    name = static_settings.get("solver", "pcg")
    precision = static_settings.get("precision", "float64")
    precond = static_settings.get("type of preconditioner", "jacobi")
    direct = name in ("lapack", "umfpack", "direct", "lu", "cholesky")
    symmetric = all(getattr(m, "kernel", None) != N.AGX_MODEL_HEAT_BE for m in static_settings.get("model", ()))
    if direct:
        method = N.AGX_CHOL_BAND if symmetric else N.AGX_BICGSTAB
    elif name in ("pcg", "cg"):
        method = N.AGX_PCG_MIXED if precision == "mixed" else N.AGX_PCG
    elif name == "bicgstab":
        if precision == "mixed":
            raise NotImplementedError("BiCGStab runs in float64 only")
        method = N.AGX_BICGSTAB
    elif name == "fcg":
        method = N.AGX_FCG_F64 if precision == "float64" else N.AGX_FCG_MIXED
    else:
        raise NotImplementedError(f"solver {name!r} is not available in the gb300 backend")
    if precond == "learned":
        # float32 FCG for 'mixed'; float64 FCG with the float32 / bf16 preconditioner for
        # 'float64' (tangents whose conditioning float32 Krylov vectors cannot resolve)
        method = N.AGX_FCG_F64 if precision == "float64" else N.AGX_FCG_MIXED
    elif precond != "jacobi":
        raise NotImplementedError(f"preconditioner {precond!r} is not available in the gb300 backend")
    mixed = method in (N.AGX_PCG_MIXED, N.AGX_FCG_MIXED)
    # inner tolerances of the refinement loops: the float32 inner solves gain ~1e-3 per outer
    # step whatever they are asked for, so the flexible CG (the learned preconditioner) stops at
    # 1e-3 (measured on the 1024^2 heat problem: 1e-3 / 1e-4 / 1e-5 -> 79 / 93 / 113 FCG
    # iterations, four outer steps each)
    default_tol = 1e-13 if direct else (
        1e-3 if method == N.AGX_FCG_MIXED else (1e-5 if mixed else (1e-4 if method == N.AGX_FCG_F64 else 1e-11)))
    opts = N.SolveOpts()
    opts.method = method
    opts.rtol = float(kwargs.get("krylov_tol", default_tol))
    opts.atol = float(kwargs.get("krylov_atol", 0.0))
    opts.maxiter = int(kwargs.get("krylov_maxiter", 100000))
    # iterations between host checks of convergence (one CUDA graph replay each); the learned
    # preconditioner converges in tens of iterations, so its chunks are shorter (a replay past
    # convergence still runs the network)
    opts.check_every = int(kwargs.get("krylov_check_every", 8 if precond == "learned" else 32))
    return opts, (N.AGX_F32 if mixed else N.AGX_F64)


def _reuse_default(static_settings):
    """Tangents of the quadratic potentials do not depend on the DOFs."""
    from . import _native as NN
    return all(getattr(m, "kernel", None) in (NN.AGX_MODEL_POISSON_SINCOS, NN.AGX_MODEL_HEAT_POTENTIAL,
                                               NN.AGX_MODEL_NEUMANN) for m in static_settings["model"])


def _backend_check(static_settings):
    if static_settings.get("solver backend") != "gb300":
        raise ValueError("autopdex_gb300.solver needs static_settings['solver backend'] == 'gb300'")
    if not torch.cuda.is_available():
        raise RuntimeError("the gb300 backend needs a CUDA device (there is no CPU fallback)")
    sol = static_settings.get("solution structure", ())
    if any(s != "nodal imposition" for s in sol):
        raise NotImplementedError("the gb300 backend implements 'nodal imposition' of Dirichlet DOFs")


def _out_like(flat_dev, dofs, key):
    """Result with the structure and array type of ``dofs``: NumPy in, NumPy out; torch in,
    torch out; a DLPack array of another framework in, a torch tensor on the device out
    (hand it to that framework's from_dlpack)."""
    ref = dofs[key] if isinstance(dofs, dict) else dofs
    if is_foreign(ref):
        out = flat_dev.reshape(tuple(ref.shape))
    elif isinstance(ref, torch.Tensor):
        out = flat_dev.reshape(ref.shape).to(ref.device)
    else:
        out = flat_dev.cpu().numpy().reshape(np.shape(ref))
    return {key: out} if isinstance(dofs, dict) else out


def solver(dofs, settings, static_settings, **kwargs):
    """General solver (solver.py:41-137): dispatch on static_settings['solver type']."""
    _backend_check(static_settings)
    solver_type = static_settings["solver type"]
    if solver_type == "newton":
        return solve_newton(dofs, settings, static_settings, **kwargs)
    if solver_type == "damped newton":
        return solve_damped_newton(dofs, settings, static_settings, **kwargs)
    if solver_type == "linear":
        return solve_linear(dofs, settings, static_settings, **kwargs), None
    assert False, "Solver type not implemented!"


def solve_newton(dofs, settings, static_settings, newton_tol=1e-8, maxiter=30, **kwargs):
    """Newton-Raphson: damped Newton with damping 1 (solver.py:740-768)."""
    return solve_damped_newton(dofs, settings, static_settings, newton_tol, 1.0, maxiter, **kwargs)


def solve_damped_newton(dofs, settings, static_settings, newton_tol=1e-8, damping_coefficient=0.8, maxiter=30,
                        **kwargs):
    """Damped Newton (solver.py:770-948) with the loop, the assembly and the linear solves
    on the GPU.  Returns (dofs, (n_iter, res_norm, diverged))."""
    global last_info
    _backend_check(static_settings)
    prob = get_problem(dofs, settings, static_settings)
    prob.update_models(settings)
    opts = N.NewtonOpts()
    kopts, tdt = _method(static_settings, kwargs)
    if kopts.method in (N.AGX_FCG_MIXED, N.AGX_FCG_F64):
        _attach_learned(prob, static_settings)
    opts.newton_tol = float(newton_tol)
    opts.newton_rtol = float(kwargs.get("newton_rtol", 0.0))
    opts.maxiter = int(maxiter)
    opts.damping = float(damping_coefficient)
    opts.tangent_dtype = tdt
    opts.krylov = kopts
    opts.reuse_tangent = int(kwargs.get("reuse_tangent", _reuse_default(static_settings)))
    opts.verbose = int(static_settings.get("verbose", 0))
    x = prob.to_device(dofs)
    ref = dofs[prob.key] if isinstance(dofs, dict) else dofs
    if isinstance(ref, torch.Tensor) or is_foreign(ref):
        x = x.clone()  # the caller's array is never modified
    cond = settings.get("dirichlet conditions")
    g = prob.to_device(cond) if cond is not None else torch.zeros(prob.n_dofs, dtype=torch.float64,
                                                                   device=prob.device)
    if kwargs.get("autotune", True):
        prob.ensure_tuned(x, tdt)
    info = N.NewtonInfo()
    prob._call("agx_newton", N.C.c_void_p(x.data_ptr()), N.C.c_void_p(g.data_ptr()), N.C.byref(opts),
               N.C.byref(info))
    last_info = info
    sol = _out_like(x, dofs, prob.key)
    return sol, (int(info.iterations), float(info.res_norm), bool(info.diverged))


def solve_linear(dofs, settings, static_settings, **kwargs):
    """One linear solve with nodal imposition (solver.py:544-659): the returned DOFs hold
    the increment on free DOFs and the prescribed values on Dirichlet DOFs."""
    _backend_check(static_settings)
    prob = get_problem(dofs, settings, static_settings)
    prob.update_models(settings)
    kopts, tdt = _method(static_settings, kwargs)
    if kopts.method in (N.AGX_FCG_MIXED, N.AGX_FCG_F64):
        _attach_learned(prob, static_settings)
    x = prob.to_device(dofs).clone()
    cond = settings.get("dirichlet conditions")
    g = prob.to_device(cond) if cond is not None else torch.zeros_like(x)
    m = torch.as_tensor(prob.mask.astype(bool), device=prob.device)
    x = torch.where(m, g, x)
    R = torch.empty_like(x)
    prob._call("agx_assemble", N.C.c_void_p(x.data_ptr()), N.C.c_void_p(R.data_ptr()), tdt)
    dx = torch.empty_like(x)
    info = N.SolveInfo()
    # agx_solve solves K dx = rhs on the free DOFs; rhs = -R
    rhs = -R
    prob._call("agx_solve", N.C.c_void_p(rhs.data_ptr()), N.C.c_void_p(dx.data_ptr()), N.C.byref(kopts),
               N.C.byref(info))
    if kopts.method == N.AGX_CHOL_BAND and info.status == N.AGX_DIVERGED:
        raise RuntimeError("the direct solve found the tangent not positive (or negative) definite at these DOFs; "
                           "use an iterative solver ('bicgstab') for indefinite tangents")
    out = torch.where(m, g, dx)
    return _out_like(out, dofs, prob.key)


def adaptive_load_stepping(dofs, settings, static_settings,
                           multiplier_settings=lambda settings, multiplier: (
                               settings.update({"load multiplier": multiplier}), settings)[1],
                           path_dependent=True, implicit_diff_mode=None, max_multiplier=1.0, min_increment=0.01,
                           max_increment=1.0, init_increment=0.2, max_load_steps=1000, target_num_newton_iter=7,
                           newton_tol=1e-10, **kwargs):
    """Adaptive load stepping (solver.py:139-457): multiplier loop around :func:`solver` with
    the same increment control, roll-back on divergence and returned carry
    (dofs, multiplier, increment, load_step, settings, res_norm)."""
    if implicit_diff_mode is not None:
        raise NotImplementedError("JAX-traced implicit differentiation needs JAX; use "
                                  "autopdex_gb300.solver.sensitivities on the converged DOFs instead")
    verbose = static_settings.get("verbose", 0)
    multiplier, increment, load_step, res = 0.0, float(init_increment), 0.0, 0.0
    while multiplier < max_multiplier and increment > min_increment:
        multiplier += increment
        if verbose > -1:
            if verbose > 0:
                print("")
            print(f"Multiplier: {multiplier}")
        settings = multiplier_settings(settings, multiplier)
        new, (steps, res, div) = solver(dofs, settings, static_settings, newton_tol=newton_tol, **kwargs)
        if div:
            multiplier -= increment
            increment *= 0.5
        else:
            increment *= 1 + 0.5 * (target_num_newton_iter - steps) / target_num_newton_iter
            dofs = new
        increment = min(increment, max_increment)
        if multiplier + increment > max_multiplier:
            increment = max_multiplier - multiplier
        load_step = 1.0 * load_step
        if multiplier < max_multiplier - min_increment and increment < min_increment:
            print("Adaptive load stepping could not converge; increment size below min_increment!")
    return dofs, multiplier, increment, load_step, settings, res


def _checked_solve(prob, rhs, x, opts, what):
    """agx_solve that raises when the Krylov solve stops without meeting its tolerance
    (iteration limit, breakdown on an indefinite tangent, non-finite values): a derivative from
    an unconverged solve would be returned as if it were exact."""
    info = N.SolveInfo()
    rc = prob._call("agx_solve", N.C.c_void_p(rhs.data_ptr()), N.C.c_void_p(x.data_ptr()), N.C.byref(opts),
                    N.C.byref(info))
    if rc != N.AGX_OK or info.status != N.AGX_OK:
        kind = "diverged (breakdown or non-finite values)" if N.AGX_DIVERGED in (rc, info.status) else \
            "did not converge"
        raise RuntimeError(f"the linear solve of the {what} {kind}: {info.iterations} iterations, relative "
                           f"residual {info.rel_residual:.3e} against a tolerance of {opts.rtol:.1e}")
    return info


def sensitivities(dofs, settings, static_settings, params, rel_step=1e-6, krylov_tol=1e-12, **kwargs):
    """Forward-mode implicit derivatives du/dp of a converged solution with respect to scalar
    settings entries (the 'forward' implicit differentiation of adaptive_load_stepping,
    solver.py:200-300 with implicit_diff.custom_root, implicit_diff.py:487-542, at the final
    state of a path-independent problem): K du/dp = -dR/dp on the free DOFs, du/dp = 0 on
    the prescribed ones.

    K is the float64 tangent at ``dofs`` with Dirichlet elimination; dR/dp is the central
    difference of the float64 residual with step rel_step |p| (exact up to rounding for
    parameters the residual is linear in, such as a Young's modulus; O(step^2) otherwise);
    the linear solves are float64 Jacobi-PCG to ``krylov_tol``.  Returns {key: du/dp} with the
    structure of ``dofs``."""
    _backend_check(static_settings)
    prob = get_problem(dofs, settings, static_settings)
    x = prob.to_device(dofs)
    m = torch.as_tensor(prob.mask.astype(bool), device=prob.device)
    opts = N.SolveOpts()
    opts.method, opts.rtol, opts.atol = N.AGX_PCG, float(krylov_tol), 0.0
    opts.maxiter, opts.check_every = int(kwargs.get("krylov_maxiter", 1000000)), 32
    out = {}
    for key in params:
        p0 = float(np.asarray(settings[key]))
        h = rel_step * (abs(p0) if p0 != 0.0 else 1.0)
        res = []
        for v in (p0 + h, p0 - h):
            st = dict(settings)
            st[key] = v
            prob.update_models(st)
            R = torch.empty_like(x)
            prob._call("agx_assemble", N.C.c_void_p(x.data_ptr()), N.C.c_void_p(R.data_ptr()), -1)
            res.append(R)
        dR = (res[0] - res[1]) / (2.0 * h)
        prob.update_models(settings)
        prob._call("agx_assemble", N.C.c_void_p(x.data_ptr()), None, N.AGX_F64)
        rhs = torch.where(m, torch.zeros_like(dR), -dR)
        du = torch.empty_like(x)
        _checked_solve(prob, rhs, du, opts, f"du/d{key}")
        out[key] = _out_like(du, dofs, prob.key)
    return out


class _DeviceOps:
    """The float64 residual, tangent product and tangent solve of one problem on the GPU, in
    the interface of ``implicit_diff`` (base point ``u`` with ``settings``)."""

    def __init__(self, prob, u, settings, krylov_tol, krylov_maxiter):
        self.prob, self.u, self.settings = prob, u, settings
        self.free = torch.as_tensor(~prob.mask.astype(bool), device=prob.device).to(torch.float64)
        self.opts = N.SolveOpts()
        self.opts.method, self.opts.rtol, self.opts.atol = N.AGX_PCG, float(krylov_tol), 0.0
        self.opts.maxiter, self.opts.check_every = int(krylov_maxiter), 32

    def residual(self, w, settings):
        w = w.contiguous()
        self.prob.update_models(settings)
        R = torch.empty_like(w)
        self.prob._call("agx_assemble", N.C.c_void_p(w.data_ptr()), N.C.c_void_p(R.data_ptr()), -1)
        return R

    def tangent_apply(self, w, settings, v):
        w, v = w.contiguous(), v.contiguous()
        self.prob.update_models(settings)
        self.prob._call("agx_assemble", N.C.c_void_p(w.data_ptr()), None, N.AGX_F64)
        y = torch.empty_like(v)
        self.prob._call("agx_spmv", N.AGX_F64, N.C.c_void_p(v.data_ptr()), N.C.c_void_p(y.data_ptr()))
        return y

    def solve(self, rhs):
        rhs = rhs.contiguous()
        self.prob.update_models(self.settings)
        self.prob._call("agx_assemble", N.C.c_void_p(self.u.data_ptr()), None, N.AGX_F64)
        x = torch.empty_like(rhs)
        _checked_solve(self.prob, rhs, x, self.opts, "implicit differentiation")
        return x


def second_order_sensitivities(dofs, settings, static_settings, params, rel_step=1e-3, dir_step=1e-3,
                               krylov_tol=1e-12, **kwargs):
    """First and second forward implicit derivatives of a converged solution with respect to
    scalar settings entries: what jacfwd of jacfwd of adaptive_load_stepping with
    implicit_diff_mode='forward' gives at the final state of a path-independent problem
    (tests/test_user_elem_impl_diff_and_adaptive_load_step.py:121-133).

    K u_p = -dR/dp, then K u_pq = -D^2 R[(u_p, e_p), (u_q, e_q)] with the second directional
    derivative of the float64 residual from four-point differences of tangent products
    (``implicit_diff.second_directional_residual``); Jacobi-PCG to ``krylov_tol`` for every
    solve.  Returns ``(first, second)``: {key: du/dp} and {(key_p, key_q): d2u/dp dq} (both
    orders of every pair), each with the structure of ``dofs``."""
    from . import implicit_diff
    _backend_check(static_settings)
    prob = get_problem(dofs, settings, static_settings)
    u = prob.to_device(dofs)
    ops = _DeviceOps(prob, u, settings, krylov_tol, kwargs.get("krylov_maxiter", 1000000))
    first = implicit_diff.first_order(ops, u, settings, params, kwargs.get("first_rel_step", 1e-6))
    second = implicit_diff.second_order(ops, u, settings, first, rel_step, dir_step)
    prob.update_models(settings)
    return ({k: _out_like(v, dofs, prob.key) for k, v in first.items()},
            {k: _out_like(v, dofs, prob.key) for k, v in second.items()})


def adjoint_sensitivities(dofs, settings, static_settings, params, dJ_du, rel_step=1e-6, krylov_tol=1e-12,
                          **kwargs):
    """Reverse implicit derivatives dJ/dp of a scalar J(u) of a converged solution (what jacrev
    through adaptive_load_stepping with implicit_diff_mode='backward' gives at the final state
    of a path-independent problem): one adjoint solve K^T lam = dJ/du, then dJ/dp =
    -lam . dR/dp for every entry of ``params``.  ``dJ_du`` has the structure of ``dofs``.  The
    tangent must be symmetric (potential-based models and hyperelastic elements; not the
    backward-Euler 'user residual' model).  Returns {key: float}."""
    from . import implicit_diff
    _backend_check(static_settings)
    if any(getattr(m, "kernel", None) == N.AGX_MODEL_HEAT_BE for m in static_settings["model"]):
        raise NotImplementedError("the adjoint solve needs K^T; the backward-Euler residual model has a "
                                  "non-symmetric tangent")
    prob = get_problem(dofs, settings, static_settings)
    u = prob.to_device(dofs)
    g = prob.to_device(dJ_du)
    ops = _DeviceOps(prob, u, settings, krylov_tol, kwargs.get("krylov_maxiter", 1000000))
    out = implicit_diff.adjoint(ops, u, settings, params, g, rel_step)
    prob.update_models(settings)
    return out


# ---- learned preconditioner hook ------------------------------------------------------
_learned = {}


def set_learned_preconditioner(static_settings_or_key, preconditioner):
    """Register a learned preconditioner (``autopdex_gb300.learned.GridPreconditioner``)
    for problems solved with ``'type of preconditioner': 'learned'``."""
    _learned["default"] = preconditioner


def _attach_learned(prob, static_settings):
    pc = _learned.get("default")
    if static_settings.get("type of preconditioner") != "learned" or pc is None:
        prob._call("agx_set_preconditioner", N.PRECOND_FN(0), None)
        prob.learned = None
        return
    if prob.learned is not pc:
        pc.attach(prob)
