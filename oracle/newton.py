"""Oracle: global assembly, SciPy linear solve and the damped Newton loop (float64).

Test infrastructure only (see ``oracle/__init__.py``).

A problem is a list of element *sets* sharing one flat DOF vector laid out node-major
(``dof = node * ndof + component``), which is how AutoPDEx numbers the DOFs of a
single-field dict or an ``(n_nodes, ndof)`` array (assembler.py:47-141, :331-436).
"""
import numpy as np
import scipy.sparse
import scipy.sparse.linalg
import torch

from . import elements as el

DT = torch.float64


class ElementSet:
    """One domain of the problem ('assembling mode' entry).

    kind: 'potential' | 'element' | 'residual' | 'neumann'
    fun:  the element routine from ``oracle.elements``
    params(settings) -> per-element parameters, shape (n_e, p)
    """

    def __init__(self, kind, conn, fun, params, ndof, traction=None):
        self.kind = kind
        self.conn = np.asarray(conn, dtype=np.int64)
        self.fun = fun
        self.params = params
        self.ndof = ndof
        self.traction = traction

    def element_dofs(self):
        """Global DOF indices per element, node-major: (n_e, nen*ndof)."""
        c = self.conn[:, :, None] * self.ndof + np.arange(self.ndof)[None, None, :]
        return c.reshape(self.conn.shape[0], -1)


def element_contributions(s, dofs, coords, settings):
    """R_e (n_e, m) and K_e (n_e, m, m) for every element of set ``s``."""
    conn = s.conn
    xI = torch.as_tensor(coords[conn], dtype=DT)
    if s.kind == "neumann":
        t = s.traction(settings)
        R = np.stack([s.fun(coords[c], t) for c in conn])
        m = R.shape[1]
        return R, np.zeros((conn.shape[0], m, m))
    p = torch.as_tensor(s.params(settings), dtype=DT)
    if s.ndof == 1:
        fI = torch.as_tensor(dofs[conn], dtype=DT)
    else:
        fI = torch.as_tensor(dofs.reshape(-1, s.ndof)[conn], dtype=DT)
    if s.kind == "residual":
        TnI = torch.as_tensor(np.asarray(settings["dofs n"]).reshape(-1)[conn], dtype=DT)
        R, K = el.batched(s.fun, fI, TnI, xI, p)
    else:
        R, K = el.batched(s.fun, fI, xI, p)
    n_e = conn.shape[0]
    return R.reshape(n_e, -1).numpy(), K.reshape(n_e, R.reshape(n_e, -1).shape[1], -1).numpy()


def assemble(sets, dofs, coords, settings, n_dofs, tangent=True):
    """Residual (n_dofs,) and the COO tangent with duplicates (rows, cols, data).

    Residual: scatter-add of element vectors (assembler.py:331-436).  Tangent entries in
    the order of ``_get_indices`` -- per element, rows repeated, columns tiled
    (assembler.py:123-141) -- with the duplicates kept, as the BCOO of
    assembler.py:1142-1148 keeps them.
    """
    R = np.zeros(n_dofs)
    rows, cols, data = [], [], []
    for s in sets:
        Re, Ke = element_contributions(s, dofs, coords, settings)
        ed = s.element_dofs()
        np.add.at(R, ed.ravel(), Re.ravel())
        if tangent:
            m = ed.shape[1]
            rows.append(np.repeat(ed, m, axis=1).ravel())
            cols.append(np.tile(ed, (1, m)).ravel())
            data.append(Ke.reshape(-1))
    if not tangent:
        return R, None
    return R, (np.concatenate(rows), np.concatenate(cols), np.concatenate(data))


def scipy_assembling(coo, n_dofs, free):
    """COO -> CSR with duplicates summed, then Dirichlet columns and rows deleted
    (solver.py:1180-1222)."""
    rows, cols, data = coo
    A = scipy.sparse.csr_matrix(scipy.sparse.coo_matrix((data, (rows, cols)), shape=(n_dofs, n_dofs)))
    if free is not None:
        A = A[:, free]
        A = A[free]
    return A


def linear_solve_scipy(coo, rhs, n_dofs, free):
    """spsolve on the reduced system; zeros on Dirichlet entries (solver.py:1493-1539)."""
    A = scipy_assembling(coo, n_dofs, free)
    b = rhs[free] if free is not None else rhs
    x = scipy.sparse.linalg.spsolve(A.tocsc(), b)
    sol = np.zeros_like(rhs)
    if free is not None:
        sol[free] = x
    else:
        sol[:] = x
    return sol


def linear_solve_cg_jacobi(coo, rhs, n_dofs, free, rtol=1e-10, maxiter=100000):
    """Jacobi-preconditioned CG on the reduced assembled system (the algorithm of the
    reference's 'jax' backend with 'cg' + 'jacobi', solver.py:1093-1116, on an assembled
    matrix instead of a matrix-free product)."""
    A = scipy_assembling(coo, n_dofs, free)
    b = rhs[free]
    d = A.diagonal()
    M = scipy.sparse.linalg.LinearOperator(A.shape, matvec=lambda v: v / d)
    x, info = scipy.sparse.linalg.cg(A, b, rtol=rtol, atol=0.0, M=M, maxiter=maxiter)
    sol = np.zeros_like(rhs)
    sol[free] = x
    return sol


class Problem:
    """settings/static_settings equivalent for the oracle."""

    def __init__(self, sets, coords, n_dofs, dirichlet_mask, dirichlet_values, linear_solver="lapack"):
        self.sets = sets
        self.coords = np.asarray(coords, dtype=np.float64)
        self.n_dofs = n_dofs
        self.dirichlet = np.asarray(dirichlet_mask, dtype=bool).reshape(-1)
        self.values = np.asarray(dirichlet_values, dtype=np.float64).reshape(-1)
        self.linear_solver = linear_solver

    def residual(self, dofs, settings):
        return assemble(self.sets, dofs, self.coords, settings, self.n_dofs, tangent=False)[0]

    def solve_linear(self, dofs, settings):
        """solver.solve_linear with nodal imposition (solver.py:544-659): set the Dirichlet
        values, rhs = -R, solve on the free DOFs, return dofs with free entries replaced by
        the increment and Dirichlet entries holding the prescribed values."""
        dofs = np.where(self.dirichlet, self.values, dofs)
        R, coo = assemble(self.sets, dofs, self.coords, settings, self.n_dofs)
        free = ~self.dirichlet
        if self.linear_solver == "lapack":
            sol = linear_solve_scipy(coo, -R, self.n_dofs, free)
        else:
            sol = linear_solve_cg_jacobi(coo, -R, self.n_dofs, free)
        return np.where(free, sol, dofs)


def damped_newton(problem, dofs0, settings, newton_tol=1e-8, maxiter=30, damping=1.0, verbose=-1):
    """solver.damped_newton (solver.py:837-948), one loop iteration per step:
    solve, damped update of the free DOFs, Dirichlet DOFs set, residual norm over the free
    DOFs, stop at ||R_free|| <= tol, divergence if the norm grows tenfold after the second
    iteration or is NaN/Inf, and a final forced stop after ``maxiter``."""
    free = ~problem.dirichlet
    dofs = np.asarray(dofs0, dtype=np.float64).reshape(-1).copy()
    itt, not_stop, res_old, div = 0, True, 0.0, False
    history = []
    while not_stop:
        delta = problem.solve_linear(dofs, settings)
        delta = np.where(free, damping * delta, delta)
        dofs = np.where(free, dofs + delta, delta)
        R = problem.residual(dofs, settings)
        rf = np.where(free, R, 0.0)
        res = float(np.linalg.norm(rf))
        history.append(res)
        keep = res > newton_tol
        if itt < maxiter:
            with np.errstate(divide="ignore", invalid="ignore"):
                div = bool((res / res_old > 10 if res_old != 0 else res > 0) and itt > 1)
            if not np.all(np.isfinite(rf)):
                div = True
            nxt = not div
        else:
            nxt, div = False, True
        itt += 1
        res_old = res
        not_stop = keep and nxt
    return dofs, (itt, res, div), history


def load_stepping(problem, dofs0, settings, multipliers, set_multiplier, newton_tol=1e-10, maxiter=30):
    """Fixed load steps, each a Newton solve started from the previous solution (the loop of
    solver.adaptive_load_stepping, solver.py:308-378, with prescribed increments)."""
    dofs = np.asarray(dofs0, dtype=np.float64).reshape(-1).copy()
    infos = []
    for m in multipliers:
        settings = set_multiplier(settings, m)
        problem.values = settings.get("__dirichlet_values__", problem.values)
        dofs, info, _ = damped_newton(problem, dofs, settings, newton_tol, maxiter)
        infos.append(info)
    return dofs, infos


def implicit_sensitivity(problem, dofs, settings, key, rel_step=1e-6):
    """du/dp of a converged solution for a scalar settings entry p (forward implicit
    differentiation at the final state, as adaptive_load_stepping's implicit_diff_mode
    'forward' with implicit_diff.custom_root, solver.py:200-300, implicit_diff.py:487-542):
    K du = -dR/dp on the free DOFs, dR/dp by a central difference of the residual."""
    p0 = float(settings[key])
    h = rel_step * (abs(p0) if p0 != 0.0 else 1.0)
    res = []
    for v in (p0 + h, p0 - h):
        st = dict(settings)
        st[key] = v
        res.append(problem.residual(dofs, st))
    dR = (res[0] - res[1]) / (2.0 * h)
    _, coo = assemble(problem.sets, dofs, problem.coords, settings, problem.n_dofs)
    return linear_solve_scipy(coo, -dR, problem.n_dofs, ~problem.dirichlet)


def _param_direction(s, settings, key):
    """d(element parameters)/d settings[key] for a set whose parameters are affine in that
    entry (checked with two unit steps)."""
    def at(v):
        st = dict(settings)
        st[key] = float(np.asarray(settings[key])) + v
        return np.asarray(s.params(st), dtype=np.float64)
    base = at(0.0)
    d1, d2 = at(1.0) - base, (at(2.0) - base) / 2.0
    if not np.allclose(d1, d2, rtol=1e-12, atol=1e-14 * (1.0 + np.abs(base).max())):
        raise NotImplementedError("element parameters must be affine in the differentiated settings entry")
    return d1


def _traction_second(s, settings, key_i, key_j):
    """Second mixed difference of a Neumann set's traction in two settings entries, exact for a
    traction of degree <= 2 in them (unit steps)."""
    def at(a, b):
        st = dict(settings)
        st[key_i] = float(np.asarray(st[key_i])) + a
        st[key_j] = float(np.asarray(st[key_j])) + b
        return np.asarray(s.traction(st), dtype=np.float64)
    return at(1.0, 1.0) - at(1.0, 0.0) - at(0.0, 1.0) + at(0.0, 0.0)


def second_directional_residual(problem, dofs, settings, du_i, key_i, du_j, key_j):
    """D^2 R[d_i, d_j], the second derivative of the residual along the two directions
    d = (du/dp, e_p) of (dofs, settings entry p), exact by nested forward-mode AD
    (torch.func.jvp) of the element residuals; Neumann sets by the traction's second
    difference (the traction enters the residual linearly)."""
    from torch.func import jvp
    D2 = np.zeros(problem.n_dofs)
    for s in problem.sets:
        ed = s.element_dofs()
        if s.kind == "neumann":
            t2 = _traction_second(s, settings, key_i, key_j)
            Re = np.stack([s.fun(problem.coords[c], t2) for c in s.conn])
            np.add.at(D2, ed.ravel(), Re.ravel())
            continue
        conn = s.conn
        xI = torch.as_tensor(problem.coords[conn], dtype=DT)
        p = torch.as_tensor(s.params(settings), dtype=DT)
        dpi = torch.as_tensor(_param_direction(s, settings, key_i), dtype=DT)
        dpj = torch.as_tensor(_param_direction(s, settings, key_j), dtype=DT)
        shape = (-1,) if s.ndof == 1 else (-1, s.ndof)
        fI = torch.as_tensor(np.asarray(dofs).reshape(shape)[conn], dtype=DT)
        fIi = torch.as_tensor(np.asarray(du_i).reshape(shape)[conn], dtype=DT)
        fIj = torch.as_tensor(np.asarray(du_j).reshape(shape)[conn], dtype=DT)
        if s.kind == "residual":
            TnI = torch.as_tensor(np.asarray(settings["dofs n"]).reshape(-1)[conn], dtype=DT)
            res = lambda f, q, xe, tn: s.fun(f, tn, xe, q)[0].reshape(-1)
            extra = (TnI,)
        else:
            res = lambda f, q, xe: s.fun(f, xe, q)[0].reshape(-1)
            extra = ()

        def one(f, q, xe, fi, qi, fj, qj, *ex):
            first = lambda a, b: jvp(lambda u, v: res(u, v, xe, *ex), (a, b), (fi, qi))[1]
            return jvp(first, (f, q), (fj, qj))[1]
        Re = el.batched(one, fI, p, xI, fIi, dpi, fIj, dpj, *extra)
        np.add.at(D2, ed.ravel(), Re.reshape(conn.shape[0], -1).numpy().ravel())
    return D2


def implicit_second_sensitivity(problem, dofs, settings, du_i, key_i, du_j, key_j):
    """d^2u/(dp_i dp_j) of a converged solution (forward-over-forward implicit
    differentiation, as jacfwd of jacfwd of adaptive_load_stepping with implicit_diff_mode
    'forward', tests/test_user_elem_impl_diff_and_adaptive_load_step.py:121-133): from
    R(u(p), p) = 0, K u_ij = -D^2 R[d_i, d_j] with d = (u_p, e_p), on the free DOFs."""
    D2 = second_directional_residual(problem, dofs, settings, du_i, key_i, du_j, key_j)
    _, coo = assemble(problem.sets, dofs, problem.coords, settings, problem.n_dofs)
    return linear_solve_scipy(coo, -D2, problem.n_dofs, ~problem.dirichlet)


def adjoint_sensitivity(problem, dofs, settings, dJ_du, key, rel_step=1e-6):
    """dJ/dp of a scalar J(u) of a converged solution by reverse implicit differentiation
    (implicit_diff_mode 'backward' with jacrev): K^T lam = dJ/du on the free DOFs,
    dJ/dp = -lam . dR/dp."""
    p0 = float(settings[key])
    h = rel_step * (abs(p0) if p0 != 0.0 else 1.0)
    res = []
    for v in (p0 + h, p0 - h):
        st = dict(settings)
        st[key] = v
        res.append(problem.residual(dofs, st))
    dR = (res[0] - res[1]) / (2.0 * h)
    _, coo = assemble(problem.sets, dofs, problem.coords, settings, problem.n_dofs)
    rows, cols, data = coo
    lam = linear_solve_scipy((cols, rows, data), np.asarray(dJ_du, dtype=np.float64), problem.n_dofs,
                             ~problem.dirichlet)
    return -float(lam[~problem.dirichlet] @ dR[~problem.dirichlet])
