"""Oracle: element routines derived by automatic differentiation (float64, torch.func).

Test infrastructure only (see ``oracle/__init__.py``).  AutoPDEx derives every element
quantity with JAX AD: a 'user potential' gives R = jacrev(Pi) and K = jacfwd(jacrev(Pi))
(assembler.py:1064-1149); a Galerkin 'user element' gives R = jacrev(weak form, test) and
K = jacfwd(R, trial) per Gauss point (models.py:1616-1718); a 'user residual' gives
R = jacrev(weak form, test) and K = jacfwd(R) (models.py:1272-1357, assembler.py:1270-1306).
This module restates those derivations with ``torch.func`` so that the oracle does not rely
on hand-derived tangents.

The physical-gradient rule of ``fem_iso_line_quad_brick(..., overwrite_diff=True)``
(spaces.py:12162-12190) -- d f/dx = (d f/d xi) J^-1 with J = dX/d xi -- is written out
explicitly in :func:`_iso`.
"""
import numpy as np
import torch
from torch.func import jacfwd, jacrev, vmap

from .mesh import shape_functions, gauss_legendre_nd

DT = torch.float64


def _t(a):
    return torch.as_tensor(np.asarray(a), dtype=DT)


def matrix_det(m):
    """Closed-form 1x1..3x3 determinant (utility.matrix_det, utility.py:772-817)."""
    n = m.shape[0]
    if n == 1:
        return m[0, 0]
    if n == 2:
        return m[0, 0] * m[1, 1] - m[0, 1] * m[1, 0]
    a, b, c = m[0, 0], m[0, 1], m[0, 2]
    d, e, f = m[1, 0], m[1, 1], m[1, 2]
    g, h, i = m[2, 0], m[2, 1], m[2, 2]
    return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g)


def matrix_inv(m):
    """Closed-form inverse by the adjugate (utility.matrix_inv, utility.py:706-770)."""
    n = m.shape[0]
    if n == 1:
        return 1.0 / m
    if n == 2:
        det = matrix_det(m)
        return torch.stack([torch.stack([m[1, 1], -m[0, 1]]), torch.stack([-m[1, 0], m[0, 0]])]) / det
    a, b, c = m[0, 0], m[0, 1], m[0, 2]
    d, e, f = m[1, 0], m[1, 1], m[1, 2]
    g, h, i = m[2, 0], m[2, 1], m[2, 2]
    adj = torch.stack([
        torch.stack([e * i - f * h, c * h - b * i, b * f - c * e]),
        torch.stack([f * g - d * i, a * i - c * g, c * d - a * f]),
        torch.stack([d * h - e * g, b * g - a * h, a * e - b * d])])
    return adj / matrix_det(m)


def _iso(xi, xI, fI, n_dim, nen):
    """Value and physical gradient of the isoparametric field at reference point ``xi``.

    ``xI``: (nen, dim) nodal coordinates; ``fI``: (nen,) or (nen, nf) nodal values.
    Returns (N, f, grad_f, x, detJ) with grad_f of shape (dim,) or (nf, dim).
    """
    N = shape_functions(xi, n_dim, nen, xp=torch)
    dN = jacfwd(lambda z: shape_functions(z, n_dim, nen, xp=torch))(xi)  # (nen, n_dim)
    J = xI.T @ dN  # dX/dxi, (dim, n_dim)
    Jinv = matrix_inv(J)
    dNdx = dN @ Jinv  # (nen, dim)
    f = torch.tensordot(N, fI, dims=([0], [0]))
    g = torch.tensordot(fI, dNdx, dims=([0], [0]))  # (dim,) or (nf, dim)
    x = N @ xI
    return N, f, g, x, matrix_det(J)


# ----------------------------------------------------------------------------------
# 'user potential' built from models.mixed_reference_domain_potential (models.py:1188-1269)
# ----------------------------------------------------------------------------------
def poisson_sincos_integrand(amp=20.0, freq=10.0, center=(1.0, 0.5)):
    """The integrand of the reference's golden test and short example:
    1/2 grad(phi).grad(phi) - b(x) phi,  b = amp (sin(freq x.x) - cos(freq (x-c).(x-c)))
    (tests/test_dicts_as_dofs_user_potential.py:25-35)."""
    c = torch.tensor(center, dtype=DT)

    def integrand(x, phi, g, elem_params):
        x2 = x - c
        b = amp * (torch.sin(freq * (x @ x)) - torch.cos(freq * (x2 @ x2)))
        return 0.5 * (g @ g) - b * phi
    return integrand


def heat_potential_integrand(source=1.0):
    """1/2 k_e grad(T).grad(T) - f T with an element-wise conductivity k_e."""
    def integrand(x, phi, g, elem_params):
        return 0.5 * elem_params[0] * (g @ g) - source * phi
    return integrand


def user_potential_element(integrand, dim, nen, order=2, rule=None):
    """Returns fun(fI, xI, elem_params) -> (R_e, K_e) for a scalar field potential; ``rule``
    (points, weights) replaces the Gauss-Legendre rule (simplex elements)."""
    xq, wq = rule if rule is not None else gauss_legendre_nd(dim, order)
    xq = _t(xq)
    wq = _t(wq)

    def potential(fI, xI, p):
        tot = torch.zeros((), dtype=DT)
        for q in range(xq.shape[0]):
            N, f, g, x, detJ = _iso(xq[q], xI, fI, dim, nen)
            tot = tot + integrand(x, f, g, p) * wq[q] * detJ
        return tot

    R = jacrev(potential, argnums=0)
    K = jacfwd(R, argnums=0)
    return lambda fI, xI, p: (R(fI, xI, p), K(fI, xI, p))


# ----------------------------------------------------------------------------------
# 'user element': hyperelastic_steady_state_weak + neo_hooke + isoparametric_domain_element_galerkin
# (models.py:917-1000, :1122-1146, :1616-1718)
# ----------------------------------------------------------------------------------
def neo_hooke(F, lam, mu):
    """Ciarlet neo-Hooke: mu/2 (tr C - 3 - 2 ln J) + lam/4 (J^2 - 1 - 2 ln J) (models.py:1122-1146)."""
    trC = torch.sum(F * F)
    J = matrix_det(F)
    lnJ = torch.log(J)
    return (mu / 2) * (trC - 3 - 2 * lnJ) + (lam / 4) * (J ** 2 - 1 - 2 * lnJ)


def lame(E, nu):
    """Lame parameters as models.py:955-956."""
    return E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))


def hyperelastic_element(dim, nen, order, mode, rule=None):
    """Returns fun(uI, xI, (E, nu)) -> (R_e (nen*dim,), K_e (nen*dim, nen*dim)).

    Per Gauss point: P = jacrev(psi)(F), weak form P:dF, R = jacrev(weak, test),
    K = jacfwd(R, trial) (models.py:1674-1711); plane strain embeds the 2x2
    displacement gradient into a 3x3 F with F33 = 1 (models.py:963-976).  ``rule``
    (points, weights) replaces the Gauss-Legendre rule (simplex elements).
    """
    xq, wq = rule if rule is not None else gauss_legendre_nd(dim, order)
    xq = _t(xq)
    wq = _t(wq)

    def embed(H):
        if mode == "plain strain":
            return torch.nn.functional.pad(H, (0, 1, 0, 1))
        return H

    def weak(test_uI, trial_uI, xI, params, q):
        E, nu = params[0], params[1]
        lam, mu = lame(E, nu)
        _, _, Hu, _, detJ = _iso(xq[q], xI, trial_uI, dim, nen)
        _, _, Hv, _, _ = _iso(xq[q], xI, test_uI, dim, nen)
        F = embed(Hu) + torch.eye(3, dtype=DT)
        P = jacrev(neo_hooke, argnums=0)(F, lam, mu)
        return wq[q] * detJ * torch.sum(P * embed(Hv))

    def fun(uI, xI, params):
        Rt = torch.zeros(nen * dim, dtype=DT)
        Kt = torch.zeros((nen * dim, nen * dim), dtype=DT)
        for q in range(xq.shape[0]):
            rfun = jacrev(weak, argnums=0)
            r = rfun(uI, uI, xI, params, q).reshape(-1)
            k = jacfwd(lambda tr: rfun(uI, tr, xI, params, q).reshape(-1))(uI).reshape(nen * dim, nen * dim)
            Rt = Rt + r
            Kt = Kt + k
        return Rt, Kt
    return fun


# ----------------------------------------------------------------------------------
# Neumann traction: neumann_weak + isoparametric_surface_element_galerkin, 2-D line
# (models.py:744-780, :1723-1851; tangent_contributions=False)
# ----------------------------------------------------------------------------------
def neumann_line_element(nen, order):
    """Returns fun(xI (nen,2), traction (2,)) -> R_e (nen*2,).

    R_a,i = -sum_q N_a(xi_q) t_i w_q |G1 x E3|, G1 = dX/dxi (models.py:1818-1827).
    """
    xq, wq = gauss_legendre_nd(1, order)

    def fun(xI, t):
        xI = np.asarray(xI, dtype=np.float64)
        R = np.zeros((nen, 2))
        for q in range(len(xq)):
            N = shape_functions(xq[q], 1, nen)
            dN = np.asarray(jacfwd(lambda z: shape_functions(z, 1, nen, xp=torch))(torch.tensor(xq[q], dtype=DT)))
            G1 = dN @ xI
            scale = np.linalg.norm(G1)
            R += -np.outer(N, t) * wq[q] * scale
        return R.reshape(-1)
    return fun


# ----------------------------------------------------------------------------------
# 'user residual': backward-Euler nonlinear heat conduction weak form
# (models.mixed_reference_domain_residual, models.py:1272-1357; assembler.py:1216-1306)
# ----------------------------------------------------------------------------------
def nonlinear_heat_be_element(dim, nen, order=2):
    """Returns fun(TI, TnI, xI, (k0, k2, rho_c, dt)) -> (R_e, K_e).

    Weak form per Gauss point: rho_c (T - T_n)/dt v + (k0 + k2 T^2) grad T . grad v;
    R = jacrev(weak, test), K = jacfwd(R, trial).  K is not symmetric (k'(T) term).
    """
    xq, wq = gauss_legendre_nd(dim, order)
    xq = _t(xq)
    wq = _t(wq)

    def weak(test, trial, TnI, xI, p):
        k0, k2, rc, dt = p[0], p[1], p[2], p[3]
        tot = torch.zeros((), dtype=DT)
        for q in range(xq.shape[0]):
            _, T, gT, _, detJ = _iso(xq[q], xI, trial, dim, nen)
            _, v, gv, _, _ = _iso(xq[q], xI, test, dim, nen)
            _, Tn, _, _, _ = _iso(xq[q], xI, TnI, dim, nen)
            tot = tot + (rc * (T - Tn) / dt * v + (k0 + k2 * T * T) * (gT @ gv)) * wq[q] * detJ
        return tot

    def fun(TI, TnI, xI, p):
        rfun = jacrev(weak, argnums=0)
        R = rfun(TI, TI, TnI, xI, p)
        K = jacfwd(lambda tr: rfun(TI, tr, TnI, xI, p))(TI)
        return R, K
    return fun


def batched(fun, *args, chunk=4096):
    """vmap ``fun`` over the leading axis of every argument (element batches)."""
    vf = vmap(fun)
    n = args[0].shape[0]
    outs = []
    for s in range(0, n, chunk):
        outs.append(vf(*[a[s:s + chunk] for a in args]))
    if isinstance(outs[0], tuple):
        return tuple(torch.cat([o[i] for o in outs]) for i in range(len(outs[0])))
    return torch.cat(outs)
