"""Implicit derivatives of a converged solution of R(u, p) = 0 with respect to scalar settings
entries p: second-order forward and first-order reverse (adjoint) modes.

AutoPDEx differentiates ``adaptive_load_stepping`` through ``implicit_diff.custom_root``
(implicit_diff.py:487-542, wired up at solver.py:200-300) with jacfwd ('forward') or jacrev
('backward'), and nests jacfwd for second derivatives
(tests/test_user_elem_impl_diff_and_adaptive_load_step.py:121-148).  At the final state of a
path-independent problem those transforms reduce to linear solves with the tangent K:

* first order, forward:  K u_i = -R_p_i;
* second order, forward: K u_ij = -D^2 R[d_i, d_j], the second derivative of the residual
  along the directions d = (u_p, e_p) of (DOFs, settings entry);
* first order, reverse, for a scalar J(u): K^T lam = dJ/du, dJ/dp = -lam . R_p, one solve for
  every p.

The algebra here works on any vector type with ``+ - *`` and ``.sum()`` (the backend's
float64 device tensors) through four operations a backend supplies:

* ``residual(w, settings)``: R(w) for the settings' parameters (all rows);
* ``tangent_apply(w, settings, v)``: K(w) v on the free rows for v zero on prescribed DOFs;
* ``solve(rhs)``: K(u)^-1 rhs on the free DOFs, zero on prescribed ones, at the base point;
* ``free``: 1 on free DOFs, 0 on prescribed ones (same vector type).

Parameter derivatives of the residual are central differences (exact up to rounding for
parameters the residual is affine in, such as Young's modulus); the directional derivative of
``K u_i + R_p_i`` along d_j is a central difference of exact tangent products and of those
residual differences.  First order uses the two-point stencil (O(h^2)), second order the
four-point one (O(h^4)), so that wider steps keep the rounding of the nested differences small.
"""


def _with(settings, key, value):
    st = dict(settings)
    st[key] = value
    return st


def _step(p0, rel):
    return rel * (abs(p0) if p0 != 0.0 else 1.0)


def _central(f, h, points):
    """f'(0) from f(+-h) (two points, O(h^2)) or f(+-h), f(+-2h) (four points, O(h^4))."""
    d1 = f(h) - f(-h)
    if points == 2:
        return d1 * (1.0 / (2.0 * h))
    return (d1 * 8.0 - (f(2.0 * h) - f(-2.0 * h))) * (1.0 / (12.0 * h))


def residual_parameter_derivative(ops, w, settings, key, rel_step=1e-6, points=2):
    """dR/dp at state ``w`` by a central difference with step rel_step |p|."""
    p0 = float(settings[key])
    return _central(lambda e: ops.residual(w, _with(settings, key, p0 + e)), _step(p0, rel_step), points)


def first_order(ops, u, settings, keys, rel_step=1e-6):
    """{p: du/dp}: K u_p = -R_p on the free DOFs."""
    return {k: ops.solve(-residual_parameter_derivative(ops, u, settings, k, rel_step) * ops.free) for k in keys}


def second_directional_residual(ops, u, settings, du_i, key_i, du_j, key_j, rel_step=1e-3, dir_step=1e-3):
    """D^2 R[d_i, d_j] with d = (du/dp, e_p): the four-point central difference, along d_j
    with step t = dir_step |p_j|, of G_i(w, s) = K(w, s) u_i + R_p_i(w, s), whose parameter
    derivative is a four-point central difference with step rel_step |p_i|."""
    pj = float(settings[key_j])

    def G(e):
        w = u + du_j * e
        st = _with(settings, key_j, pj + e)
        return ops.tangent_apply(w, st, du_i) + residual_parameter_derivative(ops, w, st, key_i, rel_step, 4)
    return _central(G, _step(pj, dir_step), 4)


def second_order(ops, u, settings, first, rel_step=1e-3, dir_step=1e-3):
    """{(p_i, p_j): d^2u/dp_i dp_j} for every ordered pair of the keys of ``first``
    ({p: du/dp}); each unordered pair is solved once (the result is symmetric)."""
    keys = list(first)
    out = {}
    for a, ki in enumerate(keys):
        for kj in keys[a:]:
            D2 = second_directional_residual(ops, u, settings, first[ki], ki, first[kj], kj, rel_step, dir_step)
            out[(ki, kj)] = ops.solve(-D2 * ops.free)
            out[(kj, ki)] = out[(ki, kj)]
    return out


def adjoint(ops, u, settings, keys, dJ_du, rel_step=1e-6):
    """{p: dJ/dp} for a scalar J(u) with gradient ``dJ_du``: one solve K^T lam = dJ/du (the
    backend passes a symmetric tangent, K^T = K) and one residual difference per p."""
    lam = ops.solve(dJ_du * ops.free)
    return {k: -float((lam * residual_parameter_derivative(ops, u, settings, k, rel_step) * ops.free).sum())
            for k in keys}
