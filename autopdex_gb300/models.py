"""Model descriptors for the GB300 backend, built with the names of AutoPDEx's builders.

AutoPDEx's ``static_settings['model']`` holds JAX closures that the assembler
differentiates (models.py).  Arbitrary Python cannot run inside a CUDA kernel, so this
backend accepts descriptors that name one of its element kernels and carry the model's
parameters.  The builders below take the same arguments as their AutoPDEx namesakes;
only the innermost callable (the integrand or the strain energy) is replaced by a
descriptor from this module.  An unknown integrand raises ``NotImplementedError``:
there is no CPU fallback.

Supported (element kernel <- AutoPDEx construction):

* ``mixed_reference_domain_potential(poisson_sincos_integrand(...), ...)``
    'user potential' of tests/test_dicts_as_dofs_user_potential.py (models.py:1188-1269)
* ``mixed_reference_domain_potential(heat_conduction_integrand(...), ...)``
    'user potential' 1/2 k_e |grad T|^2 - f T with an element-wise conductivity
* ``isoparametric_domain_element_galerkin(hyperelastic_steady_state_weak(neo_hooke, E, nu, mode), ...)``
    'user element', models.py:917-1000, :1122-1146, :1616-1718
* ``isoparametric_surface_element_galerkin(neumann_weak(traction), ..., tangent_contributions=False)``
    'user element' on 2-node lines, models.py:744-780, :1723-1851
* ``mixed_reference_domain_residual(heat_backward_euler_integrand(...), ...)``
    'user residual' backward Euler, k(T) = k0 + k2 T^2, models.py:1272-1357
"""
from inspect import signature

import numpy as np

from . import _native as N
from . import seeder, spaces


# ------------------------------------------------------------------------------------
# integrand descriptors
# ------------------------------------------------------------------------------------
class Integrand:
    """Names a kernel-side integrand and its parameters."""

    def __init__(self, kind, **params):
        self.kind = kind
        self.params = params

    def __repr__(self):
        return f"Integrand({self.kind!r}, {self.params})"


def poisson_sincos_integrand(amplitude=20.0, frequency=10.0, center=(1.0, 0.5)):
    """1/2 grad(phi).grad(phi) - b(x) phi with
    b = amplitude (sin(frequency x.x) - cos(frequency (x - center).(x - center))),
    the integrand of AutoPDEx's user-potential test (test_dicts_as_dofs_user_potential.py:25-35)."""
    return Integrand("poisson_sincos", amplitude=float(amplitude), frequency=float(frequency),
                     center=tuple(float(c) for c in center))


def heat_conduction_integrand(conductivity="conductivity", source=1.0):
    """1/2 k |grad T|^2 - f T.  ``conductivity`` is a float or the settings key of a
    per-element array; ``source`` is a float or a settings key of a scalar."""
    return Integrand("heat", conductivity=conductivity, source=source)


def heat_backward_euler_integrand(k0=1.0, k2=0.5, rho_c=1.0, time_increment="time increment",
                                  dofs_n="dofs n"):
    """Weak form rho_c (T - T_n)/dt v + (k0 + k2 T^2) grad T . grad v of backward-Euler
    nonlinear heat conduction, T_n = settings[dofs_n], dt = settings[time_increment]."""
    return Integrand("heat_be", k0=k0, k2=k2, rho_c=rho_c, time_increment=time_increment, dofs_n=dofs_n)


# ------------------------------------------------------------------------------------
# strain energy / weak forms (AutoPDEx names)
# ------------------------------------------------------------------------------------
def neo_hooke(F, param):
    """Ciarlet neo-Hooke strain energy (models.py:1122-1146); host evaluation only.
    Passing this function to ``hyperelastic_steady_state_weak`` selects the kernel."""
    lam, mu = param
    F = np.asarray(F, dtype=np.float64)
    J = np.linalg.det(F)
    return mu / 2 * (np.sum(F * F) - 3 - 2 * np.log(J)) + lam / 4 * (J ** 2 - 1 - 2 * np.log(J))


class WeakForm:
    def __init__(self, kind, **params):
        self.kind = kind
        self.params = params


def hyperelastic_steady_state_weak(strain_energy_fun, youngs_mod_fun, poisson_ratio_fun, mode,
                                   volume_load_fun=None):
    """Descriptor of models.hyperelastic_steady_state_weak (models.py:917-1000)."""
    if strain_energy_fun is not neo_hooke:
        raise NotImplementedError("the gb300 backend implements the neo_hooke strain energy only")
    if mode not in ("plain strain", "3d"):
        raise NotImplementedError("Hyperelastic model supports only 'plain strain' and '3d' modes.")
    if volume_load_fun is not None:
        raise NotImplementedError("volume loads are not implemented in the gb300 backend")
    return WeakForm("neo_hooke", E=youngs_mod_fun, nu=poisson_ratio_fun, mode=mode)


def neumann_weak(neumann_fun):
    """Descriptor of models.neumann_weak (models.py:744-780): -t(x).v on the boundary;
    ``neumann_fun(x)`` or ``neumann_fun(x, settings)`` must not depend on x."""
    return WeakForm("neumann", traction=neumann_fun)


# ------------------------------------------------------------------------------------
# element builders
# ------------------------------------------------------------------------------------
class ModelDescriptor:
    """What ``static_settings['model'][set]`` holds for the gb300 backend."""

    def __init__(self, mode, kernel, integrand=None, weak=None, field_key=None, dim=None, ngauss=2, rule=None):
        self.mode = mode            # 'user potential' | 'user element' | 'user residual'
        self.kernel = kernel        # AGX_MODEL_*
        self.integrand = integrand
        self.weak = weak
        self.field_key = field_key
        self.dim = dim
        self.ngauss = ngauss        # Gauss-Legendre points per reference direction
        # simplex spaces: the integration points and weights as given to the builder
        self.qpoints, self.qweights = rule if rule is not None else (None, None)

    def resolve(self, settings, coords, conn):
        """(model id, params, per-element field or None, per-node field or None)."""
        k = self.kernel
        if k == N.AGX_MODEL_POISSON_SINCOS:
            p = self.integrand.params
            c = list(p["center"])
            if len(c) != coords.shape[1]:
                raise ValueError("center must have one entry per space dimension")
            return k, [p["amplitude"], p["frequency"]] + c, None, None
        if k == N.AGX_MODEL_HEAT_POTENTIAL:
            p = self.integrand.params
            f = _scalar(p["source"], settings, coords)
            cond = p["conductivity"]
            if isinstance(cond, str):
                field = np.asarray(settings[cond], dtype=np.float64).reshape(-1)
                if field.shape[0] != conn.shape[0]:
                    raise ValueError(f"settings[{cond!r}] must hold one value per element")
            else:
                field = np.full(conn.shape[0], float(cond))
            return k, [f], field, None
        if k == N.AGX_MODEL_NEO_HOOKE:
            w = self.weak.params
            return k, [_scalar(w["E"], settings, coords), _scalar(w["nu"], settings, coords)], None, None
        if k == N.AGX_MODEL_NEUMANN:
            t = np.asarray(_call_xs(self.weak.params["traction"], settings, coords), dtype=np.float64).reshape(-1)
            return k, list(t), None, None
        if k == N.AGX_MODEL_HEAT_BE:
            p = self.integrand.params
            dt = _scalar(p["time_increment"], settings, coords)
            return k, [_scalar(p["k0"], settings, coords), _scalar(p["k2"], settings, coords),
                       _scalar(p["rho_c"], settings, coords), dt], None, p["dofs_n"]
        raise NotImplementedError(f"unknown kernel {k}")


def _call_xs(fun, settings, coords):
    """Evaluate a spatially constant AutoPDEx coefficient function on the host."""
    if not callable(fun):
        return fun
    n = len(signature(fun).parameters)
    x0, x1 = coords[0], coords[-1]
    v0 = fun(x0) if n == 1 else fun(x0, settings)
    v1 = fun(x1) if n == 1 else fun(x1, settings)
    if not np.allclose(np.asarray(v0, dtype=np.float64), np.asarray(v1, dtype=np.float64), rtol=0, atol=0):
        raise NotImplementedError("spatially varying coefficients are not implemented in the gb300 backend")
    return v0


def _scalar(v, settings, coords):
    if isinstance(v, str):
        return float(np.asarray(settings[v]))
    return float(np.asarray(_call_xs(v, settings, coords)))


def _check_rule(ref_int_coor, ref_int_weights, dim):
    """Points per direction of a tensor Gauss-Legendre rule the kernels implement: the rules of
    seeder.gauss_legendre_nd(dim, order) for order 2-3 (2 points) and 4-5 (3 points)."""
    coor = np.asarray(ref_int_coor, dtype=np.float64)
    for order, npts in ((2, 2), (4, 3)):
        x, w = seeder.gauss_legendre_nd(dim, order)
        if (coor.reshape(x.shape) if coor.size == x.size else None) is not None and \
                np.allclose(coor.reshape(x.shape), x, rtol=0, atol=1e-15) and \
                np.allclose(ref_int_weights, w, rtol=0, atol=1e-15):
            return npts
    raise NotImplementedError("the gb300 kernels integrate with the 2- or 3-point Gauss-Legendre rule "
                              "(seeder.gauss_legendre_nd(dim, order), order 2-5)")


def _check_space(fun):
    if fun is not spaces.fem_iso_line_quad_brick and fun is not spaces.fem_iso_line_tri_tet:
        raise NotImplementedError("the gb300 backend implements spaces.fem_iso_line_quad_brick (Q1 and Q2 quads, "
                                  "Q1 bricks) and spaces.fem_iso_line_tri_tet (P1/P2 triangles, P1 tetrahedra)")


def _quadrature(space, ref_int_coor, ref_int_weights, dim):
    """(ngauss, rule): a tensor Gauss-Legendre rule for fem_iso_line_quad_brick, or any table
    of at most 16 points (as seeder.int_pts_ref_tri / int_pts_ref_tet give) for the simplices."""
    if space is spaces.fem_iso_line_tri_tet:
        pts = np.asarray(ref_int_coor, dtype=np.float64).reshape(-1, dim)
        w = np.asarray(ref_int_weights, dtype=np.float64).reshape(-1)
        if pts.shape[0] != w.shape[0] or not 1 <= pts.shape[0] <= 16:
            raise NotImplementedError("simplex rules of 1 to 16 points with one weight each are supported")
        return 2, (pts, w)
    return _check_rule(ref_int_coor, ref_int_weights, dim), None


def mixed_reference_domain_potential(integrand_fun, ansatz_fun, ref_int_coor, ref_int_weights, mapping_key):
    """Descriptor of models.mixed_reference_domain_potential (models.py:1188-1269)."""
    if not isinstance(integrand_fun, Integrand) or integrand_fun.kind not in ("poisson_sincos", "heat"):
        raise NotImplementedError("the gb300 backend needs an integrand descriptor from autopdex_gb300.models "
                                  "(poisson_sincos_integrand, heat_conduction_integrand)")
    if len(ansatz_fun) != 1 or mapping_key not in ansatz_fun:
        raise NotImplementedError("one field, mapped by its own space, is supported")
    space = next(iter(ansatz_fun.values()))
    _check_space(space)
    dim = np.asarray(ref_int_coor).shape[1]
    ng, rule = _quadrature(space, ref_int_coor, ref_int_weights, dim)
    kernel = N.AGX_MODEL_POISSON_SINCOS if integrand_fun.kind == "poisson_sincos" else N.AGX_MODEL_HEAT_POTENTIAL
    return ModelDescriptor("user potential", kernel, integrand=integrand_fun, field_key=mapping_key, dim=dim,
                           ngauss=ng, rule=rule)


def mixed_reference_domain_residual(integrand_fun, ansatz_fun, ref_int_coor, ref_int_weights, mapping_key):
    """Descriptor of models.mixed_reference_domain_residual (models.py:1272-1357)."""
    if not isinstance(integrand_fun, Integrand) or integrand_fun.kind != "heat_be":
        raise NotImplementedError("the gb300 backend needs heat_backward_euler_integrand(...) here")
    if len(ansatz_fun) != 1 or mapping_key not in ansatz_fun:
        raise NotImplementedError("one field, mapped by its own space, is supported")
    if next(iter(ansatz_fun.values())) is not spaces.fem_iso_line_quad_brick:
        raise NotImplementedError("the backward-Euler heat residual is implemented on Q1 quads and bricks")
    dim = np.asarray(ref_int_coor).shape[1]
    ng = _check_rule(ref_int_coor, ref_int_weights, dim)
    return ModelDescriptor("user residual", N.AGX_MODEL_HEAT_BE, integrand=integrand_fun, field_key=mapping_key,
                           dim=dim, ngauss=ng)


def isoparametric_domain_element_galerkin(weak_form_fun, ansatz_fun, ref_int_coor, ref_int_weights,
                                          initial_config=True):
    """Descriptor of models.isoparametric_domain_element_galerkin (models.py:1616-1718)."""
    if not isinstance(weak_form_fun, WeakForm) or weak_form_fun.kind != "neo_hooke":
        raise NotImplementedError("the gb300 backend needs hyperelastic_steady_state_weak(neo_hooke, ...) here")
    if not initial_config:
        raise NotImplementedError("only the initial configuration mapping is implemented")
    _check_space(ansatz_fun)
    dim = np.asarray(ref_int_coor).shape[1]
    ng, rule = _quadrature(ansatz_fun, ref_int_coor, ref_int_weights, dim)
    if (weak_form_fun.params["mode"] == "plain strain") != (dim == 2):
        raise NotImplementedError("'plain strain' needs 2-D elements, '3d' 3-D elements")
    return ModelDescriptor("user element", N.AGX_MODEL_NEO_HOOKE, weak=weak_form_fun, dim=dim, ngauss=ng,
                           rule=rule)


def isoparametric_surface_element_galerkin(weak_form_fun, ansatz_fun, ref_int_coor, ref_int_weights,
                                           tangent_contributions, initial_config=True):
    """Descriptor of models.isoparametric_surface_element_galerkin (models.py:1723-1851)."""
    if not isinstance(weak_form_fun, WeakForm) or weak_form_fun.kind != "neumann":
        raise NotImplementedError("the gb300 backend needs neumann_weak(...) here")
    if tangent_contributions:
        raise NotImplementedError("traction loads carry no tangent (tangent_contributions=False)")
    if not initial_config:
        raise NotImplementedError("only the initial configuration mapping is implemented")
    _check_space(ansatz_fun)
    ng = _check_rule(np.asarray(ref_int_coor).reshape(-1), ref_int_weights, 1)
    return ModelDescriptor("user element", N.AGX_MODEL_NEUMANN, weak=weak_form_fun, dim=1, ngauss=ng)
