"""Host-side logic of the backend (no GPU): set-up helpers against the oracle's
restatements, descriptor validation, DOF layout, and the load-stepping controller."""
import numpy as np
import pytest

from autopdex_gb300 import configs, geometry, mesher, models, seeder, spaces, utility
from autopdex_gb300 import _problem
from oracle import mesh as omesh


@pytest.mark.parametrize("dim,n", [(2, (3, 4)), (3, (2, 3, 2))])
def test_mesher_matches_oracle(dim, n):
    if dim == 2:
        v = [[0., 0.], [48., 44.], [48., 60.], [0., 44.]]
        a = mesher.structured_mesh(n, v, "quad")
        b = omesh.structured_mesh(n, v, "quad")
    else:
        v = [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]]
        a = mesher.structured_mesh(n, v, "brick")
        b = omesh.structured_mesh(n, v, "brick")
    assert np.array_equal(a[1], b[1])
    assert np.allclose(a[0], b[0], rtol=0, atol=1e-14)


@pytest.mark.parametrize("dim,order", [(1, 2), (2, 2), (3, 2), (2, 4)])
def test_quadrature_matches_oracle(dim, order):
    a = seeder.gauss_legendre_nd(dim, order)
    b = omesh.gauss_legendre_nd(dim, order)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_boundary_selection_matches_oracle():
    pts = [[0., 0.], [1., 0.], [1., 1.], [0., 1.]]
    coords, _ = mesher.structured_mesh((7, 7), pts, "quad")
    a = geometry.in_sdfs(coords, lambda x: geometry.psdf_polygon(x, pts))
    b = omesh.in_sdfs(coords, pts)
    assert np.array_equal(a, b) and a.sum() == 4 * 7 - 4


def test_q1_shape_functions_partition_of_unity():
    for d in (1, 2, 3):
        xi = np.linspace(-0.7, 0.6, d)
        N = spaces.q1_shape_functions(xi, d)
        assert abs(N.sum() - 1) < 1e-15
        assert np.allclose(N, omesh.shape_functions(xi if d > 1 else xi[0], d, 2 ** d))


def test_dict_utilities():
    d = {"a": np.arange(6.).reshape(3, 2)}
    f = utility.dict_flatten(d)
    assert np.array_equal(utility.reshape_as(f, d)["a"], d["a"])
    with pytest.raises(ValueError):
        utility.reshape_as(np.zeros(5), d)


def test_dof_layout():
    assert _problem.dof_layout({"phi": np.zeros(9)}) == ("phi", 9, 1)
    assert _problem.dof_layout(np.zeros((9, 3))) == (None, 9, 3)
    with pytest.raises(NotImplementedError):
        _problem.dof_layout({"u": np.zeros(3), "p": np.zeros(3)})


def test_descriptors_reject_unknown_models():
    x, w = seeder.gauss_legendre_nd(2, 2)
    with pytest.raises(NotImplementedError):
        models.mixed_reference_domain_potential(lambda *a: 0.0, {"phi": spaces.fem_iso_line_quad_brick}, x, w, "phi")
    with pytest.raises(NotImplementedError):  # a rule that is not a 2- or 3-point Gauss-Legendre rule
        models.mixed_reference_domain_potential(models.poisson_sincos_integrand(), {"phi": spaces.fem_iso_line_quad_brick},
                                                0.5 * x, w, "phi")
    # the 3-point rule (order 4) is accepted and recorded
    d = models.mixed_reference_domain_potential(models.poisson_sincos_integrand(), {"phi": spaces.fem_iso_line_quad_brick},
                                                *seeder.gauss_legendre_nd(2, 4), "phi")
    assert d.ngauss == 3
    with pytest.raises(NotImplementedError):
        models.hyperelastic_steady_state_weak(lambda F, p: 0.0, 1.0, 0.3, "3d")


def test_descriptor_resolves_settings_parameters():
    w = configs.cook_membrane(n=4, n_steps=2)
    dom, surf = w.static_settings["model"]
    st = dict(w.settings)
    st["load multiplier"] = 0.25
    m, p, ef, nf = surf.resolve(st, w.raw["coords"], w.raw["conns"][1])
    assert p == [0.0, 0.25] and ef is None
    m, p, ef, nf = dom.resolve(st, w.raw["coords"], w.raw["conns"][0])
    assert p == [240.565, 0.4999]


def test_spatially_varying_coefficient_rejected():
    weak = models.hyperelastic_steady_state_weak(models.neo_hooke, lambda x: 1.0 + x[0], 0.3, "plain strain")
    d = models.isoparametric_domain_element_galerkin(weak, spaces.fem_iso_line_quad_brick, *seeder.gauss_legendre_nd(2, 2))
    coords = np.array([[0., 0.], [1., 0.]])
    with pytest.raises(NotImplementedError):
        d.resolve({}, coords, np.zeros((1, 4), dtype=np.int64))


def test_grf_statistics():
    g = configs.gaussian_random_field(128, seed=3)
    assert g.shape == (128, 128)
    assert abs(g.mean()) < 1e-12 and abs(g.std() - 1) < 1e-12
    # correlated at short range, decorrelated at long range (length 0.05 = 6.4 cells)
    c1 = np.mean(g[:-1] * g[1:])
    c30 = np.mean(g[:-30] * g[30:])
    assert c1 > 0.9 and abs(c30) < 0.2


def test_adaptive_load_stepping_controller(monkeypatch):
    """Increment control of solver.py:355-378 with a fake Newton solve: divergence halves
    the increment and rolls the DOFs back; the multiplier ends at max_multiplier."""
    from autopdex_gb300 import solver as S
    calls = []

    def fake(dofs, settings, static_settings, newton_tol=None, **kw):
        calls.append(settings["load multiplier"])
        div = len(calls) == 2
        return dofs + 1, (3, 1e-12, div)
    monkeypatch.setattr(S, "solver", fake)
    out = S.adaptive_load_stepping(np.zeros(2), {}, {"verbose": -1})
    dofs, mult, inc = out[0], out[1], out[2]
    assert abs(mult - 1.0) < 1e-12
    assert np.isclose(calls[0], 0.2) and np.isclose(calls[1], 0.2 + 0.2 * (1 + 0.5 * 4 / 7))
    # the diverged step did not advance the DOFs
    assert dofs[0] == len(calls) - 1


def test_dlpack_host_arrays_are_read():
    """Arrays of other frameworks arrive through DLPack (host ones are read as NumPy)."""
    import torch

    class Foreign:
        def __init__(self, t):
            self._t, self.shape = t, tuple(t.shape)

        def __dlpack__(self, stream=None, **kw):
            return self._t.__dlpack__()

        def __dlpack_device__(self):
            return self._t.__dlpack_device__()

    f = Foreign(torch.arange(6.0).reshape(3, 2))
    assert _problem.is_foreign(f) and not _problem.is_foreign(np.zeros(2))
    assert np.array_equal(_problem.flatten({"u": f}, "u"), np.arange(6.0))
    assert _problem.dof_layout(f) == (None, 3, 2)


def test_q2_host_shape_functions_match_oracle():
    """The host Q2 interpolation of spaces.fem_iso_line_quad_brick against the oracle's."""
    from autopdex_gb300 import spaces
    from oracle import mesh as om
    rng = np.random.default_rng(2)
    for dim, nen in ((2, 9), (3, 27)):
        xi = rng.uniform(-1, 1, dim)
        assert np.allclose(spaces.q2_shape_functions(xi, dim), om.shape_functions(xi, dim, nen), rtol=0, atol=1e-15)
        f = rng.standard_normal(nen)
        v = spaces.fem_iso_line_quad_brick(xi, np.zeros((nen, dim)), f, {}, False, dim)
        assert np.isclose(v, om.shape_functions(xi, dim, nen) @ f)


def test_no_cpu_fallback():
    """Without a CUDA device the backend refuses to solve instead of falling back to the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from autopdex_gb300 import solver
    w = configs.poisson(n=4)
    with pytest.raises(RuntimeError, match="CUDA"):
        solver.solver(w.dofs, w.settings, w.static_settings)
    for fn in (lambda: solver.sensitivities(w.dofs, w.settings, w.static_settings, []),
               lambda: solver.second_order_sensitivities(w.dofs, w.settings, w.static_settings, []),
               lambda: solver.adjoint_sensitivities(w.dofs, w.settings, w.static_settings, [], w.dofs)):
        with pytest.raises(RuntimeError, match="CUDA"):
            fn()


def test_implicit_diff_stencils():
    """The central differences of the implicit-differentiation algebra: the two-point stencil
    is exact for quadratics, the four-point one for quartics."""
    from autopdex_gb300 import implicit_diff
    f2 = lambda e: 3.0 + 2.0 * e + 5.0 * e * e
    f4 = lambda e: 1.0 - e + 0.5 * e ** 2 + 7.0 * e ** 3 - 2.0 * e ** 4
    assert abs(implicit_diff._central(f2, 0.1, 2) - 2.0) < 1e-13
    assert abs(implicit_diff._central(f4, 0.1, 4) + 1.0) < 1e-12
    assert abs(implicit_diff._central(f4, 0.1, 2) + 1.0) > 1e-3


def test_network_tables_are_consistent():
    """Host-side tables of the learned preconditioners: the 3-D network shares the 2-D graph's
    layer names (the forward and backward passes walk both by name), its concatenating layers are
    the decoder's first ones, and the 3-D grid padding rounds up to a multiple of 8 (three
    2 x 2 x 2 poolings)."""
    from autopdex_gb300 import learned
    names = [n for n, *_ in learned.LAYERS]
    assert [n for n, *_ in learned.LAYERS3] == names
    assert all(c2 == (16 if n in ("d2a", "d1a", "d0a") else 0) for n, c1, c2, co, relu in learned.LAYERS3)
    assert [learned.padded3(n) for n in (1, 8, 9, 17, 33, 40)] == [8, 8, 16, 24, 40, 40]
    assert learned.UNet3D.dims == 3 and learned.UNet3D.pool == 2
