"""The row-by-row tangent of structured quad grids against the element-scatter tangent.

A mesh in the mesher's numbering is assembled by the atomic-free row kernel; the same mesh
with its elements listed in a shuffled order is not recognised as a grid and goes through
the element kernel with its atomic scatter.  Both must give the same matrix: float64 to
1e-13 of the largest entry (summation order differs), float32 to 5e-6 (both are float32
element integrals with different rounding sequences, each within 2e-6 of float64); with and without
Dirichlet elimination, for the Poisson and heat (random conductivity) potentials, on grids
whose extents are not multiples of the 31-node strip of the row kernel (101 nodes per row: two
strips with both column neighbours inside the grid); the unit-square grids take the
parallelogram branch of the row kernel, the grid on Cook's quadrilateral the general one.
"""
import ctypes as C

import numpy as np
import pytest

from autopdex_gb300 import assembler, configs

pytestmark = pytest.mark.gpu


def _shuffled(w, seed=3):
    rng = np.random.default_rng(seed)
    conn_obj = w.settings["connectivity"][0]
    key = next(iter(conn_obj)) if isinstance(conn_obj, dict) else None
    conn = np.asarray(conn_obj[key] if key else conn_obj)
    perm = rng.permutation(conn.shape[0])
    settings = dict(w.settings)
    settings["connectivity"] = ({key: conn[perm]} if key else conn[perm],)
    if "conductivity" in settings:
        settings["conductivity"] = np.asarray(settings["conductivity"])[perm]
    return settings, w.static_settings  # a new connectivity array: a new native context


def _heat_on_trapezoid(n=33):
    """Heat with random conductivity on Cook's quadrilateral: a structured grid whose
    elements are not parallelograms (the row kernel's general, non-affine integral)."""
    from autopdex_gb300 import mesher
    w = configs.heat_grf(n=n, seed=5)
    coords, _ = mesher.structured_mesh((n, n), [[0., 0.], [48., 44.], [48., 60.], [0., 44.]], "quad")
    settings = dict(w.settings)
    settings["node coordinates"] = {"T": coords}
    w.settings = settings
    return w


@pytest.mark.parametrize("case", ["poisson", "heat", "heat_trapezoid", "heat_wide"])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("eliminate", [False, True])
def test_grid_rows_match_element_scatter(case, dtype, eliminate):
    w = {"poisson": lambda: configs.poisson(n=45), "heat": lambda: configs.heat_grf(n=37, seed=11),
         "heat_trapezoid": _heat_on_trapezoid, "heat_wide": lambda: configs.heat_grf(n=100, seed=12)}[case]()
    ref = assembler.assemble_tangent(w.dofs, w.settings, w.static_settings, dtype=dtype,
                                     eliminate_dirichlet=eliminate).to_scipy()
    settings, static = _shuffled(w)
    other = assembler.assemble_tangent(w.dofs, settings, static, dtype=dtype,
                                       eliminate_dirichlet=eliminate).to_scipy()
    tol = 1e-13 if dtype == "float64" else 5e-6
    scale = abs(ref).max()
    assert abs(ref - other).max() <= tol * scale
    assert ref.nnz == other.nnz


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_grid_inverse_diagonal(dtype):
    """The row kernel's fused Jacobi diagonal: z = D^-1 r with r = 1 equals 1 / diag(K) of the
    assembled, Dirichlet-eliminated matrix (identity rows: 1) to rounding."""
    import torch
    from autopdex_gb300 import _native as N
    from autopdex_gb300._problem import get_problem
    w = configs.heat_grf(n=100, seed=12)
    K = assembler.assemble_tangent(w.dofs, w.settings, w.static_settings, dtype=dtype,
                                   eliminate_dirichlet=True).to_scipy()
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    x = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
    dt = N.AGX_F64 if dtype == "float64" else N.AGX_F32
    prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, dt)
    tdt = torch.float64 if dtype == "float64" else torch.float32
    r = torch.ones(prob.n_dofs, dtype=tdt, device=prob.device)
    z = torch.empty_like(r)
    prob._call("agx_jacobi", dt, C.c_void_p(r.data_ptr()), C.c_void_p(z.data_ptr()))
    expect = 1.0 / K.diagonal()
    tol = 1e-15 if dtype == "float64" else 1e-6
    assert np.abs(z.cpu().numpy() - expect).max() <= tol * np.abs(expect).max()
