"""The row-by-row tangent of structured quad grids against the element-scatter tangent.

A mesh in the mesher's numbering is assembled by the atomic-free row kernel; the same mesh
with its elements listed in a shuffled order is not recognised as a grid and goes through
the element kernel with its atomic scatter.  Both must give the same matrix: float64 to
1e-13 of the largest entry (summation order differs), float32 to 5e-6 (both are float32
element integrals with different rounding sequences, each within 2e-6 of float64); with and without
Dirichlet elimination, for the Poisson and heat (random conductivity) potentials, on grids
whose extents are not multiples of the 32 x 8 node tile; the unit-square grids take the
parallelogram branch of the row kernel, the grid on Cook's quadrilateral the general one.
"""
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


@pytest.mark.parametrize("case", ["poisson", "heat", "heat_trapezoid"])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("eliminate", [False, True])
def test_grid_rows_match_element_scatter(case, dtype, eliminate):
    w = {"poisson": lambda: configs.poisson(n=45), "heat": lambda: configs.heat_grf(n=37, seed=11),
         "heat_trapezoid": _heat_on_trapezoid}[case]()
    ref = assembler.assemble_tangent(w.dofs, w.settings, w.static_settings, dtype=dtype,
                                     eliminate_dirichlet=eliminate).to_scipy()
    settings, static = _shuffled(w)
    other = assembler.assemble_tangent(w.dofs, settings, static, dtype=dtype,
                                       eliminate_dirichlet=eliminate).to_scipy()
    tol = 1e-13 if dtype == "float64" else 5e-6
    scale = abs(ref).max()
    assert abs(ref - other).max() <= tol * scale
    assert ref.nnz == other.nnz
