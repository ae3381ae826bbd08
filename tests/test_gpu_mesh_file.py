"""A mesh that arrives as a file: the 40 x 40 Poisson problem written to a Gmsh file with its
elements in shuffled order (so not recognised as a structured grid: the element-scatter
path), read back with mesh_io and solved through solver.solver.  The solution equals the
one of the structured mesh in memory to the Newton tolerance of the parity tests."""
import numpy as np
import pytest

from autopdex_gb300 import configs, mesh_io, solver

pytestmark = pytest.mark.gpu


def test_poisson_from_gmsh_file(tmp_path):
    w = configs.poisson(n=40)
    ref, info = solver.solver(w.dofs, w.settings, w.static_settings, newton_tol=1e-10, newton_rtol=1e-12)
    assert not info[2]
    coords = w.raw["coords"]
    elems = w.raw["conns"][0][np.random.default_rng(5).permutation(w.raw["conns"][0].shape[0])]
    path = str(tmp_path / "poisson.msh")
    mesh_io.write_gmsh(path, coords, {"quad": elems})
    m = mesh_io.read(path)
    settings = dict(w.settings)
    settings["node coordinates"] = {"phi": m.points[:, :2]}
    settings["connectivity"] = ({"phi": m.cells_dict["quad"]},)
    sol, info = solver.solver(w.dofs, settings, w.static_settings, newton_tol=1e-10, newton_rtol=1e-12)
    assert not info[2]
    u, u_ref = np.asarray(sol["phi"]), np.asarray(ref["phi"])
    assert np.abs(u - u_ref).max() <= 1e-8 * max(1.0, np.abs(u_ref).max())
