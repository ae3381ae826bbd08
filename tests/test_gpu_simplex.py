"""Simplex elements on the GPU against the oracle (fem_iso_line_tri_tet, spaces.py:12193):
linear and quadratic triangles and tetrahedra for the Poisson potential and neo-Hooke,
float64 residuals and tangents to 1e-12 and float32 tangents to 5e-6 of the oracle's at
random DOFs (float32 rounding: 2.5e-6 measured for neo-Hooke on 6-node triangles), and a
Newton solve on linear triangles to the oracle's solution.  Meshes: the
structured quads / bricks split into 2 triangles / 6 tetrahedra, quadratic elements with a
node added on every edge."""
import numpy as np
import pytest

from autopdex_gb300 import assembler, geometry, mesher, models, seeder, solver, spaces, utility

pytestmark = pytest.mark.gpu


def _tri_mesh(n, quadratic=False):
    coords, quads = mesher.structured_mesh((n, n), [[0., 0.], [1., 0.], [1.2, 0.9], [0.1, 1.1]], "quad")
    tris = np.concatenate([quads[:, [0, 1, 2]], quads[:, [0, 2, 3]]])
    if not quadratic:
        return coords, tris
    pts = [c for c in coords]
    mid = {}

    def node(a, b):
        k = (min(a, b), max(a, b))
        if k not in mid:
            mid[k] = len(pts)
            pts.append(0.5 * (coords[a] + coords[b]))
        return mid[k]
    t6 = np.array([[a, b, c, node(a, b), node(b, c), node(c, a)] for a, b, c in tris])
    return np.array(pts), t6


def _tet_mesh(n, quadratic=False):
    coords, hexes = mesher.structured_mesh((n, n, n), [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                                                       [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], "brick")
    kuhn = [[0, 1, 2, 6], [0, 2, 3, 6], [0, 3, 7, 6], [0, 7, 4, 6], [0, 4, 5, 6], [0, 5, 1, 6]]
    tets = np.concatenate([hexes[:, k] for k in kuhn])
    if not quadratic:
        return coords, tets
    pts = [c for c in coords]
    mid = {}

    def node(a, b):
        k = (min(a, b), max(a, b))
        if k not in mid:
            mid[k] = len(pts)
            pts.append(0.5 * (coords[a] + coords[b]))
        return mid[k]
    edges = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]  # the 10-node order
    t10 = np.array([list(t) + [node(t[i], t[j]) for i, j in edges] for t in tets])
    return np.array(pts), t10


CASES = {  # name: (dim, nodes per element, rule order)
    "tri3": (2, 3, 1), "tri6": (2, 6, 2), "tet4": (3, 4, 2), "tet10": (3, 10, 2),
}


def _problem(case, kind):
    from oracle import elements as el, newton
    dim, nen, order = CASES[case]
    if dim == 2:
        coords, conn = _tri_mesh(6, quadratic=nen == 6)
        rule = seeder.int_pts_ref_tri(order)
    else:
        coords, conn = _tet_mesh(3 if nen == 4 else 2, quadratic=nen == 10)
        rule = seeder.int_pts_ref_tet(order)
    n = coords.shape[0]
    on_bnd = np.zeros(n, dtype=bool)
    on_bnd[np.argmin(coords[:, 0])] = True
    on_bnd[np.argmax(coords[:, 0])] = True
    if kind == "poisson":
        pot = models.mixed_reference_domain_potential(
            models.poisson_sincos_integrand(20.0, 10.0, (1.0, 0.5) if dim == 2 else (1.0, 0.5, 0.2)),
            {"phi": spaces.fem_iso_line_tri_tet}, *rule, "phi")
        static = {"assembling mode": ("user potential",), "solution structure": ("nodal imposition",),
                  "model": (pot,), "solver type": "newton", "solver backend": "gb300", "solver": "pcg", "verbose": -1}
        settings = {"dirichlet dofs": {"phi": on_bnd}, "connectivity": ({"phi": conn},),
                    "node coordinates": {"phi": coords}, "dirichlet conditions": {"phi": np.zeros(n)}}
        fun = el.user_potential_element(el.poisson_sincos_integrand(20.0, 10.0, (1.0, 0.5) if dim == 2 else
                                                                  (1.0, 0.5, 0.2)), dim, nen, rule=rule)
        s1 = newton.ElementSet("potential", conn, fun, lambda st: np.zeros((conn.shape[0], 1)), 1)
        prob = newton.Problem([s1], coords, n, on_bnd, np.zeros(n))
        return static, settings, prob, None
    mode = "plain strain" if dim == 2 else "3d"
    weak = models.hyperelastic_steady_state_weak(models.neo_hooke, 100.0, 0.3, mode)
    dom = models.isoparametric_domain_element_galerkin(weak, spaces.fem_iso_line_tri_tet, *rule)
    dd = utility.dof_select(on_bnd, np.ones(dim, dtype=bool))
    static = {"assembling mode": ("user element",), "solution structure": ("nodal imposition",), "model": (dom,),
              "solver type": "newton", "solver backend": "gb300", "solver": "pcg", "verbose": -1}
    settings = {"dirichlet dofs": dd, "connectivity": (conn,), "node coordinates": coords,
                "dirichlet conditions": np.zeros_like(dd, dtype=np.float64)}
    s1 = newton.ElementSet("element", conn, el.hyperelastic_element(dim, nen, 0, mode, rule=rule),
                           lambda st: np.tile([100.0, 0.3], (conn.shape[0], 1)), dim)
    prob = newton.Problem([s1], coords, n * dim, dd.reshape(-1), np.zeros(n * dim))
    return static, settings, prob, (n, dim)


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("kind", ["poisson", "neo_hooke"])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_simplex_element_parity(case, kind, dtype):
    from oracle import newton
    static, settings, prob, shape = _problem(case, kind)
    scale = 0.5 if kind == "poisson" else 0.02
    u = np.random.default_rng(3).uniform(-scale, scale, prob.n_dofs)
    dofs = u.reshape(shape) if shape else {"phi": u}
    R_or, coo = newton.assemble(prob.sets, u, prob.coords, {}, prob.n_dofs)
    K_or = newton.scipy_assembling(coo, prob.n_dofs, None)
    if dtype == "float64":
        R = assembler.assemble_residual(dofs, settings, static)
        R = np.asarray(R if shape else R["phi"], dtype=np.float64).reshape(-1)
        assert np.linalg.norm(R - R_or) <= 1e-12 * np.linalg.norm(R_or)
    K = assembler.assemble_tangent(dofs, settings, static, dtype=dtype).to_scipy()
    tol = 1e-12 if dtype == "float64" else 5e-6
    assert abs(K - K_or).max() <= tol * abs(K_or).max()


def test_newton_on_linear_triangles_matches_oracle():
    from oracle import newton
    static, settings, prob, _ = _problem("tri3", "poisson")
    sol, (it, res, div) = solver.solver({"phi": np.zeros(prob.n_dofs)}, settings, static, newton_tol=1e-10)
    assert not div
    ref, info, _ = newton.damped_newton(prob, np.zeros(prob.n_dofs), {}, 1e-10)
    u = np.asarray(sol["phi"])
    assert np.abs(u - ref).max() <= 1e-8 * max(1.0, np.abs(ref).max())
