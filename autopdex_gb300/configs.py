"""Synthetic workloads of the benchmark configurations, as AutoPDEx inputs.

Each builder returns a :class:`Workload` holding the ``dofs`` / ``settings`` /
``static_settings`` triple for ``autopdex_gb300.solver.solver`` plus the raw arrays
(coordinates, connectivities, Dirichlet masks, parameters) from which an independent CPU
oracle can set up the same problem.  Sizes are parameters so that the same builders make
the full-size benchmark inputs and the small parity cases.

1. 2-D Poisson on [0,1]^2, Q1 quads, source 20 (sin(10 x.x) - cos(10 |x-(1,.5)|^2)),
   boundary selected as in AutoPDEx's example (geometry.in_sdfs with psdf_polygon).
2. 3-D compressible neo-Hooke cube [0,1]^3, Q1 bricks, E = 1, nu = 0.3; x = 0 clamped,
   u_x = 0.3 k / n_steps prescribed on x = 1 (u_y, u_z free there).
3. Plane-strain neo-Hooke Cook membrane (0,0),(48,44),(48,60),(0,44), E = 240.565,
   nu = 0.4999, left edge clamped, shear traction (0, 1/16 k / n_steps) on x = 48.
4. Heat conduction -div(k grad T) = 1 on [0,1]^2, k = exp(g) per element, g a Gaussian
   random field (squared-exponential covariance, length 0.05, std 1) sampled by FFT
   spectral synthesis on a padded periodic grid, T = 0 on the boundary.
5. Backward-Euler nonlinear heat on [0,1]^3, k(T) = 1 + 0.5 T^2, rho c = 1, dt = 1e-3,
   T_0 ~ U[0,1] (seeded), T = 0 on all faces.
"""
import numpy as np

from . import geometry, mesher, models, seeder, spaces


class Workload:
    def __init__(self, name, dofs, settings, static_settings, raw, steps=None):
        self.name = name
        self.dofs = dofs
        self.settings = settings
        self.static_settings = static_settings
        self.raw = raw
        self.steps = steps  # list of callables settings -> settings, one per load/time step

    @property
    def n_dofs(self):
        d = self.dofs
        a = next(iter(d.values())) if isinstance(d, dict) else d
        return int(np.size(a))


def poisson(n=200, solver="pcg", precision="float64"):
    pts = [[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]]
    coords, elems = mesher.structured_mesh((n, n), pts, "quad")
    dn = geometry.in_sdfs(coords, lambda x: geometry.psdf_polygon(x, pts))
    integrand = models.poisson_sincos_integrand(20.0, 10.0, (1.0, 0.5))
    model = models.mixed_reference_domain_potential(integrand, {"phi": spaces.fem_iso_line_quad_brick},
                                                    *seeder.gauss_legendre_nd(2, 2), "phi")
    static = {"assembling mode": ("user potential",), "solution structure": ("nodal imposition",),
              "model": (model,), "solver type": "newton", "solver backend": "gb300", "solver": solver,
              "precision": precision, "verbose": -1}
    settings = {"connectivity": ({"phi": elems},), "dirichlet dofs": {"phi": dn},
                "node coordinates": {"phi": coords}, "dirichlet conditions": {"phi": np.zeros(coords.shape[0])}}
    raw = dict(coords=coords, conns=[elems], dirichlet=dn.astype(bool), values=np.zeros(coords.shape[0]),
               kind="poisson")
    return Workload(f"poisson_{n}x{n}_q1", {"phi": np.zeros(coords.shape[0])}, settings, static, raw)


def gaussian_random_field(n, length=0.05, std=1.0, seed=0, pad=2):
    """Element-centred GRF g on an n x n grid over [0,1]^2: white noise filtered by the
    square root of the squared-exponential spectrum on a periodic grid padded by ``pad``,
    then cropped.  Returns (n, n) with row index i along x."""
    rng = np.random.default_rng(seed)
    m = n * pad
    h = 1.0 / n
    k = np.fft.fftfreq(m, d=h) * 2 * np.pi
    KX, KY = np.meshgrid(k, k, indexing="ij")
    # spectral density of exp(-r^2 / (2 l^2)) in 2-D: 2 pi l^2 exp(-l^2 |k|^2 / 2)
    S = 2 * np.pi * length ** 2 * np.exp(-0.5 * length ** 2 * (KX ** 2 + KY ** 2))
    w = rng.standard_normal((m, m))
    f = np.fft.ifft2(np.fft.fft2(w) * np.sqrt(S / (h * h))).real
    f = f[:n, :n]
    f = (f - f.mean()) / (f.std() + 1e-30) * std
    return f


def heat_grf(n=1024, seed=0, solver="pcg", precision="float64"):
    pts = [[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]]
    coords, elems = mesher.structured_mesh((n, n), pts, "quad")
    on_bnd = (np.abs(coords[:, 0]) < 1e-12) | (np.abs(coords[:, 0] - 1) < 1e-12) | \
             (np.abs(coords[:, 1]) < 1e-12) | (np.abs(coords[:, 1] - 1) < 1e-12)
    g = gaussian_random_field(n, seed=seed)
    k = np.exp(g).reshape(-1)  # element (i, j) -> i * n + j, the mesher's element order
    integrand = models.heat_conduction_integrand("conductivity", 1.0)
    model = models.mixed_reference_domain_potential(integrand, {"T": spaces.fem_iso_line_quad_brick},
                                                    *seeder.gauss_legendre_nd(2, 2), "T")
    static = {"assembling mode": ("user potential",), "solution structure": ("nodal imposition",),
              "model": (model,), "solver type": "newton", "solver backend": "gb300", "solver": solver,
              "precision": precision, "verbose": -1}
    settings = {"connectivity": ({"T": elems},), "dirichlet dofs": {"T": on_bnd},
                "node coordinates": {"T": coords}, "dirichlet conditions": {"T": np.zeros(coords.shape[0])},
                "conductivity": k}
    raw = dict(coords=coords, conns=[elems], dirichlet=on_bnd, values=np.zeros(coords.shape[0]), k=k,
               kind="heat", n=n)
    return Workload(f"heat_grf_{n}x{n}_q1", {"T": np.zeros(coords.shape[0])}, settings, static, raw)


def neo_hooke_cube(n=64, n_steps=10, solver="pcg", precision="float64", E=1.0, nu=0.3, stretch=0.3):
    verts = [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]]
    coords, elems = mesher.structured_mesh((n, n, n), verts, "brick")
    x0 = np.abs(coords[:, 0]) < 1e-12
    x1 = np.abs(coords[:, 0] - 1) < 1e-12
    mask = np.zeros((coords.shape[0], 3), dtype=bool)
    mask[x0, :] = True
    mask[x1, 0] = True
    weak = models.hyperelastic_steady_state_weak(models.neo_hooke, E, nu, "3d")
    model = models.isoparametric_domain_element_galerkin(weak, spaces.fem_iso_line_quad_brick,
                                                         *seeder.gauss_legendre_nd(3, 2))
    static = {"assembling mode": ("user element",), "solution structure": ("nodal imposition",),
              "model": (model,), "solver type": "newton", "solver backend": "gb300", "solver": solver,
              "precision": precision, "verbose": -1}
    values = np.zeros((coords.shape[0], 3))
    settings = {"connectivity": (elems,), "dirichlet dofs": mask, "node coordinates": coords,
                "dirichlet conditions": values}

    def step(k):
        def f(st):
            v = np.zeros((coords.shape[0], 3))
            v[x1, 0] = stretch * k / n_steps
            st["dirichlet conditions"] = v
            return st
        return f
    raw = dict(coords=coords, conns=[elems], dirichlet=mask.reshape(-1), values=values.reshape(-1), E=E, nu=nu,
               kind="neo_hooke_3d", x1=x1, stretch=stretch, n_steps=n_steps)
    return Workload(f"neo_hooke_cube_{n}^3_hex8", np.zeros((coords.shape[0], 3)), settings, static, raw,
                    steps=[step(k) for k in range(1, n_steps + 1)])


def cook_membrane(n=512, n_steps=20, solver="pcg", precision="float64", E=240.565, nu=0.4999, q=1.0 / 16):
    pts = [[0.0, 0.0], [48.0, 44.0], [48.0, 60.0], [0.0, 44.0]]
    coords, elems = mesher.structured_mesh((n, n), pts, "quad")
    lines = mesher.structured_boundary_lines((n, n), "right")
    left = geometry.in_planes(coords, pts[0], [1.0, 0.0])
    mask = np.zeros((coords.shape[0], 2), dtype=bool)
    mask[left, :] = True
    weak = models.hyperelastic_steady_state_weak(models.neo_hooke, E, nu, "plain strain")
    dom = models.isoparametric_domain_element_galerkin(weak, spaces.fem_iso_line_quad_brick,
                                                       *seeder.gauss_legendre_nd(2, 2))
    trac = models.neumann_weak(lambda x, settings: np.array([0.0, settings["load multiplier"]]))
    surf = models.isoparametric_surface_element_galerkin(trac, spaces.fem_iso_line_quad_brick,
                                                         *seeder.gauss_legendre_nd(1, 2),
                                                         tangent_contributions=False)
    static = {"assembling mode": ("user element", "user element"),
              "solution structure": ("nodal imposition", "nodal imposition"), "model": (dom, surf),
              "solver type": "newton", "solver backend": "gb300", "solver": solver, "precision": precision,
              "verbose": -1}
    settings = {"connectivity": (elems, lines), "dirichlet dofs": mask, "node coordinates": coords,
                "dirichlet conditions": np.zeros((coords.shape[0], 2)), "load multiplier": 0.0}

    def step(k):
        def f(st):
            st["load multiplier"] = q * k / n_steps
            return st
        return f
    raw = dict(coords=coords, conns=[elems, lines], dirichlet=mask.reshape(-1), values=np.zeros(2 * coords.shape[0]),
               E=E, nu=nu, q=q, kind="cook", n_steps=n_steps)
    return Workload(f"cook_membrane_{n}x{n}_q1", np.zeros((coords.shape[0], 2)), settings, static, raw,
                    steps=[step(k) for k in range(1, n_steps + 1)])


def heat_transient(n=128, n_steps=100, dt=1e-3, seed=0, solver="bicgstab", precision="float64"):
    verts = [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]]
    coords, elems = mesher.structured_mesh((n, n, n), verts, "brick")
    bnd = np.zeros(coords.shape[0], dtype=bool)
    for d in range(3):
        bnd |= (np.abs(coords[:, d]) < 1e-12) | (np.abs(coords[:, d] - 1) < 1e-12)
    rng = np.random.default_rng(seed)
    T0 = rng.uniform(0.0, 1.0, coords.shape[0])
    T0[bnd] = 0.0
    integrand = models.heat_backward_euler_integrand(1.0, 0.5, 1.0, "time increment", "dofs n")
    model = models.mixed_reference_domain_residual(integrand, {"T": spaces.fem_iso_line_quad_brick},
                                                   *seeder.gauss_legendre_nd(3, 2), "T")
    static = {"assembling mode": ("user residual",), "solution structure": ("nodal imposition",),
              "model": (model,), "solver type": "newton", "solver backend": "gb300", "solver": solver,
              "precision": precision, "verbose": -1}
    settings = {"connectivity": ({"T": elems},), "dirichlet dofs": {"T": bnd}, "node coordinates": {"T": coords},
                "dirichlet conditions": {"T": np.zeros(coords.shape[0])}, "dofs n": {"T": T0.copy()},
                "time increment": dt}
    raw = dict(coords=coords, conns=[elems], dirichlet=bnd, values=np.zeros(coords.shape[0]), T0=T0, dt=dt,
               kind="heat_be", n_steps=n_steps)
    return Workload(f"heat_be_{n}^3_hex8", {"T": T0.copy()}, settings, static, raw)
