"""The oracle's two restatements against each other: the closed-form C elements
(oracle/c/orc.c: neo-Hooke bricks and plane-strain quads in both evaluation forms, the Poisson
and heat potentials, backward-Euler heat bricks, traction lines) against the torch.func AD
elements (oracle/elements.py) at random distorted elements and states, and the C Jacobi-PCG
against SciPy's CG on the same system.  No GPU."""
import numpy as np
import scipy.sparse as sps
import scipy.sparse.linalg as sla
import torch

from autopdex_gb300 import configs
from oracle import corc
from oracle import elements as el


def test_c_neo_hooke_matches_ad_oracle():
    w = configs.neo_hooke_cube(n=3, n_steps=1)
    rng = np.random.default_rng(0)
    coords = w.raw["coords"] + rng.uniform(-0.05, 0.05, w.raw["coords"].shape)
    conn = w.raw["conns"][0]
    u = rng.uniform(-0.03, 0.03, coords.shape)
    Rc, Kc = corc.neo_hooke_hex8(conn, coords, u, 1.0, 0.3)
    fun = el.hyperelastic_element(3, 8, 2, "3d")
    Ra, Ka = el.batched(fun, torch.as_tensor(u[conn]), torch.as_tensor(coords[conn]),
                        torch.tensor([[1.0, 0.3]] * conn.shape[0], dtype=torch.float64))
    Ra = Ra.numpy().reshape(Rc.shape)
    Ka = Ka.numpy().reshape(Kc.shape)
    assert np.abs(Rc - Ra).max() <= 1e-13 * np.abs(Ra).max()
    assert np.abs(Kc - Ka).max() <= 1e-13 * np.abs(Ka).max()


def test_c_pcg_matches_scipy_cg():
    rng = np.random.default_rng(1)
    n = 400
    A = sps.random(n, n, density=0.02, random_state=1, format="csr")
    A = (A + A.T + sps.diags(np.full(n, 5.0))).tocsr()
    A.sort_indices()
    b = rng.standard_normal(n)
    x, rr = corc.pcg_csr(A, b, 300)
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
    xs, info = sla.cg(A, b, rtol=1e-13, M=sps.diags(1.0 / A.diagonal()))
    assert np.abs(x - xs).max() <= 1e-9 * np.abs(xs).max()


def _ad_elements(fun, conn, *per_elem):
    out = el.batched(fun, *[torch.as_tensor(a) for a in per_elem])
    return out[0].numpy().reshape(conn.shape[0], -1), out[1].numpy().reshape(conn.shape[0], out[0][0].numel(), -1)


def _distorted(coords, seed, amp):
    return coords + np.random.default_rng(seed).uniform(-amp, amp, coords.shape)


def test_c_q1_poisson_heat_quads():
    w = configs.poisson(n=4)
    conn = w.raw["conns"][0]
    coords = _distorted(w.raw["coords"], 2, 0.03)
    u = np.random.default_rng(3).uniform(-1, 1, coords.shape[0])
    Rc, Kc = corc.q1_elements("poisson", conn, coords, u, [20.0, 10.0, 1.0, 0.5])
    Ra, Ka = _ad_elements(el.user_potential_element(el.poisson_sincos_integrand(), 2, 4), conn, u[conn], coords[conn],
                          np.zeros((conn.shape[0], 1)))
    assert np.abs(Rc - Ra).max() <= 1e-13 * np.abs(Ra).max()
    assert np.abs(Kc - Ka).max() <= 1e-13 * np.abs(Ka).max()
    k = np.exp(np.random.default_rng(4).standard_normal(conn.shape[0]))
    Rc, Kc = corc.q1_elements("heat", conn, coords, u, [1.0], elem_field=k)
    Ra, Ka = _ad_elements(el.user_potential_element(el.heat_potential_integrand(1.0), 2, 4), conn, u[conn],
                          coords[conn], k.reshape(-1, 1))
    assert np.abs(Rc - Ra).max() <= 1e-13 * np.abs(Ra).max()
    assert np.abs(Kc - Ka).max() <= 1e-13 * np.abs(Ka).max()


def test_c_q1_neo_hooke_quads_both_forms():
    w = configs.cook_membrane(n=4, n_steps=1)
    conn = w.raw["conns"][0]
    coords = _distorted(w.raw["coords"], 5, 0.3)
    u = np.random.default_rng(6).uniform(-0.05, 0.05, coords.shape)
    fun = el.hyperelastic_element(2, 4, 2, "plain strain")
    p = np.tile([240.565, 0.4999], (conn.shape[0], 1))
    Ra, Ka = _ad_elements(fun, conn, u[conn], coords[conn], p)
    for accurate in (False, True):
        Rc, Kc = corc.q1_elements("neo_hooke", conn, coords, u, [240.565, 0.4999], accurate=accurate)
        assert np.abs(Rc - Ra).max() <= 1e-12 * np.abs(Ra).max()
        assert np.abs(Kc - Ka).max() <= 1e-12 * np.abs(Ka).max()


def test_c_q1_heat_be_bricks():
    w = configs.heat_transient(n=3, n_steps=1)
    conn = w.raw["conns"][0]
    coords = _distorted(w.raw["coords"], 7, 0.02)
    rng = np.random.default_rng(8)
    T, Tn = rng.uniform(0, 1, coords.shape[0]), rng.uniform(0, 1, coords.shape[0])
    prm = [1.0, 0.5, 1.0, 1e-3]
    Rc, Kc = corc.q1_elements("heat_be", conn, coords, T, prm, node_field=Tn)
    fun = el.nonlinear_heat_be_element(3, 8, 2)
    Ra, Ka = _ad_elements(fun, conn, T[conn], Tn[conn], coords[conn], np.tile(prm, (conn.shape[0], 1)))
    assert np.abs(Rc - Ra).max() <= 1e-13 * np.abs(Ra).max()
    assert np.abs(Kc - Ka).max() <= 1e-13 * np.abs(Ka).max()


def test_c_neumann_lines_and_scatter():
    w = configs.cook_membrane(n=4, n_steps=1)
    lines = w.raw["conns"][1]
    coords = w.raw["coords"]
    Rc = corc.neumann_lines(lines, coords, (0.0, 0.3))
    fun = el.neumann_line_element(2, 2)
    Ra = np.stack([fun(coords[c], np.array([0.0, 0.3])) for c in lines])
    assert np.abs(Rc - Ra).max() <= 1e-14 * np.abs(Ra).max()
    R = corc.scatter(lines, 2, Rc, coords.shape[0] * 2)
    ref = np.zeros(coords.shape[0] * 2)
    ed = (lines[:, :, None] * 2 + np.arange(2)).reshape(lines.shape[0], -1)
    np.add.at(ref, ed.ravel(), Rc.ravel())
    assert np.abs(R - ref).max() <= 1e-15


def test_c_pcg_stops_at_tolerance():
    rng = np.random.default_rng(2)
    n = 300
    A = sps.random(n, n, density=0.03, random_state=2, format="csr")
    A = (A + A.T + sps.diags(np.full(n, 6.0))).tocsr()
    b = rng.standard_normal(n)
    x, rr, its = corc.pcg_csr_tol(A, b, 1e-10, 1000)
    assert 0 < its < 1000 and np.sqrt(rr) <= 1e-10 * np.linalg.norm(b)
    assert np.linalg.norm(A @ x - b) <= 2e-10 * np.linalg.norm(b)
