"""The oracle's two restatements against each other: the closed-form C neo-Hooke brick
(oracle/c/orc.c) against the torch.func AD element (oracle/elements.py) at random distorted
elements and displacements, and the C Jacobi-PCG against SciPy's CG on the same system.
No GPU."""
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
