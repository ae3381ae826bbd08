"""Float64 flexible CG with a float32 preconditioner (AGX_FCG_F64) and the vector-field grid
transfers of the learned preconditioner, on the nearly incompressible Cook membrane.

Tolerances, written where they are used:
* FCG solutions: ||u_fcg - u_direct||_inf <= 1e-6 ||u_direct||_inf after a Newton solve to 1e-7
  (the float64 floor of this problem is near 1e-8 at these sizes)
* transfers: <P y, x> = <y, P^T x> within 1e-5 relative (float32 arithmetic); image round trip
  within bf16 rounding (1e-2 relative)
"""
import ctypes as C

import numpy as np
import pytest
import torch

from autopdex_gb300 import configs, solver

pytestmark = pytest.mark.gpu


def _flat(d):
    a = next(iter(d.values())) if isinstance(d, dict) else d
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.asarray(a, dtype=np.float64).reshape(-1)


def test_fcg_f64_jacobi_matches_direct_newton():
    """FCG in float64 with Jacobi (no callback) through solver.solver ('fcg', 'float64')
    against the direct-solve Newton solution of the same load step."""
    w = configs.cook_membrane(n=16, n_steps=2, solver="lapack")
    st = w.steps[0](dict(w.settings))
    ref, (it, res, div) = solver.solver(w.dofs, st, w.static_settings, newton_tol=0.0, newton_rtol=1e-7, maxiter=12)
    assert not div
    static = dict(w.static_settings, solver="fcg", precision="float64")
    solver.set_learned_preconditioner(None, None)
    sol, (it2, res2, div2) = solver.solver(w.dofs, st, static, newton_tol=0.0, newton_rtol=1e-7, maxiter=12,
                                           krylov_tol=1e-6, krylov_maxiter=200000)
    assert not div2
    r = _flat(ref)
    assert np.abs(_flat(sol) - r).max() <= 1e-6 * np.abs(r).max()


def test_field_transfers_adjoint_and_round_trip():
    from autopdex_gb300 import _native as N
    from autopdex_gb300 import learned
    lib = N.load()
    dev = torch.device("cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    Hc, Wc, f, nd = 9, 7, 4, 2
    Hf, Wf = (Hc - 1) * f + 1, (Wc - 1) * f + 1
    g = torch.Generator(device="cuda").manual_seed(0)
    y = torch.randn(Hc * Wc * nd, device=dev, generator=g)
    x = torch.randn(Hf * Wf * nd, device=dev, generator=g)
    Py = torch.empty(Hf * Wf * nd, device=dev)
    Ptx = torch.empty(Hc * Wc * nd, device=dev)
    assert lib.agx_nn_prolong_field(C.c_void_p(y.data_ptr()), nd, Hc, Wc, f, C.c_void_p(Py.data_ptr()), st) == 0
    assert lib.agx_nn_restrict_field(C.c_void_p(x.data_ptr()), None, nd, Hc, Wc, f, C.c_void_p(Ptx.data_ptr()),
                                     st) == 0
    torch.cuda.synchronize()
    a, b = float((Py.double() * x.double()).sum()), float((y.double() * Ptx.double()).sum())
    assert abs(a - b) <= 1e-5 * (abs(a) + abs(b))
    # coarse node (I, J) is fine node (f I, f J): the prolongation keeps its values
    Pyr = Py.reshape(Hf, Wf, nd)
    assert torch.allclose(Pyr[::f, ::f].reshape(-1), y, rtol=1e-6, atol=1e-6)
    # the network image and back: channels 0..nd-1 the field, nd..nd+1 the features
    Hn, Wn = 9, 7
    r = torch.randn(Hn * Wn * nd, device=dev, generator=g)
    aux = torch.randn(Hn * Wn * 2, device=dev, generator=g)
    img, sc = learned.to_image(lib, r, aux, Hn, Wn, normalize=False, nd=nd, naux=2)
    z = torch.empty_like(r)
    assert lib.agx_nn_field_from_grid(C.c_void_p(img.data_ptr()), learned.C_IN, nd, Hn, Wn, img.shape[2],
                                      C.c_void_p(z.data_ptr()), st) == 0
    torch.cuda.synchronize()
    assert torch.allclose(z, r, rtol=1e-2, atol=1e-2)
    assert torch.allclose(img[0, :Hn, :Wn, nd:nd + 2].float().reshape(-1), aux, rtol=1e-2, atol=1e-2)
    assert float(img[0, Hn:, :, :].float().abs().max()) == 0.0
