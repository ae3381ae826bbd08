"""The allocation-free entry point agx_pcg_noalloc against the context-based agx_solve.

agx_pcg_noalloc serves callers that cannot allocate device memory during a solve (fixed
memory pools, hosts that forbid cudaMalloc after start-up, callers without a context): its
work vectors live in a fixed file-scope device array.  Here it solves the same float64
systems as agx_solve (assembled through a context, copied out with agx_copy_matrix) and must
agree with it within the solution tolerance of the parity tests, on two calls in a row
(the shared array keeps the first call's contents, which the second call must not see).
This file is collected last so that a run stopping at the first failure has run every
other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from autopdex_gb300 import _native as N
from autopdex_gb300 import configs

pytestmark = pytest.mark.gpu


def _system(w):
    import torch
    from autopdex_gb300._problem import get_problem
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    rng = np.random.default_rng(11)
    u = torch.as_tensor(rng.uniform(-0.01, 0.01, w.n_dofs), device=prob.device)
    prob._call("agx_assemble", C.c_void_p(u.data_ptr()), None, N.AGX_F64)
    rp = torch.empty(prob.n_nodes + 1, dtype=torch.int32, device=prob.device)
    col = torch.empty(prob.nnzb, dtype=torch.int32, device=prob.device)
    vals = torch.empty(prob.nnzb * prob.ndof * prob.ndof, dtype=torch.float64, device=prob.device)
    prob._call("agx_copy_matrix", N.AGX_F64, C.c_void_p(rp.data_ptr()), C.c_void_p(col.data_ptr()),
               C.c_void_p(vals.data_ptr()))
    rhs = torch.as_tensor(rng.standard_normal(w.n_dofs), device=prob.device)
    rhs[torch.as_tensor(prob.mask.astype(bool), device=prob.device)] = 0.0
    return prob, rp, col, vals, rhs


@pytest.mark.parametrize("case", ["poisson", "neo_hooke_3d"])
def test_noalloc_pcg_matches_context_solve(case):
    import torch
    w = configs.poisson(n=24) if case == "poisson" else configs.neo_hooke_cube(n=4, n_steps=1)
    prob, rp, col, vals, rhs = _system(w)
    lib = N.load()
    # existing entry point
    x_ref = torch.zeros_like(rhs)
    o = N.SolveOpts()
    o.method, o.rtol, o.atol, o.maxiter, o.check_every = N.AGX_PCG, 1e-12, 0.0, 20000, 16
    info = N.SolveInfo()
    assert lib.agx_solve(prob.ctx, C.c_void_p(rhs.data_ptr()), C.c_void_p(x_ref.data_ptr()), C.byref(o),
                         C.byref(info)) == N.AGX_OK
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    sols = []
    for call in range(2):
        x = torch.full_like(rhs, np.nan)  # every entry must be written by the solve
        na_info = N.SolveInfo()
        err = C.create_string_buffer(256)
        rc = lib.agx_pcg_noalloc(C.c_void_p(rp.data_ptr()), C.c_void_p(col.data_ptr()), C.c_void_p(vals.data_ptr()),
                                 prob.n_nodes, prob.ndof, C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()),
                                 1e-12, 20000, stream, C.byref(na_info), err, 256)
        torch.cuda.synchronize()
        assert rc == N.AGX_OK, err.value
        assert na_info.rel_residual <= 1e-12
        sols.append(x.cpu().numpy())
    ref = x_ref.cpu().numpy()
    scale = max(1e-300, np.abs(ref).max())
    for s in sols:
        assert np.abs(s - ref).max() <= 1e-8 * scale
    assert np.abs(sols[0] - sols[1]).max() <= 1e-14 * scale


def test_noalloc_rejects_oversized_systems():
    lib = N.load()
    err = C.create_string_buffer(256)
    one = C.c_void_p(1)  # never dereferenced: the size check comes first
    n_nodes = N.AGX_NOALLOC_MAX_DOFS // 3 + 1
    rc = lib.agx_pcg_noalloc(one, one, one, n_nodes, 3, one, one, 1e-8, 10, None, None, err, 256)
    assert rc == -1 and b"exceed" in err.value
