"""The autotuner's SpMV variants (1, 2, 4, 8 or 16 lanes per block row with two blocks per lane
and trip; 2, 4 or 8 lanes with four blocks, code lanes + 256; on a structured QUAD4 grid the
index-free grid product, code 512, or with two rows per lane, 1024) solve identically, the autotuner picks one of them per
precision, and invalid tuning values are rejected.

Tolerances, written where used: float64 products of one variant against SciPy's CSR product of
the same matrix <= 1e-13 of max |y| (summation order differs); solutions of the variants within
1e-8 (float64 PCG to 1e-10) or 1e-3 (float32 PCG to 1e-5) of each other."""
import ctypes as C

import numpy as np
import pytest
import torch

from autopdex_gb300 import _native as N
from autopdex_gb300 import configs
from autopdex_gb300._problem import get_problem

pytestmark = pytest.mark.gpu

VARIANTS = (1, 2, 4, 8, 16, 2 + 256, 4 + 256, 8 + 256, 512, 1024)  # 512, 1024: the structured grid's products


def _solve(prob, rhs, method):
    o = N.SolveOpts()
    o.method, o.rtol, o.atol, o.maxiter, o.check_every = method, 1e-10 if method == N.AGX_PCG else 1e-5, 0.0, 20000, 32
    info = N.SolveInfo()
    x = torch.zeros_like(rhs)
    prob._call("agx_solve", C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()), C.byref(o), C.byref(info))
    assert info.status == N.AGX_OK
    return x.cpu().numpy(), info.iterations


@pytest.mark.parametrize("dtype", [N.AGX_F64, N.AGX_F32])
def test_variants_agree_and_autotuner_picks_one(dtype):
    w = configs.heat_grf(n=48, seed=2)
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    x0 = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
    prob._call("agx_assemble", C.c_void_p(x0.data_ptr()), None, dtype)
    mask = torch.as_tensor(prob.mask.astype(bool), device=prob.device)
    rhs = torch.where(mask, torch.zeros_like(x0), torch.ones_like(x0))
    method = N.AGX_PCG if dtype == N.AGX_F64 else N.AGX_PCG_MIXED
    sols = {}
    for tpr in VARIANTS:
        prob._call("agx_set_tuning", dtype, tpr)
        sols[tpr] = _solve(prob, rhs, method)
    ref, its = sols[4]
    tol = 1e-8 if dtype == N.AGX_F64 else 1e-3
    for tpr, (x, n) in sols.items():
        assert np.abs(x - ref).max() <= tol * np.abs(ref).max(), tpr
        assert abs(n - its) <= 2 + its // 50, (tpr, n, its)
    tpr = C.c_int()
    ms = C.c_float()
    prob._call("agx_autotune", C.byref(tpr), C.byref(ms))
    assert tpr.value in VARIANTS and ms.value > 0.0
    prob._call("agx_set_tuning", dtype, 0)


def test_invalid_tuning_is_rejected():
    w = configs.neo_hooke_cube(n=2, n_steps=1)
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    lib = prob.lib
    assert lib.agx_set_tuning(prob.ctx, N.AGX_F32, 3) != N.AGX_OK
    assert lib.agx_set_tuning(prob.ctx, N.AGX_F32, 2) != N.AGX_OK  # 3 DOFs per node need >= 4 lanes
    assert lib.agx_set_tuning(prob.ctx, 7, 4) != N.AGX_OK
    assert lib.agx_set_tuning(prob.ctx, N.AGX_F32, 16 + 256) != N.AGX_OK  # no four-block variant with 16 lanes
    assert lib.agx_set_tuning(prob.ctx, N.AGX_F32, 2 + 256) != N.AGX_OK  # 3 DOFs per node need >= 4 lanes
    assert lib.agx_set_tuning(prob.ctx, N.AGX_F32, 8 + 256) == N.AGX_OK
    assert lib.agx_set_tuning(prob.ctx, N.AGX_F64, 8) == N.AGX_OK
    assert lib.agx_set_tuning(prob.ctx, N.AGX_F64, 512) != N.AGX_OK  # hexahedra: no grid product
    assert lib.agx_set_tuning(prob.ctx, N.AGX_F64, 2048) == N.AGX_OK  # a structured brick grid
    w2 = configs.heat_grf(n=8, seed=1)
    prob2 = get_problem(w2.dofs, w2.settings, w2.static_settings)
    assert prob2.lib.agx_set_tuning(prob2.ctx, N.AGX_F32, 2048) != N.AGX_OK  # quads: no brick product


@pytest.mark.parametrize("case", ["heat", "cook"])
def test_grid_product_matches_scipy(case):
    """agx_spmv with the grid product (code 512) on a structured QUAD4 grid -- one DOF per node
    (heat) and two (the Cook membrane's skewed grid) -- against SciPy's product of the copied
    CSR matrix, float64 and float32 tangents."""
    import scipy.sparse as sps
    w = configs.heat_grf(n=37, seed=3) if case == "heat" else configs.cook_membrane(n=23, n_steps=2)
    if case == "cook":
        w.settings["load multiplier"] = 0.03
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    rng = np.random.default_rng(4)
    u = torch.as_tensor(rng.uniform(-1e-3, 1e-3, prob.n_dofs), device=prob.device)
    nd = prob.ndof
    for dtype, tdt, tol in ((N.AGX_F64, torch.float64, 1e-13), (N.AGX_F32, torch.float32, 2e-6)):
        prob._call("agx_assemble", C.c_void_p(u.data_ptr()), None, dtype)
        nn = prob.n_dofs // nd
        rowptr = torch.empty(nn + 1, dtype=torch.int32, device=prob.device)
        col = torch.empty(prob.nnzb, dtype=torch.int32, device=prob.device)
        vals = torch.empty(prob.nnzb * nd * nd, dtype=tdt, device=prob.device)
        prob._call("agx_copy_matrix", dtype, C.c_void_p(rowptr.data_ptr()), C.c_void_p(col.data_ptr()),
                   C.c_void_p(vals.data_ptr()))
        blocks = vals.double().cpu().numpy().reshape(-1, nd, nd)  # row-major blocks
        A = sps.bsr_matrix((blocks, col.cpu().numpy(), rowptr.cpu().numpy()), shape=(prob.n_dofs, prob.n_dofs))
        x = torch.as_tensor(rng.standard_normal(prob.n_dofs), device=prob.device).to(tdt)
        ref = A @ x.double().cpu().numpy()
        for code in (512, 1024, 4):
            prob._call("agx_set_tuning", dtype, code)
            y = torch.empty_like(x)
            prob._call("agx_spmv", dtype, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))
            assert np.abs(y.double().cpu().numpy() - ref).max() <= tol * np.abs(ref).max(), (case, dtype, code)
        prob._call("agx_set_tuning", dtype, 0)


def test_autotuner_times_real_products():
    """Every timed launch does the full product: the reported time is not below what the
    matrix bytes need at 8 TB/s (a launch that found the solve flagged as finished would
    return at once and report a few microseconds)."""
    w = configs.heat_grf(n=1024, seed=1)
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    x0 = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
    for dtype, s in ((N.AGX_F32, 4), (N.AGX_F64, 8)):
        prob._call("agx_assemble", C.c_void_p(x0.data_ptr()), None, dtype)
        tpr = C.c_int()
        ms = C.c_float()
        prob._call("agx_autotune", C.byref(tpr), C.byref(ms))
        matrix_bytes = prob.nnzb * (s + (0 if tpr.value in (512, 1024, 2048) else 4))  # the grid products read no indices
        assert ms.value * 1e-3 >= matrix_bytes / 8e12, (dtype, tpr.value, ms.value)


@pytest.mark.parametrize("case", ["heat_be", "neo_hooke", "sheared"])
def test_brick_product_matches_scipy(case):
    """agx_spmv with the brick product (code 2048) on structured HEX8 grids -- one DOF per node
    (the backward-Euler heat workload, non-cubic 9 x 7 x 5 and a sheared lattice) and three (the
    neo-Hooke cube) -- against SciPy's product of the copied matrix, float64 and float32
    tangents; the fused Krylov product of the variant solves like the default one."""
    import scipy.sparse as sps
    if case == "neo_hooke":
        w = configs.neo_hooke_cube(n=6, n_steps=2)
    elif case == "heat_be":
        w = configs.heat_transient(n=8, n_steps=1)
    else:
        from test_gpu_parity import _sheared_brick_heat_be
        w = _sheared_brick_heat_be(shape=(9, 7, 5))
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    code = C.c_int()
    prob._call("agx_brick_pattern", C.byref(code))
    assert code.value > 0
    rng = np.random.default_rng(6)
    u = torch.as_tensor(rng.uniform(-1e-3, 1e-3, prob.n_dofs), device=prob.device)
    nd = prob.ndof
    for dtype, tdt, tol in ((N.AGX_F64, torch.float64, 1e-13), (N.AGX_F32, torch.float32, 2e-6)):
        prob._call("agx_assemble", C.c_void_p(u.data_ptr()), None, dtype)
        nn = prob.n_dofs // nd
        rowptr = torch.empty(nn + 1, dtype=torch.int32, device=prob.device)
        col = torch.empty(prob.nnzb, dtype=torch.int32, device=prob.device)
        vals = torch.empty(prob.nnzb * nd * nd, dtype=tdt, device=prob.device)
        prob._call("agx_copy_matrix", dtype, C.c_void_p(rowptr.data_ptr()), C.c_void_p(col.data_ptr()),
                   C.c_void_p(vals.data_ptr()))
        blocks = vals.double().cpu().numpy().reshape(-1, nd, nd)
        A = sps.bsr_matrix((blocks, col.cpu().numpy(), rowptr.cpu().numpy()), shape=(prob.n_dofs, prob.n_dofs))
        x = torch.as_tensor(rng.standard_normal(prob.n_dofs), device=prob.device).to(tdt)
        ref = A @ x.double().cpu().numpy()
        for c in (2048, 8):
            prob._call("agx_set_tuning", dtype, c)
            y = torch.empty_like(x)
            prob._call("agx_spmv", dtype, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))
            assert np.abs(y.double().cpu().numpy() - ref).max() <= tol * np.abs(ref).max(), (case, dtype, c)
        if case != "neo_hooke":  # at T = 0 the heat tangent is SPD: the fused product inside PCG
            zero = torch.zeros_like(u)
            prob._call("agx_assemble", C.c_void_p(zero.data_ptr()), None, dtype)
            mask = torch.as_tensor(prob.mask.astype(bool), device=prob.device)
            rhs = torch.where(mask, torch.zeros_like(u), torch.ones_like(u))
            method = N.AGX_PCG if dtype == N.AGX_F64 else N.AGX_PCG_MIXED
            sols = {}
            for c in (2048, 8):
                prob._call("agx_set_tuning", dtype, c)
                sols[c] = _solve(prob, rhs, method)
            tol_s = 1e-8 if dtype == N.AGX_F64 else 1e-3
            assert np.abs(sols[2048][0] - sols[8][0]).max() <= tol_s * np.abs(sols[8][0]).max()
        prob._call("agx_set_tuning", dtype, 0)
