"""BF16 tensor-core kernels of the learned preconditioner against the float64 oracle,
and the gain of the trained network inside flexible CG.

Tolerances (written where used): inputs and weights are bf16-representable, products are
accumulated in f32 and outputs rounded to bf16, so single convolutions agree with the
float64 oracle to 1e-2 of the output's max magnitude; weight gradients (f32 out) to 2e-3;
the whole network (bf16 activations between 15 layers) to 5e-2.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import nn as onn

pytestmark = pytest.mark.gpu


def _bf(t):
    return t.to(torch.bfloat16).to(torch.float64)


@pytest.mark.parametrize("c1,c2,co,relu", [(16, 0, 32, 1), (32, 0, 32, 1), (32, 32, 32, 1), (32, 0, 16, 0)])
def test_conv_forward_and_gradients(c1, c2, co, relu):
    from autopdex_gb300 import _native as N
    lib = N.load()
    dev = torch.device("cuda")
    g = torch.Generator().manual_seed(c1 * 7 + c2 + co)
    B, H, W = 2, 24, 40
    x1 = _bf(torch.randn(B, H, W, c1, generator=g, dtype=torch.float64))
    x2 = _bf(torch.randn(B, H, W, c2, generator=g, dtype=torch.float64)) if c2 else None
    w = _bf(torch.randn(co, c1 + c2, 3, 3, generator=g, dtype=torch.float64) * 0.2)
    b = torch.randn(co, generator=g, dtype=torch.float64) * 0.1
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    wd = w.float().to(dev).contiguous()
    imgf = torch.empty(co * (c1 + c2) * 9, dtype=torch.bfloat16, device=dev)
    imgb = torch.empty_like(imgf)
    assert lib.agx_nn_pack_weights(p(wd), co, c1 + c2, 0, p(imgf), s) == 0
    assert lib.agx_nn_pack_weights(p(wd), co, c1 + c2, 1, p(imgb), s) == 0
    x1d = x1.to(torch.bfloat16).to(dev).contiguous()
    x2d = x2.to(torch.bfloat16).to(dev).contiguous() if c2 else None
    bd = b.float().to(dev)
    out = torch.empty(B, H, W, co, dtype=torch.bfloat16, device=dev)
    assert lib.agx_nn_conv3x3(p(x1d), p(x2d), c1, c2, p(imgf), p(bd), p(out), None, co, co, relu, B, H, W, p(err),
                              s) == 0
    # oracle
    xin = torch.cat([x1, x2], -1) if c2 else x1
    xin.requires_grad_(True)
    wr = w.clone().requires_grad_(True)
    ref = onn.conv(xin, wr, b.float().double(), relu)
    got = out.double().cpu()
    assert (got - ref.detach()).abs().max() <= 1e-2 * ref.abs().max()
    # gradients of sum(ref * gy) for a bf16 gy at the pre-activation
    gy = _bf(torch.randn(B, H, W, co, generator=g, dtype=torch.float64))
    pre = onn.conv(xin, wr, b.float().double(), 0)
    (pre * gy).sum().backward()
    gyd = gy.to(torch.bfloat16).to(dev).contiguous()
    d1 = torch.empty(B, H, W, c1, dtype=torch.bfloat16, device=dev)
    d2 = torch.empty(B, H, W, c2, dtype=torch.bfloat16, device=dev) if c2 else None
    assert lib.agx_nn_conv3x3(p(gyd), None, co, 0, p(imgb), None, p(d1), p(d2), c1, c1 + c2, 0, B, H, W, p(err),
                              s) == 0
    dx = torch.cat([d1.double().cpu(), d2.double().cpu()], -1) if c2 else d1.double().cpu()
    assert (dx - xin.grad).abs().max() <= 1e-2 * xin.grad.abs().max()
    rows = torch.zeros(9 * (c1 + c2) * co, dtype=torch.float32, device=dev)
    assert lib.agx_nn_wgrad3x3(p(x1d), p(x2d), c1, c2, p(gyd), co, p(rows), B, H, W, p(err), s) == 0
    dw = torch.empty(co, c1 + c2, 3, 3, dtype=torch.float32, device=dev)
    assert lib.agx_nn_unpack_wgrad(p(rows), co, c1 + c2, p(dw), s) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert (dw.double().cpu() - wr.grad).abs().max() <= 2e-3 * wr.grad.abs().max()


def test_unet_forward_and_backward_match_oracle():
    """Forward against the float64 oracle; parameter gradients against the oracle's autograd
    with the ReLU masks taken from the GPU's own activations (a pre-activation within bf16
    rounding of zero may switch sides between precisions, which alone changes gradients by
    O(1) at that point)."""
    from autopdex_gb300 import learned
    net = learned.UNet(seed=3)
    B, H, W = 2, 32, 48
    g = torch.Generator().manual_seed(5)
    x = torch.zeros(B, H, W, 16, dtype=torch.float64)
    x[..., :2] = _bf(torch.randn(B, H, W, 2, generator=g, dtype=torch.float64))
    out, acts = net.forward(x.to(torch.bfloat16).cuda(), keep=True)
    P = {n: (_bf(net.w[n].double().cpu()).requires_grad_(True), net.b[n].double().cpu().requires_grad_(True))
         for n, *_ in learned.LAYERS}
    ref = onn.unet(x, {n: (w.detach(), b.detach()) for n, (w, b) in P.items()})
    assert (out.double().cpu() - ref).abs().max() <= 5e-2 * ref.abs().max()
    masks = {n: (acts[n].double().cpu() > 0).double() for n, c1, c2, co, relu in learned.LAYERS if relu}
    ref_m = onn.unet(x, P, masks=masks)
    gy = _bf(torch.randn(B, H, W, 16, generator=g, dtype=torch.float64))
    (ref_m * gy).sum().backward()
    gw, gb = net.backward(gy.to(torch.bfloat16).cuda(), acts)
    torch.cuda.synchronize()
    net.check()
    rel = {}
    for n, *_ in learned.LAYERS:
        rw, rb = P[n][0].grad, P[n][1].grad
        rel[n] = (float((gw[n].double().cpu() - rw).norm() / rw.norm()),
                  float((gb[n].double().cpu() - rb).norm() / rb.norm().clamp_min(1e-12)))
    assert all(a <= 3e-2 and b <= 3e-2 for a, b in rel.values()), rel


def test_trained_network_reduces_fcg_iterations():
    """A network trained for a few hundred steps on 64 x 64 problems, used as the flexible-CG
    preconditioner on an unseen conductivity field, needs fewer iterations than Jacobi-PCG to
    the same relative residual (both float32 with float64 dots)."""
    from autopdex_gb300 import _native as N
    from autopdex_gb300 import configs, learned
    from autopdex_gb300._problem import get_problem
    n = 64
    R, A, E = learned.make_training_set(48, n=n, seed0=0)
    net = learned.UNet(seed=1)
    losses = learned.train(net, R, A, E, n, steps=400, batch=8, lr=2e-3)
    assert sum(losses[-20:]) / 20 < 0.5 * sum(losses[:20]) / 20
    w = configs.heat_grf(n=n, seed=1000, precision="mixed")
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    x0 = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
    prob._call("agx_assemble", C.c_void_p(x0.data_ptr()), None, N.AGX_F32)
    mask = torch.as_tensor(prob.mask.astype(bool), device=prob.device)
    rhs = torch.where(mask, torch.zeros_like(x0), torch.ones_like(x0))
    its = {}
    pc = learned.GridPreconditioner(net, n, n, w.settings["conductivity"])
    cb = pc.callback(prob)
    for method in (N.AGX_PCG_MIXED, N.AGX_FCG_MIXED):
        prob._call("agx_set_preconditioner", cb if method == N.AGX_FCG_MIXED else N.PRECOND_FN(0), None)
        o = N.SolveOpts()
        o.method, o.rtol, o.atol, o.maxiter, o.check_every = method, 1e-6, 0.0, 20000, 8
        info = N.SolveInfo()
        x = torch.zeros_like(x0)
        prob._call("agx_solve", C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()), C.byref(o), C.byref(info))
        its[method] = (info.iterations, info.status)
    prob._call("agx_set_preconditioner", N.PRECOND_FN(0), None)
    assert its[N.AGX_FCG_MIXED][1] == N.AGX_OK and its[N.AGX_PCG_MIXED][1] == N.AGX_OK
    assert its[N.AGX_FCG_MIXED][0] < 0.7 * its[N.AGX_PCG_MIXED][0], its
