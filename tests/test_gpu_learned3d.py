"""The 3-D learned preconditioner's BF16 tensor-core kernels (3x3x3 convolutions, their input
and weight gradients, 2x2x2 pooling and upsampling, the brick-mesh transfers) against the
float64 oracle, and the preconditioner inside flexible CG on the backward-Euler heat workload.

Tolerances (written where used) follow the 2-D kernels': bf16-representable inputs and weights,
f32 accumulation and bf16 outputs -> single convolutions within 1e-2 of the output's max
magnitude; weight gradients (f32 out) within 2e-3; the whole network within 5e-2; transfers
(f32) within 1e-5.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import nn as onn

pytestmark = pytest.mark.gpu


def _bf(t):
    return t.to(torch.bfloat16).to(torch.float64)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("c1,c2,relu", [(16, 0, 1), (16, 16, 1), (16, 0, 0)])
def test_conv3x3x3_forward_input_and_weight_gradients(c1, c2, relu):
    """Forward, input gradient (the flipped weight image, split into the two inputs' channels)
    and weight gradient of one 3x3x3 layer against F.conv3d in float64, on a volume whose
    extents are not multiples of the 8 x 16 tile (partial tiles at both edges) with two batch
    entries and more tiles than CTAs."""
    from autopdex_gb300 import _native as N
    lib = N.load()
    dev = torch.device("cuda")
    g = torch.Generator().manual_seed(7 + c2 + relu)
    B, D, H, W, co = 2, 9, 37, 21, 16
    x1 = _bf(torch.randn(B, D, H, W, c1, generator=g, dtype=torch.float64))
    x2 = _bf(torch.randn(B, D, H, W, c2, generator=g, dtype=torch.float64)) if c2 else None
    w = _bf(torch.randn(co, c1 + c2, 3, 3, 3, generator=g, dtype=torch.float64) * 0.1)
    b = torch.randn(co, generator=g, dtype=torch.float64) * 0.1
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    s = _stream()
    wd = w.float().to(dev).contiguous()
    n = co * (c1 + c2) * 27
    imgf = torch.empty(n, dtype=torch.bfloat16, device=dev)
    imgb = torch.empty(n, dtype=torch.bfloat16, device=dev)
    assert lib.agx_nn_pack_weights3d(_ptr(wd), co, c1 + c2, 0, _ptr(imgf), s) == 0
    assert lib.agx_nn_pack_weights3d(_ptr(wd), co, c1 + c2, 1, _ptr(imgb), s) == 0
    x1d = x1.to(torch.bfloat16).to(dev).contiguous()
    x2d = x2.to(torch.bfloat16).to(dev).contiguous() if c2 else None
    bd = b.float().to(dev)
    out = torch.empty(B, D, H, W, co, dtype=torch.bfloat16, device=dev)
    assert lib.agx_nn_conv3x3x3(_ptr(x1d), _ptr(x2d), c1, c2, _ptr(imgf), _ptr(bd), _ptr(out), None, co, co, relu, B,
                                D, H, W, _ptr(err), s) == 0
    xin = torch.cat([x1, x2], -1) if c2 else x1
    ref = onn.conv3d(xin, w, b, relu)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert (out.double().cpu() - ref).abs().max() <= 1e-2 * ref.abs().max()
    # input gradient: out = conv(x) (pre-activation), gy random -> dx = conv^T gy
    gy = _bf(torch.randn(B, D, H, W, co, generator=g, dtype=torch.float64))
    gyd = gy.to(torch.bfloat16).to(dev).contiguous()
    d1 = torch.empty(B, D, H, W, c1, dtype=torch.bfloat16, device=dev)
    d2 = torch.empty(B, D, H, W, c2, dtype=torch.bfloat16, device=dev) if c2 else None
    assert lib.agx_nn_conv3x3x3(_ptr(gyd), None, co, 0, _ptr(imgb), None, _ptr(d1), _ptr(d2), c1, c1 + c2, 0, B, D,
                                H, W, _ptr(err), s) == 0
    xr = xin.clone().requires_grad_(True)
    wr = w.clone().requires_grad_(True)
    (onn.conv3d(xr, wr, b, 0) * gy).sum().backward()
    got = torch.cat([d1, d2], -1) if c2 else d1
    torch.cuda.synchronize()
    assert (got.double().cpu() - xr.grad).abs().max() <= 1e-2 * xr.grad.abs().max()
    # weight gradient
    rows = torch.zeros(27 * (c1 + c2) * co, dtype=torch.float32, device=dev)
    assert lib.agx_nn_wgrad3x3x3(_ptr(x1d), _ptr(x2d), c1, c2, _ptr(gyd), co, _ptr(rows), B, D, H, W, _ptr(err),
                                 s) == 0
    dw = torch.empty(co, c1 + c2, 3, 3, 3, dtype=torch.float32, device=dev)
    assert lib.agx_nn_unpack_wgrad3d(_ptr(rows), co, c1 + c2, _ptr(dw), s) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert (dw.double().cpu() - wr.grad).abs().max() <= 2e-3 * wr.grad.abs().max()


def test_conv3x3x3_refuses_unsupported_shapes():
    from autopdex_gb300 import _native as N
    lib = N.load()
    dev = torch.device("cuda")
    x = torch.zeros(1, 4, 4, 8, 16, dtype=torch.bfloat16, device=dev)
    wimg = torch.zeros(27 * 32 * 16, dtype=torch.bfloat16, device=dev)
    out = torch.empty_like(x)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    s = _stream()
    assert lib.agx_nn_conv3x3x3(_ptr(x), None, 32, 0, _ptr(wimg), None, _ptr(out), None, 16, 16, 0, 1, 4, 4, 8,
                                _ptr(err), s) == N.AGX_ERR_UNSUPPORTED
    assert lib.agx_nn_conv3x3x3(_ptr(x), None, 16, 16, _ptr(wimg), None, _ptr(out), None, 16, 16, 1, 1, 4, 4, 8,
                                _ptr(err), s) == N.AGX_ERR_ARG  # second input missing
    assert lib.agx_nn_conv3x3x3(_ptr(x), None, 16, 0, C.c_void_p(wimg.data_ptr() + 2), None, _ptr(out), None, 16,
                                16, 1, 1, 4, 4, 8, _ptr(err), s) == N.AGX_ERR_ARG  # misaligned weights


def test_pool3d_and_upsample3d_match_torch():
    import torch.nn.functional as F
    from autopdex_gb300 import _native as N
    lib = N.load()
    s = _stream()
    g = torch.Generator().manual_seed(19)
    B, Dc, Hc, Wc, Cc, f = 2, 3, 5, 4, 16, 2
    D, H, W = Dc * f, Hc * f, Wc * f
    x = _bf(torch.randn(B, D, H, W, Cc, generator=g, dtype=torch.float64))
    xc = _bf(torch.randn(B, Dc, Hc, Wc, Cc, generator=g, dtype=torch.float64))
    ncdhw = lambda t: t.permute(0, 4, 1, 2, 3)
    ndhwc = lambda t: t.permute(0, 2, 3, 4, 1)
    out = torch.empty(B, Dc, Hc, Wc, Cc, dtype=torch.bfloat16, device="cuda")
    assert lib.agx_nn_pool3d(_ptr(x.to(torch.bfloat16).cuda()), _ptr(out), B, D, H, W, Cc, f, 0, s) == 0
    ref = ndhwc(F.avg_pool3d(ncdhw(x), f))
    assert (out.double().cpu() - ref).abs().max() <= 2 ** -8 * ref.abs().max()
    up = torch.empty(B, D, H, W, Cc, dtype=torch.bfloat16, device="cuda")
    assert lib.agx_nn_upsample3d(_ptr(xc.to(torch.bfloat16).cuda()), _ptr(up), B, Dc, Hc, Wc, Cc, f, 0, s) == 0
    rup = ndhwc(F.interpolate(ncdhw(xc), scale_factor=f, mode="nearest"))
    assert torch.equal(up.double().cpu(), rup)
    pt = torch.empty(B, D, H, W, Cc, dtype=torch.bfloat16, device="cuda")
    assert lib.agx_nn_pool3d(_ptr(xc.to(torch.bfloat16).cuda()), _ptr(pt), B, D, H, W, Cc, f, 1, s) == 0
    assert torch.equal(pt.double().cpu(), rup / f ** 3)
    ut = torch.empty(B, Dc, Hc, Wc, Cc, dtype=torch.bfloat16, device="cuda")
    assert lib.agx_nn_upsample3d(_ptr(x.to(torch.bfloat16).cuda()), _ptr(ut), B, Dc, Hc, Wc, Cc, f, 1, s) == 0
    ref = ndhwc(F.avg_pool3d(ncdhw(x), f)) * f ** 3
    assert (ut.double().cpu() - ref).abs().max() <= 2 ** -8 * ref.abs().max()
    assert lib.agx_nn_pool3d(_ptr(x.cuda()), _ptr(out), B, D + 1, H, W, Cc, f, 0, s) != 0


def test_unet3d_forward_and_backward_match_oracle():
    """As the 2-D test: forward against the float64 oracle, parameter gradients against its
    autograd with the ReLU masks of the GPU's own activations."""
    from autopdex_gb300 import learned
    net = learned.UNet3D(seed=3)
    B, D, H, W = 2, 8, 16, 24
    g = torch.Generator().manual_seed(5)
    x = torch.zeros(B, D, H, W, 16, dtype=torch.float64)
    x[..., :2] = _bf(torch.randn(B, D, H, W, 2, generator=g, dtype=torch.float64))
    out, acts = net.forward(x.to(torch.bfloat16).cuda(), keep=True)
    P = {n: (_bf(net.w[n].double().cpu()).requires_grad_(True), net.b[n].double().cpu().requires_grad_(True))
         for n, *_ in learned.LAYERS3}
    ref = onn.unet3d(x, {n: (w.detach(), b.detach()) for n, (w, b) in P.items()})
    assert (out.double().cpu() - ref).abs().max() <= 5e-2 * ref.abs().max()
    masks = {n: (acts[n].double().cpu() > 0).double() for n, c1, c2, co, relu in learned.LAYERS3 if relu}
    ref_m = onn.unet3d(x, P, masks=masks)
    gy = _bf(torch.randn(B, D, H, W, 16, generator=g, dtype=torch.float64))
    (ref_m * gy).sum().backward()
    gw, gb = net.backward(gy.to(torch.bfloat16).cuda(), acts)
    torch.cuda.synchronize()
    net.check()
    rel = {}
    for n, *_ in learned.LAYERS3:
        rw, rb = P[n][0].grad, P[n][1].grad
        rel[n] = (float((gw[n].double().cpu() - rw).norm() / rw.norm()),
                  float((gb[n].double().cpu() - rb).norm() / rb.norm().clamp_min(1e-12)))
    assert all(a <= 3e-2 and b <= 3e-2 for a, b in rel.values()), rel


@pytest.mark.parametrize("nc,f,npad", [(5, 2, 8), (9, 4, 16), (4, 3, 8)])
def test_brick_transfers_match_oracle(nc, f, npad):
    """restrict_image3d = (P^T r, masked under fixed fine nodes) / rms in channel 0 and the
    domain indicator in channel 1 of a padded image; prolong_image3d = P (channel 0), zero at
    fixed nodes; restrict3d = P^T alone."""
    from autopdex_gb300 import _native as N
    lib = N.load()
    s = _stream()
    rng = np.random.default_rng(nc + f)
    nf = (nc - 1) * f + 1
    r = rng.standard_normal((nf, nf, nf)).astype(np.float32)
    fixed = np.zeros((nf, nf, nf), dtype=np.uint8)
    fixed[0], fixed[:, -1], fixed[:, :, 0] = 1, 1, 1
    rc = torch.empty(nc ** 3, dtype=torch.float32, device="cuda")
    work = torch.empty(lib.agx_nn_restrict_image3d_work(), dtype=torch.float64, device="cuda")
    sc = torch.empty(1, dtype=torch.float32, device="cuda")
    img = torch.full((1, npad, npad, npad, 16), 7.0, dtype=torch.bfloat16, device="cuda")
    rd = torch.as_tensor(r.reshape(-1)).cuda()
    fd = torch.as_tensor(fixed.reshape(-1)).cuda()
    assert lib.agx_nn_restrict_image3d(_ptr(rd), _ptr(fd), nc, nc, nc, f, npad, npad, npad, _ptr(rc), _ptr(work),
                                       _ptr(sc), _ptr(img), s) == 0
    ref = onn.restrict3(r.astype(np.float64), f, (nc, nc, nc)) * (fixed[::f, ::f, ::f] == 0)
    got = rc.double().cpu().numpy().reshape(nc, nc, nc)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    scale = 1.0 / np.sqrt((ref ** 2).mean())
    assert abs(float(sc.item()) - scale) <= 1e-5 * scale
    im = img.double().cpu().numpy()[0]
    assert np.abs(im[:nc, :nc, :nc, 0] - ref * scale).max() <= 2 ** -8 * np.abs(ref * scale).max()
    assert np.all(im[:nc, :nc, :nc, 1] == 1.0) and np.all(im[:nc, :nc, :nc, 2:] == 0.0)
    assert np.all(im[nc:] == 0.0) and np.all(im[:, nc:] == 0.0) and np.all(im[:, :, nc:] == 0.0)
    # prolongation of channel 0 of an image with 16 channels
    cimg = torch.zeros(1, npad, npad, npad, 16, dtype=torch.float64)
    cimg[0, :nc, :nc, :nc, 0] = _bf(torch.as_tensor(rng.standard_normal((nc, nc, nc))))
    fine = torch.empty(nf ** 3, dtype=torch.float32, device="cuda")
    assert lib.agx_nn_prolong_image3d(_ptr(cimg.to(torch.bfloat16).cuda()), 16, nc, nc, nc, npad, npad, f, _ptr(fd),
                                      _ptr(fine), s) == 0
    pref = onn.prolong3(cimg[0, :nc, :nc, :nc, 0].numpy(), f) * (fixed == 0)
    assert np.abs(fine.double().cpu().numpy().reshape(nf, nf, nf) - pref).max() <= 1e-5 * np.abs(pref).max()
    plain = torch.empty(nc ** 3, dtype=torch.float32, device="cuda")
    assert lib.agx_nn_restrict3d(_ptr(rd), None, nc, nc, nc, f, _ptr(plain), s) == 0
    ref2 = onn.restrict3(r.astype(np.float64), f, (nc, nc, nc))
    assert np.abs(plain.double().cpu().numpy().reshape(nc, nc, nc) - ref2).max() <= 1e-5 * np.abs(ref2).max()


def _heat_be_step(n, learned_pc):
    """One backward-Euler step of the heat_transient workload at n^3: Newton to a 1e-10
    residual ratio with learned + mixed FCG (learned_pc set) or mixed Jacobi-PCG."""
    from autopdex_gb300 import configs, solver
    st = dict(precision="mixed", solver="fcg", **{"type of preconditioner": "learned"}) if learned_pc \
        else dict(precision="mixed", solver="pcg")
    w = configs.heat_transient(n=n, seed=2)
    static = dict(w.static_settings, **st)
    if learned_pc is not None:
        solver.set_learned_preconditioner(None, learned_pc)
    try:
        sol, (it, res, div) = solver.solver(w.dofs, w.settings, static, newton_tol=0.0, newton_rtol=1e-10,
                                            maxiter=20)
    finally:
        solver.set_learned_preconditioner(None, None)
    return w, sol, it, res, div


def test_brick_preconditioner_in_fcg_reaches_the_oracle_solution():
    """A randomly initialised 3-D network as the coarse solver of FCG on the 32^3 backward-Euler
    heat workload (coarse grid 9^3, image 16^3): the Newton solve reaches the same time step as
    mixed Jacobi-PCG (both judged by the float64 residual), within 1e-8 of the solution's max,
    and the network was applied."""
    from autopdex_gb300 import learned
    net = learned.UNet3D(seed=1)
    pc = learned.BrickPreconditioner(net, 32, factor=4)
    w, sol, it, res, div = _heat_be_step(32, pc)
    assert not div and pc.applications > 0
    _, ref, it2, res2, div2 = _heat_be_step(32, None)
    assert not div2
    a, b = sol["T"].reshape(-1), ref["T"].reshape(-1)
    a = a.cpu().numpy() if hasattr(a, "cpu") else np.asarray(a)
    b = b.cpu().numpy() if hasattr(b, "cpu") else np.asarray(b)
    assert np.abs(a - b).max() <= 1e-8 * max(1.0, np.abs(b).max())
    net.check()


def test_trained_brick_network_cuts_krylov_iterations_at_128cube():
    """The committed 3-D network (trained on the 128^3 workload's family) inside mixed FCG on the
    first time step of the 128^3 backward-Euler heat workload: the step reaches the same
    solution as mixed Jacobi-PCG (1e-8 of its max; both Newton to a 1e-10 float64 residual
    ratio) with under a third of its Krylov iterations (measured with the default two damped
    Jacobi sweeps: about a sixth)."""
    import os
    from autopdex_gb300 import learned, solver
    path = os.path.join(learned.WEIGHTS_DIR, "brick_unet_n128.npz")
    net = learned.UNet3D.load(path)
    pc = learned.BrickPreconditioner(net, 128, factor=4)
    its = {}
    sols = {}
    for name, p in (("learned", pc), ("jacobi", None)):
        w, sol, it, res, div = _heat_be_step(128, p)
        assert not div
        its[name] = int(solver.last_info.krylov_iterations)
        a = sol["T"].reshape(-1)
        sols[name] = a.cpu().numpy() if hasattr(a, "cpu") else np.asarray(a)
    assert np.abs(sols["learned"] - sols["jacobi"]).max() <= 1e-8 * max(1.0, np.abs(sols["jacobi"]).max())
    assert its["learned"] * 3 < its["jacobi"], its
    net.check()
