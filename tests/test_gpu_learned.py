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


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


@pytest.mark.parametrize("loader", [0, 1, 2])
@pytest.mark.parametrize("c1,c2,co,relu", [(16, 0, 32, 1), (32, 0, 32, 1), (32, 32, 32, 1), (32, 0, 16, 0)])
def test_conv_forward_and_gradients(c1, c2, co, relu, loader):
    from autopdex_gb300 import _native as N
    lib = N.load()
    assert lib.agx_nn_set_halo_loader(loader) == 0
    try:
        _conv_forward_and_gradients(lib, c1, c2, co, relu)
    finally:
        lib.agx_nn_set_halo_loader(3)


@pytest.mark.parametrize("c1,c2", [(32, 0), (32, 32)])
def test_conv_halo_loaders_agree_on_many_tiles(c1, c2):
    """The halo loaders (and the warp-specialised kernel) put the same operands in shared memory,
    so their outputs agree bit for bit; on an image with partial row tiles (W = 150) and several
    tiles per persistent CTA (1200 tiles), and within bf16 rounding of the float64 oracle."""
    from autopdex_gb300 import _native as N
    lib = N.load()
    dev = torch.device("cuda")
    g = torch.Generator().manual_seed(31 + c2)
    B, H, W, co = 2, 300, 150, 32
    x1 = _bf(torch.randn(B, H, W, c1, generator=g, dtype=torch.float64))
    x2 = _bf(torch.randn(B, H, W, c2, generator=g, dtype=torch.float64)) if c2 else None
    w = _bf(torch.randn(co, c1 + c2, 3, 3, generator=g, dtype=torch.float64) * 0.2)
    b = torch.randn(co, generator=g, dtype=torch.float64) * 0.1
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    wd = w.float().to(dev).contiguous()
    imgf = torch.empty(co * (c1 + c2) * 9, dtype=torch.bfloat16, device=dev)
    assert lib.agx_nn_pack_weights(_ptr(wd), co, c1 + c2, 0, _ptr(imgf), s) == 0
    x1d = x1.to(torch.bfloat16).to(dev).contiguous()
    x2d = x2.to(torch.bfloat16).to(dev).contiguous() if c2 else None
    bd = b.float().to(dev)
    outs = []
    try:
        for loader in (0, 1, 2):
            assert lib.agx_nn_set_halo_loader(loader) == 0
            out = torch.empty(B, H, W, co, dtype=torch.bfloat16, device=dev)
            assert lib.agx_nn_conv3x3(_ptr(x1d), _ptr(x2d), c1, c2, _ptr(imgf), _ptr(bd), _ptr(out), None, co, co, 1,
                                      B, H, W, _ptr(err), s) == 0
            outs.append(out)
    finally:
        lib.agx_nn_set_halo_loader(3)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[0], outs[2])
    # AGX_NN_CONST_WEIGHTS (weights copied before the programmatic-launch wait): same result;
    # unknown flag bits are refused
    out = torch.empty_like(outs[0])
    assert lib.agx_nn_conv3x3(_ptr(x1d), _ptr(x2d), c1, c2, _ptr(imgf), _ptr(bd), _ptr(out), None, co, co,
                              1 | N.AGX_NN_CONST_WEIGHTS, B, H, W, _ptr(err), s) == 0
    assert lib.agx_nn_conv3x3(_ptr(x1d), _ptr(x2d), c1, c2, _ptr(imgf), _ptr(bd), _ptr(out), None, co, co, 1 | 4,
                              B, H, W, _ptr(err), s) != 0
    torch.cuda.synchronize()
    assert torch.equal(outs[0], out)
    xin = torch.cat([x1, x2], -1) if c2 else x1
    ref = onn.conv(xin, w, b.float().double(), 1)
    assert (outs[0].double().cpu() - ref).abs().max() <= 1e-2 * ref.abs().max()


def _conv_forward_and_gradients(lib, c1, c2, co, relu):
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
    B, H, W = 2, 64, 128
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


def test_grid_transfer_matches_oracle():
    """agx_nn_prolong is bilinear interpolation (the oracle's P) and agx_nn_restrict its
    transpose, with flagged coarse nodes set to zero."""
    from autopdex_gb300 import _native as N
    lib = N.load()
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    g = torch.Generator().manual_seed(11)
    for Hc, Wc, f in ((5, 7, 1), (9, 6, 2), (17, 17, 4), (4, 5, 3)):
        Hf, Wf = (Hc - 1) * f + 1, (Wc - 1) * f + 1
        c = torch.randn(Hc, Wc, generator=g, dtype=torch.float64)
        u = torch.randn(Hf, Wf, generator=g, dtype=torch.float64)
        fine = torch.empty(Hf * Wf, dtype=torch.float32, device="cuda")
        assert lib.agx_nn_prolong(_ptr(c.float().cuda().reshape(-1).contiguous()), Hc, Wc, f, _ptr(fine), s) == 0
        ref = torch.as_tensor(onn.prolong(c.float().double().numpy(), f))
        assert (fine.double().cpu().reshape(Hf, Wf) - ref).abs().max() <= 1e-5 * ref.abs().max()
        fixed = torch.zeros(Hf, Wf, dtype=torch.uint8)
        fixed[0, :] = 1
        fixed[:, -1] = 1
        coarse = torch.empty(Hc * Wc, dtype=torch.float32, device="cuda")
        assert lib.agx_nn_restrict(_ptr(u.float().cuda().reshape(-1).contiguous()), _ptr(fixed.cuda()), Hc, Wc, f,
                                   _ptr(coarse), s) == 0
        # P^T u through the oracle's P applied to unit vectors: (P^T u)_(I,J) = <P e_IJ, u>
        rt = torch.zeros(Hc, Wc, dtype=torch.float64)
        uf = u.float().double().numpy()
        for I in range(Hc):
            for J in range(Wc):
                e = torch.zeros(Hc, Wc, dtype=torch.float64).numpy()
                e[I, J] = 1.0
                rt[I, J] = float((onn.prolong(e, f) * uf).sum())
        keep = (fixed[::f, ::f] == 0).double()
        rt = rt * keep
        assert (coarse.double().cpu().reshape(Hc, Wc) - rt).abs().max() <= 1e-5 * rt.abs().max()


@pytest.mark.parametrize("f", [2, 4])
def test_pool_and_upsample_match_torch(f):
    """agx_nn_pool / agx_nn_upsample (one launch for an f x f block) and their adjoints against
    PyTorch in float64 on bf16 inputs: pooling means and adjoint block sums are rounded to
    bf16 once (<= 2^-8 relative), broadcasts are exact."""
    import torch.nn.functional as F
    from autopdex_gb300 import _native as N
    lib = N.load()
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    g = torch.Generator().manual_seed(17)
    B, Hc, Wc, Cc = 2, 5, 7, 32
    H, W = Hc * f, Wc * f
    x = _bf(torch.randn(B, H, W, Cc, generator=g, dtype=torch.float64))
    xc = _bf(torch.randn(B, Hc, Wc, Cc, generator=g, dtype=torch.float64))
    nchw = lambda t: t.permute(0, 3, 1, 2)
    nhwc = lambda t: t.permute(0, 2, 3, 1)
    out = torch.empty(B, Hc, Wc, Cc, dtype=torch.bfloat16, device="cuda")
    assert lib.agx_nn_pool(_ptr(x.to(torch.bfloat16).cuda()), _ptr(out), B, H, W, Cc, f, 0, s) == 0
    ref = nhwc(F.avg_pool2d(nchw(x), f))
    assert (out.double().cpu() - ref).abs().max() <= 2 ** -8 * ref.abs().max()
    up = torch.empty(B, H, W, Cc, dtype=torch.bfloat16, device="cuda")
    assert lib.agx_nn_upsample(_ptr(xc.to(torch.bfloat16).cuda()), _ptr(up), B, Hc, Wc, Cc, f, 0, s) == 0
    assert torch.equal(up.double().cpu(), nhwc(F.interpolate(nchw(xc), scale_factor=f, mode="nearest")))
    # adjoints: <pool x, y> = <x, pool^T y> and <up y, x> = <y, up^T x>
    pt = torch.empty(B, H, W, Cc, dtype=torch.bfloat16, device="cuda")
    assert lib.agx_nn_pool(_ptr(xc.to(torch.bfloat16).cuda()), _ptr(pt), B, H, W, Cc, f, 1, s) == 0
    assert torch.equal(pt.double().cpu(), nhwc(F.interpolate(nchw(xc), scale_factor=f, mode="nearest")) / (f * f))
    ut = torch.empty(B, Hc, Wc, Cc, dtype=torch.bfloat16, device="cuda")
    assert lib.agx_nn_upsample(_ptr(x.to(torch.bfloat16).cuda()), _ptr(ut), B, Hc, Wc, Cc, f, 1, s) == 0
    ref = nhwc(F.avg_pool2d(nchw(x), f)) * (f * f)
    assert (ut.double().cpu() - ref).abs().max() <= 2 ** -8 * ref.abs().max()
    # misaligned pointers and channel counts are refused
    assert lib.agx_nn_pool(C.c_void_p(out.data_ptr() + 2), _ptr(out), B, H, W, Cc, f, 0, s) != 0
    assert lib.agx_nn_upsample(_ptr(xc.cuda()), _ptr(up), B, Hc, Wc, 12, f, 0, s) != 0


@pytest.mark.parametrize("Hn,Wn,offset", [(257, 257, 0), (1001, 999, 0), (61, 67, 1), (1, 3, 0)])
def test_image_scale_is_inverse_rms(Hn, Wn, offset):
    """The 1 / rms that agx_nn_grid_from_field writes (one cluster of CTAs, float4 loads when
    the field is 16-byte aligned, float per-thread sums) against float64: within 1e-6
    relative, for sizes that are not multiples of 4 and a misaligned field."""
    from autopdex_gb300 import _native as N
    from autopdex_gb300 import learned
    lib = N.load()
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = Hn * Wn
    g = torch.Generator().manual_seed(n)
    base = torch.randn(n + offset, generator=g, dtype=torch.float64) * 3.0
    r = base.float().cuda()
    src = C.c_void_p(r.data_ptr() + 4 * offset)
    Hp, Wp = learned.padded(Hn), learned.padded(Wn)
    img = torch.empty(1, Hp, Wp, 16, dtype=torch.bfloat16, device="cuda")
    scale = torch.empty(1, dtype=torch.float32, device="cuda")
    assert lib.agx_nn_grid_from_field(src, 1, None, 0, Hn, Wn, Hp, Wp, 1, _ptr(scale), _ptr(img), s) == 0
    v = base[offset:].float().double()
    ref = 1.0 / float(torch.sqrt((v * v).mean()))
    assert abs(float(scale.item()) - ref) <= 1e-6 * ref


@pytest.mark.parametrize("Hc,Wc,f,nd", [(17, 17, 4, 1), (9, 6, 2, 2), (4, 5, 3, 1), (33, 17, 8, 3)])
def test_fused_transfers_match_separate_ones(Hc, Wc, f, nd):
    """agx_nn_restrict_image (restriction, 1 / rms and the image in two launches) against
    agx_nn_restrict_field followed by agx_nn_grid_from_field, and agx_nn_prolong_image against
    agx_nn_prolong_field of the image's channels with the fixed DOFs zeroed: coarse values and
    1 / rms within 1e-6 relative, image and prolonged values within bf16 rounding (2^-8)."""
    from autopdex_gb300 import _native as N
    from autopdex_gb300 import learned
    lib = N.load()
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    g = torch.Generator().manual_seed(Hc * 100 + f)
    Hf, Wf = (Hc - 1) * f + 1, (Wc - 1) * f + 1
    Hp, Wp = learned.padded(Hc), learned.padded(Wc)
    fine = torch.randn(Hf * Wf * nd, generator=g).cuda()
    fixed = (torch.rand(Hf * Wf * nd, generator=g) < 0.1).to(torch.uint8).cuda()
    aux = torch.randn(Hc * Wc, generator=g).cuda()
    coarse = torch.empty(Hc * Wc * nd, device="cuda")
    ref_c = torch.empty_like(coarse)
    work = torch.zeros(lib.agx_nn_restrict_image_work(), dtype=torch.float64, device="cuda")
    scale, ref_s = torch.empty(1, device="cuda"), torch.empty(1, device="cuda")
    img = torch.empty(1, Hp, Wp, 16, dtype=torch.bfloat16, device="cuda")
    ref_img = torch.empty_like(img)
    assert lib.agx_nn_restrict_image(_ptr(fine), _ptr(fixed), nd, _ptr(aux), 1, Hc, Wc, f, Hp, Wp, _ptr(coarse),
                                     _ptr(work), _ptr(scale), _ptr(img), s) == 0
    assert lib.agx_nn_restrict_field(_ptr(fine), _ptr(fixed), nd, Hc, Wc, f, _ptr(ref_c), s) == 0
    assert lib.agx_nn_grid_from_field(_ptr(ref_c), nd, _ptr(aux), 1, Hc, Wc, Hp, Wp, 1, _ptr(ref_s), _ptr(ref_img),
                                      s) == 0
    torch.cuda.synchronize()
    assert (coarse - ref_c).abs().max() <= 1e-6 * ref_c.abs().max()
    assert abs(float(scale.item()) - float(ref_s.item())) <= 1e-6 * float(ref_s.item())
    assert (img.float() - ref_img.float()).abs().max() <= 2 ** -8 * ref_img.float().abs().max()
    # prolongation from the image's first nd channels
    out = torch.empty(Hf * Wf * nd, device="cuda")
    assert lib.agx_nn_prolong_image(_ptr(img), 16, nd, Hc, Wc, Wp, f, _ptr(fixed), _ptr(out), s) == 0
    yc = img[0, :Hc, :Wc, :nd].float().contiguous().reshape(-1)
    ref = torch.empty_like(out)
    assert lib.agx_nn_prolong_field(_ptr(yc), nd, Hc, Wc, f, _ptr(ref), s) == 0
    torch.cuda.synchronize()
    ref[fixed.bool()] = 0.0
    assert (out - ref).abs().max() <= 1e-6 * ref.abs().max()
    assert torch.all(out[fixed.bool()] == 0.0)


def test_programmatic_launch_changes_nothing():
    """The flexible CG with the two-level learned preconditioner (network on the grid coarsened
    by 2, CUDA graphs on) gives bit-identical iterates with programmatic dependent launch on and
    off: the kernels wait for their predecessors either way and every reduction has a fixed
    order."""
    from autopdex_gb300 import _native as N
    from autopdex_gb300 import configs, learned
    from autopdex_gb300._problem import get_problem
    net = learned.UNet(seed=4)
    n = 64
    w = configs.heat_grf(n=n, seed=77, precision="mixed")
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    x0 = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
    prob._call("agx_assemble", C.c_void_p(x0.data_ptr()), None, N.AGX_F32)
    mask = torch.as_tensor(prob.mask.astype(bool), device=prob.device)
    rhs = torch.where(mask, torch.zeros_like(x0), torch.ones_like(x0))
    pc = learned.GridPreconditioner(net, n, n, w.settings["conductivity"], factor=2)
    pc.attach(prob)
    res = []
    try:
        for on in (1, 0, 1):
            prob.lib.agx_set_pdl(on)
            o = N.SolveOpts()
            o.method, o.rtol, o.atol, o.maxiter, o.check_every = N.AGX_FCG_MIXED, 1e-6, 0.0, 2000, 8
            info = N.SolveInfo()
            x = torch.zeros_like(x0)
            prob._call("agx_solve", C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()), C.byref(o), C.byref(info))
            assert info.status == N.AGX_OK
            res.append((info.iterations, x.cpu()))
    finally:
        prob.lib.agx_set_pdl(1)
        prob._call("agx_set_preconditioner", N.PRECOND_FN(0), None)
    assert res[0][0] == res[1][0] == res[2][0]
    assert torch.equal(res[0][1], res[1][1]) and torch.equal(res[0][1], res[2][1])


def test_bf16_smoothing_products_converge_to_the_same_solution():
    """AGX_PRECOND_BF16_SMOOTHING (the two-level products on a bf16 copy of the values) only
    changes the preconditioner: flexible CG reaches the same 1e-8 relative residual, and the two
    solutions agree within 1e-4 relative (two solutions with residuals of 1e-8 may differ by up
    to the condition number, ~1e4 here, times that; 1.7e-6 measured)."""
    from autopdex_gb300 import _native as N
    from autopdex_gb300 import configs, learned
    from autopdex_gb300._problem import get_problem
    net = learned.UNet(seed=4)
    n = 64
    w = configs.heat_grf(n=n, seed=78, precision="mixed")
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    x0 = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
    prob._call("agx_assemble", C.c_void_p(x0.data_ptr()), None, N.AGX_F32)
    mask = torch.as_tensor(prob.mask.astype(bool), device=prob.device)
    rhs = torch.where(mask, torch.zeros_like(x0), torch.ones_like(x0))
    sols = []
    try:
        for bf16 in (False, True):
            pc = learned.GridPreconditioner(net, n, n, w.settings["conductivity"], factor=2, bf16_smoothing=bf16)
            pc.attach(prob)
            o = N.SolveOpts()
            o.method, o.rtol, o.atol, o.maxiter, o.check_every = N.AGX_FCG_MIXED, 1e-8, 0.0, 4000, 8
            info = N.SolveInfo()
            x = torch.zeros_like(x0)
            prob._call("agx_solve", C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()), C.byref(o), C.byref(info))
            assert info.status == N.AGX_OK and info.rel_residual <= 1e-8
            sols.append(x.cpu())
    finally:
        prob._call("agx_set_preconditioner", N.PRECOND_FN(0), None)
    assert (sols[0] - sols[1]).abs().max() <= 1e-4 * sols[0].abs().max()


def test_trained_network_reduces_fcg_iterations():
    """A network trained for a few hundred steps on 64 x 64 problems, used by flexible CG as
    the coarse solver of the symmetric two-level preconditioner on unseen conductivity fields,
    needs far fewer iterations than Jacobi-PCG and than the same two-level method without the
    network (the smoothing only, the network output replaced by zeros) to the same
    relative residual (float32 iterations with float64 dots): on a 64 x 64 problem with the
    network on the node grid itself (damped Jacobi smoothing), and on a 128 x 128 problem with
    the network on the grid coarsened by 2 (bilinear transfer, Chebyshev smoothing)."""
    from autopdex_gb300 import _native as N
    from autopdex_gb300 import configs, learned
    from autopdex_gb300._problem import get_problem
    ts = learned.make_training_set(48, n=64, seed0=0)
    net = learned.UNet(seed=1)
    losses = learned.train(net, ts, steps=600, batch=8, lr=2e-3)
    assert sum(losses[-20:]) / 20 < 0.5 * sum(losses[:20]) / 20
    results = {}
    for n, factor, seed in ((64, 1, 1000), (128, 2, 1001)):
        w = configs.heat_grf(n=n, seed=seed, precision="mixed")
        prob = get_problem(w.dofs, w.settings, w.static_settings)
        prob.update_models(w.settings)
        x0 = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
        prob._call("agx_assemble", C.c_void_p(x0.data_ptr()), None, N.AGX_F32)
        mask = torch.as_tensor(prob.mask.astype(bool), device=prob.device)
        rhs = torch.where(mask, torch.zeros_like(x0), torch.ones_like(x0))
        pc = learned.GridPreconditioner(net, n, n, w.settings["conductivity"], factor=factor)
        zero = torch.zeros(prob.n_dofs, dtype=torch.float32, device=prob.device)

        def no_network(user, r, z, nn, stream):
            return prob.lib.agx_nn_restrict(C.c_void_p(zero.data_ptr()), None, n + 1, n + 1, 1, C.c_void_p(z),
                                            C.c_void_p(stream))
        no_network_cb = N.PRECOND_FN(no_network)

        def solve(method, cb):
            prob._call("agx_set_preconditioner", cb, None)
            prob._call("agx_set_preconditioner_mode", pc.mode, pc.omega, pc.sweeps, N.AGX_PRECOND_CAPTURABLE)
            o = N.SolveOpts()
            o.method, o.rtol, o.atol, o.maxiter, o.check_every = method, 1e-6, 0.0, 20000, 8
            info = N.SolveInfo()
            x = torch.zeros_like(x0)
            prob._call("agx_solve", C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()), C.byref(o),
                       C.byref(info))
            assert info.status == N.AGX_OK
            return info.iterations

        its = {"jacobi_pcg": solve(N.AGX_PCG_MIXED, N.PRECOND_FN(0)),
               "two_level_without_network": solve(N.AGX_FCG_MIXED, no_network_cb),
               "two_level_with_network": solve(N.AGX_FCG_MIXED, pc.callback(prob))}
        prob._call("agx_set_preconditioner", N.PRECOND_FN(0), None)
        net.check()
        results[n] = its
    print("iterations", results)
    for its in results.values():
        assert its["two_level_with_network"] < 0.3 * its["jacobi_pcg"], results
        # the weight gradient sums with float atomics, so the trained network and its count vary
        # from run to run (16-19 of 87 at 64, 23-28 of 77 at 128 observed)
        assert its["two_level_with_network"] < 0.4 * its["two_level_without_network"], results


def test_network_autotuner_picks_a_variant_per_layer_and_keeps_outputs():
    """UNet.autotune (coordinate descent over every layer's three convolution variants, each
    candidate network timed as a replayed CUDA graph) ends no slower than it started, keeps one
    variant per layer, and -- the variants giving identical outputs -- leaves the network's
    output bit-identical."""
    from autopdex_gb300 import learned
    net = learned.UNet(seed=4)
    g = torch.Generator().manual_seed(9)
    x = torch.zeros(1, 320, 320, 16, dtype=torch.float64)
    x[..., :2] = torch.randn(1, 320, 320, 2, generator=g, dtype=torch.float64)
    xd = x.to(torch.bfloat16).cuda()
    before = net.forward(xd).clone()
    chosen = net.autotune(xd)
    after = net.forward(xd)
    torch.cuda.synchronize()
    net.check()
    t0, t1 = chosen.pop("us_per_pass")
    assert 0 < t1 <= t0
    assert set(chosen) == {name for name, *_ in learned.LAYERS}
    assert all(lo in (0, 1, 2) and all(t > 0 for t in times.values()) for lo, times in chosen.values())
    assert torch.equal(before, after)
