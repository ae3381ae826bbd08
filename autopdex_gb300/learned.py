"""Learned preconditioner: a 4-level, 32-channel convolutional U-Net on the node grid.

The network maps a residual r (and the log-conductivity of the problem, averaged to the
nodes) to an approximation of K^-1 r; flexible CG (``'type of preconditioner': 'learned'``)
applies it at every iteration, and the true float64 Newton residual judges every solve.
Every convolution, pooling, upsampling and gradient runs in this package's own BF16
tensor-core kernels (include/autopdex_gb300_nn.h); PyTorch holds the float32 master
weights and runs the Adam update.  Training pairs (r, K^-1 r) come from the plain float64
Jacobi-PCG solver of this backend on seeded random-conductivity problems.

This part has no counterpart in AutoPDEx.
"""
import ctypes as C
import math
import os

import numpy as np
import torch

from . import _native as N

C_HID = 32
C_IN = 16
C_OUT = 16
# (name, c1, c2, cout, relu): encoder (two convs per level, 2x2 average pooling between levels),
# bottleneck, decoder (nearest upsampling, concatenation with the encoder output of the level)
LAYERS = [("e0a", 16, 0, 32, 1), ("e0b", 32, 0, 32, 1), ("e1a", 32, 0, 32, 1), ("e1b", 32, 0, 32, 1),
          ("e2a", 32, 0, 32, 1), ("e2b", 32, 0, 32, 1), ("b3a", 32, 0, 32, 1), ("b3b", 32, 0, 32, 1),
          ("d2a", 32, 32, 32, 1), ("d2b", 32, 0, 32, 1), ("d1a", 32, 32, 32, 1), ("d1b", 32, 0, 32, 1),
          ("d0a", 32, 32, 32, 1), ("d0b", 32, 0, 32, 1), ("out", 32, 0, 16, 0)]
WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def padded(n):
    """Grid extent padded to a multiple of 8 (three 2x poolings)."""
    return (n + 7) // 8 * 8


class UNet:
    def __init__(self, device="cuda", seed=0, params=None):
        self.lib = N.load()
        self.device = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        self.w, self.b = {}, {}
        for name, c1, c2, co, relu in LAYERS:
            cin = c1 + c2
            std = math.sqrt(2.0 / (9 * cin)) if relu else math.sqrt(1.0 / (9 * cin))
            w = torch.randn(co, cin, 3, 3, generator=g) * std
            if name == "e0a":
                w[:, 2:] = 0.0  # channels 2..15 of the input are padding
            self.w[name] = w.to(self.device)
            self.b[name] = torch.zeros(co, device=self.device)
        if params is not None:
            self.load_state(params)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.pack()

    # ---- parameters -------------------------------------------------------------------
    def state(self):
        return {f"{k}.w": v.detach().cpu().numpy() for k, v in self.w.items()} | \
               {f"{k}.b": v.detach().cpu().numpy() for k, v in self.b.items()}

    def load_state(self, st):
        for k in self.w:
            self.w[k] = torch.as_tensor(np.asarray(st[f"{k}.w"]), dtype=torch.float32, device=self.device)
            self.b[k] = torch.as_tensor(np.asarray(st[f"{k}.b"]), dtype=torch.float32, device=self.device)

    def save(self, path):
        np.savez(path, **self.state())

    @classmethod
    def load(cls, path, device="cuda"):
        return cls(device=device, params=dict(np.load(path)))

    def parameters(self):
        return [self.w[k] for k, *_ in LAYERS] + [self.b[k] for k, *_ in LAYERS]

    def pack(self):
        """bf16 operand images of every layer (forward and input-gradient)."""
        s = self._stream()
        self.img_f, self.img_b = {}, {}
        for name, c1, c2, co, relu in LAYERS:
            cin = c1 + c2
            w = self.w[name].contiguous()
            f = torch.empty(co * cin * 9, dtype=torch.bfloat16, device=self.device)
            bimg = torch.empty(co * cin * 9, dtype=torch.bfloat16, device=self.device)
            self._ok("agx_nn_pack_weights", self.lib.agx_nn_pack_weights(_p(w), co, cin, 0, _p(f), s))
            self._ok("agx_nn_pack_weights", self.lib.agx_nn_pack_weights(_p(w), co, cin, 1, _p(bimg), s))
            self.img_f[name], self.img_b[name] = f, bimg

    # ---- helpers ------------------------------------------------------------------------
    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    @staticmethod
    def _ok(fn, rc):
        if rc != 0:
            raise RuntimeError(f"{fn} failed with status {rc}")

    def _act(self, B, H, W, c):
        return torch.empty((B, H, W, c), dtype=torch.bfloat16, device=self.device)

    def _conv(self, name, x1, x2, B, H, W):
        _, c1, c2, co, relu = next(l for l in LAYERS if l[0] == name)
        out = self._act(B, H, W, co)
        rc = self.lib.agx_nn_conv3x3(_p(x1), _p(x2), c1, c2, _p(self.img_f[name]), _p(self.b[name]), _p(out), None,
                                     co, co, relu, B, H, W, _p(self.err), self._stream())
        self._ok("agx_nn_conv3x3", rc)
        return out

    def _pool(self, x, B, H, W, c):
        out = self._act(B, H // 2, W // 2, c)
        self._ok("agx_nn_pool2", self.lib.agx_nn_pool2(_p(x), _p(out), B, H, W, c, 0, self._stream()))
        return out

    def _up(self, x, B, H, W, c):
        out = self._act(B, 2 * H, 2 * W, c)
        self._ok("agx_nn_upsample2", self.lib.agx_nn_upsample2(_p(x), _p(out), B, H, W, c, 0, self._stream()))
        return out

    # ---- forward / backward -------------------------------------------------------------
    def forward(self, x, keep=False):
        """x: (B, H, W, 16) bf16 with H, W multiples of 8 -> (B, H, W, 16) bf16."""
        B, H, W, _ = x.shape
        a = {"x": x}
        a["e0a"] = self._conv("e0a", x, None, B, H, W)
        a["e0b"] = self._conv("e0b", a["e0a"], None, B, H, W)
        a["p0"] = self._pool(a["e0b"], B, H, W, C_HID)
        a["e1a"] = self._conv("e1a", a["p0"], None, B, H // 2, W // 2)
        a["e1b"] = self._conv("e1b", a["e1a"], None, B, H // 2, W // 2)
        a["p1"] = self._pool(a["e1b"], B, H // 2, W // 2, C_HID)
        a["e2a"] = self._conv("e2a", a["p1"], None, B, H // 4, W // 4)
        a["e2b"] = self._conv("e2b", a["e2a"], None, B, H // 4, W // 4)
        a["p2"] = self._pool(a["e2b"], B, H // 4, W // 4, C_HID)
        a["b3a"] = self._conv("b3a", a["p2"], None, B, H // 8, W // 8)
        a["b3b"] = self._conv("b3b", a["b3a"], None, B, H // 8, W // 8)
        a["u2"] = self._up(a["b3b"], B, H // 8, W // 8, C_HID)
        a["d2a"] = self._conv("d2a", a["u2"], a["e2b"], B, H // 4, W // 4)
        a["d2b"] = self._conv("d2b", a["d2a"], None, B, H // 4, W // 4)
        a["u1"] = self._up(a["d2b"], B, H // 4, W // 4, C_HID)
        a["d1a"] = self._conv("d1a", a["u1"], a["e1b"], B, H // 2, W // 2)
        a["d1b"] = self._conv("d1b", a["d1a"], None, B, H // 2, W // 2)
        a["u0"] = self._up(a["d1b"], B, H // 2, W // 2, C_HID)
        a["d0a"] = self._conv("d0a", a["u0"], a["e0b"], B, H, W)
        a["d0b"] = self._conv("d0b", a["d0a"], None, B, H, W)
        out = self._conv("out", a["d0b"], None, B, H, W)
        return (out, a) if keep else out

    def _layer_backward(self, name, g, x1, x2, y, B, H, W, need_input_grad=True):
        """g: gradient w.r.t. the layer output y (modified in place by the ReLU mask)."""
        _, c1, c2, co, relu = next(l for l in LAYERS if l[0] == name)
        s = self._stream()
        if relu:
            self._ok("agx_nn_relu_backward", self.lib.agx_nn_relu_backward(_p(g), _p(y), g.numel(), s))
        P = B * H * W
        self._ok("agx_nn_bias_grad", self.lib.agx_nn_bias_grad(_p(g), P, co, _p(self.gb[name]), s))
        rows = torch.zeros(9 * (c1 + c2) * co, dtype=torch.float32, device=self.device)
        self._ok("agx_nn_wgrad3x3", self.lib.agx_nn_wgrad3x3(_p(x1), _p(x2), c1, c2, _p(g), co, _p(rows), B, H, W,
                                                           _p(self.err), s))
        dw = torch.empty_like(self.w[name])
        self._ok("agx_nn_unpack_wgrad", self.lib.agx_nn_unpack_wgrad(_p(rows), co, c1 + c2, _p(dw), s))
        self.gw[name] += dw
        if not need_input_grad:
            return None, None
        d1 = self._act(B, H, W, c1)
        d2 = self._act(B, H, W, c2) if c2 else None
        rc = self.lib.agx_nn_conv3x3(_p(g), None, co, 0, _p(self.img_b[name]), None, _p(d1), _p(d2), c1, c1 + c2, 0,
                                     B, H, W, _p(self.err), s)
        self._ok("agx_nn_conv3x3 (input gradient)", rc)
        return d1, d2

    def backward(self, gout, a):
        """Accumulates parameter gradients into self.gw / self.gb for d(loss)/d(out) = gout."""
        B, H, W, _ = gout.shape
        s = self._stream()
        self.gw = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.gb = {k: torch.zeros_like(v) for k, v in self.b.items()}

        def upb(g, h, w):  # adjoint of upsampling to (h, w) -> coarse
            out = self._act(B, h // 2, w // 2, C_HID)
            self._ok("agx_nn_upsample2", self.lib.agx_nn_upsample2(_p(g), _p(out), B, h // 2, w // 2, C_HID, 1, s))
            return out

        def poolb(g, h, w):  # adjoint of pooling from (h, w)
            out = self._act(B, h, w, C_HID)
            self._ok("agx_nn_pool2", self.lib.agx_nn_pool2(_p(g), _p(out), B, h, w, C_HID, 1, s))
            return out

        def add(x, y):
            self._ok("agx_nn_add", self.lib.agx_nn_add(_p(x), _p(y), x.numel(), s))
            return x

        g = gout.clone()
        g, _ = self._layer_backward("out", g, a["d0b"], None, None, B, H, W)
        g, _ = self._layer_backward("d0b", g, a["d0a"], None, a["d0b"], B, H, W)
        g_u0, g_s0 = self._layer_backward("d0a", g, a["u0"], a["e0b"], a["d0a"], B, H, W)
        g = upb(g_u0, H, W)
        g, _ = self._layer_backward("d1b", g, a["d1a"], None, a["d1b"], B, H // 2, W // 2)
        g_u1, g_s1 = self._layer_backward("d1a", g, a["u1"], a["e1b"], a["d1a"], B, H // 2, W // 2)
        g = upb(g_u1, H // 2, W // 2)
        g, _ = self._layer_backward("d2b", g, a["d2a"], None, a["d2b"], B, H // 4, W // 4)
        g_u2, g_s2 = self._layer_backward("d2a", g, a["u2"], a["e2b"], a["d2a"], B, H // 4, W // 4)
        g = upb(g_u2, H // 4, W // 4)
        g, _ = self._layer_backward("b3b", g, a["b3a"], None, a["b3b"], B, H // 8, W // 8)
        g, _ = self._layer_backward("b3a", g, a["p2"], None, a["b3a"], B, H // 8, W // 8)
        g = add(poolb(g, H // 4, W // 4), g_s2)
        g, _ = self._layer_backward("e2b", g, a["e2a"], None, a["e2b"], B, H // 4, W // 4)
        g, _ = self._layer_backward("e2a", g, a["p1"], None, a["e2a"], B, H // 4, W // 4)
        g = add(poolb(g, H // 2, W // 2), g_s1)
        g, _ = self._layer_backward("e1b", g, a["e1a"], None, a["e1b"], B, H // 2, W // 2)
        g, _ = self._layer_backward("e1a", g, a["p0"], None, a["e1a"], B, H // 2, W // 2)
        g = add(poolb(g, H, W), g_s0)
        g, _ = self._layer_backward("e0b", g, a["e0a"], None, a["e0b"], B, H, W)
        self._layer_backward("e0a", g, a["x"], None, a["e0a"], B, H, W, need_input_grad=False)
        return self.gw, self.gb

    def check(self):
        if int(self.err.item()) != 0:
            raise RuntimeError("a tensor-core kernel timed out waiting for its MMA")


# ---- grids, features, data ---------------------------------------------------------------
def node_log_conductivity(k_elem, nx, ny):
    """log k averaged from the elements to the nodes of an nx x ny structured quad mesh
    (element (i, j) -> i * ny + j, node (i, j) -> i * (ny + 1) + j)."""
    lk = np.log(np.asarray(k_elem, dtype=np.float64)).reshape(nx, ny)
    s = np.zeros((nx + 1, ny + 1))
    c = np.zeros((nx + 1, ny + 1))
    for di in (0, 1):
        for dj in (0, 1):
            s[di:di + nx, dj:dj + ny] += lk
            c[di:di + nx, dj:dj + ny] += 1
    return (s / c).reshape(-1).astype(np.float32)


def to_image(lib, r, aux, Hn, Wn, normalize=True, out=None, scale=None, stream=None):
    Hp, Wp = padded(Hn), padded(Wn)
    dev = r.device
    img = out if out is not None else torch.empty((1, Hp, Wp, C_IN), dtype=torch.bfloat16, device=dev)
    sc = scale if scale is not None else torch.empty(1, dtype=torch.float32, device=dev)
    st = stream or C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rc = lib.agx_nn_grid_from_vector(_p(r), _p(aux), Hn, Wn, Hp, Wp, 1 if normalize else 0, _p(sc), _p(img), st)
    if rc != 0:
        raise RuntimeError("agx_nn_grid_from_vector failed")
    return img, sc


def make_training_set(n_problems, n=256, rhs_per_problem=2, seed0=0, krylov_tol=1e-6, verbose=False):
    """(r, aux, e) triples from the plain float64 Jacobi-PCG solver of this backend on
    heat-conduction problems with seeded random conductivity (config-4 family at n x n)."""
    from . import configs
    from ._problem import get_problem
    w = configs.heat_grf(n=n, seed=seed0)
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    mask = torch.as_tensor(prob.mask.astype(bool), device=prob.device)
    rng = np.random.default_rng(seed0 + 12345)
    R, A, E = [], [], []
    opts = N.SolveOpts()
    opts.method, opts.rtol, opts.atol, opts.maxiter, opts.check_every = N.AGX_PCG, krylov_tol, 0.0, 200000, 64
    x0 = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
    for i in range(n_problems):
        k = np.exp(configs.gaussian_random_field(n, seed=seed0 + i)).reshape(-1)
        w.settings["conductivity"] = k
        prob.update_models(w.settings)
        prob._call("agx_assemble", C.c_void_p(x0.data_ptr()), None, N.AGX_F64)
        aux = torch.as_tensor(node_log_conductivity(k, n, n), device=prob.device)
        for j in range(rhs_per_problem):
            r = _random_rhs(rng, n + 1, prob.device) if j else torch.ones(prob.n_dofs, dtype=torch.float64,
                                                                         device=prob.device)
            r = torch.where(mask, torch.zeros_like(r), r)
            e = torch.zeros_like(r)
            info = N.SolveInfo()
            prob._call("agx_solve", C.c_void_p(r.data_ptr()), C.c_void_p(e.data_ptr()), C.byref(opts), C.byref(info))
            R.append(r.float())
            A.append(aux)
            E.append(e.float())
        if verbose and i % 100 == 0:
            print(f"training problem {i}: {info.iterations} CG iterations")
    return torch.stack(R), torch.stack(A), torch.stack(E)


def _random_rhs(rng, m, device):
    """Smooth-plus-rough random field on an m x m node grid."""
    f = np.zeros((m, m))
    for scale in (4, 16, 64):
        c = rng.standard_normal((scale, scale))
        f += np.kron(c, np.ones((m // scale + 1, m // scale + 1)))[:m, :m] / math.sqrt(scale)
    f += 0.1 * rng.standard_normal((m, m))
    return torch.as_tensor(f.reshape(-1), dtype=torch.float64, device=device)


def train(net, R, A, E, n, steps=2000, batch=16, lr=2e-3, seed=0, verbose=False):
    """Adam on the scale-invariant loss ||z - e~||^2 / ||e~||^2 with e~ = e / rms(e),
    z = channel 0 of the network output on the node grid."""
    lib = net.lib
    Hn = Wn = n + 1
    Hp, Wp = padded(Hn), padded(Wn)
    params = net.parameters()
    opt = torch.optim.Adam(params, lr=lr)
    gen = torch.Generator().manual_seed(seed)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    losses = []
    x = torch.empty((batch, Hp, Wp, C_IN), dtype=torch.bfloat16, device=net.device)
    sc = torch.empty(batch, dtype=torch.float32, device=net.device)
    for step in range(steps):
        idx = torch.randint(0, R.shape[0], (batch,), generator=gen)
        for b, i in enumerate(idx.tolist()):
            to_image(lib, R[i], A[i], Hn, Wn, True, out=x[b:b + 1], scale=sc[b:b + 1], stream=stream)
        out, acts = net.forward(x, keep=True)
        z = out[..., 0].float()[:, :Hn, :Wn].reshape(batch, -1)
        e = E[idx]
        et = e / e.pow(2).mean(dim=1, keepdim=True).sqrt().clamp_min(1e-30)
        diff = z - et
        loss = (diff.pow(2).sum(dim=1) / et.pow(2).sum(dim=1)).mean()
        g = torch.zeros_like(out, dtype=torch.float32)
        g[:, :Hn, :Wn, 0] = (2.0 * diff / et.pow(2).sum(dim=1, keepdim=True) / batch).reshape(batch, Hn, Wn)
        gw, gb = net.backward(g.to(torch.bfloat16), acts)
        for name, *_ in LAYERS:
            net.w[name].grad = gw[name]
            net.b[name].grad = gb[name]
        opt.step()
        opt.zero_grad(set_to_none=True)
        with torch.no_grad():
            net.w["e0a"][:, 2:] = 0.0
        net.pack()
        losses.append(float(loss))
        if verbose and step % 100 == 0:
            print(f"step {step}: loss {losses[-1]:.4f}")
    net.check()
    return losses


# ---- preconditioner for flexible CG ----------------------------------------------------------
class GridPreconditioner:
    """z = net(r) on the node grid of an nx x ny structured quad mesh (scalar field)."""

    def __init__(self, net, nx, ny, k_elem):
        self.net = net
        self.nx, self.ny = nx, ny
        self.Hn, self.Wn = nx + 1, ny + 1
        self.Hp, self.Wp = padded(self.Hn), padded(self.Wn)
        self.aux = torch.as_tensor(node_log_conductivity(k_elem, nx, ny), device=net.device)
        self.img = torch.empty((1, self.Hp, self.Wp, C_IN), dtype=torch.bfloat16, device=net.device)
        self.scale = torch.empty(1, dtype=torch.float32, device=net.device)
        self.applications = 0

    def apply_ptr(self, r_ptr, z_ptr, n, stream):
        lib = self.net.lib
        rc = lib.agx_nn_grid_from_vector(C.c_void_p(r_ptr), _p(self.aux), self.Hn, self.Wn, self.Hp, self.Wp, 1,
                                         _p(self.scale), _p(self.img), C.c_void_p(stream))
        if rc != 0:
            return rc
        out = self.net.forward(self.img)
        rc = lib.agx_nn_vector_from_grid(_p(out), C_OUT, self.Hn, self.Wn, self.Wp, C.c_void_p(z_ptr),
                                         C.c_void_p(stream))
        self.applications += 1
        return rc

    def callback(self, prob):
        if prob.n_dofs != self.Hn * self.Wn:
            raise ValueError("the learned preconditioner was built for another grid")

        def fn(user, r, z, n, stream):
            try:
                return self.apply_ptr(r, z, n, stream)
            except Exception:  # noqa: BLE001 -- report through the status code
                return -1
        return N.PRECOND_FN(fn)
