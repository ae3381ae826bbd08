"""Learned preconditioner: a 4-level, 32-channel convolutional U-Net on the node grid.

The network maps a residual r (and the log-conductivity of the problem, averaged to the
nodes) to a correction y whose energy-optimal multiple approximates K^-1 r after damped
Jacobi smoothing; flexible CG (``'type of preconditioner': 'learned'``) applies it at every
iteration in a symmetric two-level form, and the true float64 Newton residual judges every
solve.
Every convolution, pooling, upsampling and gradient runs in this package's own BF16
tensor-core kernels (include/autopdex_gb300_nn.h); PyTorch holds the float32 master
weights and runs the Adam update.  Training pairs (residual, error) come from the iterates of
the plain float64 Jacobi-PCG solver of this backend on seeded random-conductivity problems,
and the loss is the fraction of the error energy the correction leaves.

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
POOL = 4  # 4 x 4 average pooling between levels: the coarsest level of a 320 x 320 grid is 5 x 5
# (name, c1, c2, cout, relu): encoder (two convs per level, POOL x POOL average pooling between
# levels), bottleneck, decoder (nearest POOL x upsampling, concatenation with the encoder output
# of the level)
LAYERS = [("e0a", 16, 0, 32, 1), ("e0b", 32, 0, 32, 1), ("e1a", 32, 0, 32, 1), ("e1b", 32, 0, 32, 1),
          ("e2a", 32, 0, 32, 1), ("e2b", 32, 0, 32, 1), ("b3a", 32, 0, 32, 1), ("b3b", 32, 0, 32, 1),
          ("d2a", 32, 32, 32, 1), ("d2b", 32, 0, 32, 1), ("d1a", 32, 32, 32, 1), ("d1b", 32, 0, 32, 1),
          ("d0a", 32, 32, 32, 1), ("d0b", 32, 0, 32, 1), ("out", 32, 0, 16, 0)]
WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def padded(n):
    """Grid extent padded to a multiple of POOL^3 (three poolings)."""
    m = POOL ** 3
    return (n + m - 1) // m * m


class UNet:
    """``n_in``: input channels in use (the field's components plus auxiliary features; the
    rest of the 16 are padding and their weights stay zero).

    The class describes the 2-D network (NHWC tensors, 3x3 convolutions, POOL x POOL pooling);
    :class:`UNet3D` changes the class attributes below for the 3-D one."""

    dims = 2          # spatial dimensions of the tensors
    layers = LAYERS
    pool = POOL
    hid = C_HID

    def __init__(self, device="cuda", seed=0, params=None, n_in=2):
        self.lib = N.load()
        self.device = torch.device(device)
        if params is not None and "meta.n_in" in params:
            n_in = int(np.asarray(params["meta.n_in"]))
        self.n_in = n_in
        g = torch.Generator().manual_seed(seed)
        self.w, self.b = {}, {}
        taps = 3 ** self.dims
        for name, c1, c2, co, relu in self.layers:
            cin = c1 + c2
            std = math.sqrt(2.0 / (taps * cin)) if relu else math.sqrt(1.0 / (taps * cin))
            w = torch.randn(co, cin, *(3,) * self.dims, generator=g) * std
            if name == "e0a":
                w[:, n_in:] = 0.0  # channels n_in..15 of the input are padding
            self.w[name] = w.to(self.device)
            self.b[name] = torch.zeros(co, device=self.device)
        if params is not None:
            self.load_state(params)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.launches = 0  # kernels this network has launched (forward and backward passes)
        self._s, self._arena = None, None
        self.loader = {}  # layer name -> halo loader of its forward convolution (autotune)
        self.pack()

    # ---- parameters -------------------------------------------------------------------
    def state(self):
        return {f"{k}.w": v.detach().cpu().numpy() for k, v in self.w.items()} | \
               {f"{k}.b": v.detach().cpu().numpy() for k, v in self.b.items()} | {"meta.n_in": np.int64(self.n_in)}

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
        return [self.w[k] for k, *_ in self.layers] + [self.b[k] for k, *_ in self.layers]

    def _layer(self, name):
        return next(l for l in self.layers if l[0] == name)

    def pack(self):
        """bf16 operand images of every layer (forward and input-gradient)."""
        # convolutions may prefetch weights ahead of their predecessor (AGX_NN_CONST_WEIGHTS)
        # only once a synchronisation has followed the packing (GridPreconditioner sets it)
        self.const_weights = False
        s = self._stream()
        fn = "agx_nn_pack_weights" if self.dims == 2 else "agx_nn_pack_weights3d"
        pack = getattr(self.lib, fn)
        taps = 3 ** self.dims
        self.img_f, self.img_b = {}, {}
        for name, c1, c2, co, relu in self.layers:
            cin = c1 + c2
            w = self.w[name].contiguous()
            f = torch.empty(co * cin * taps, dtype=torch.bfloat16, device=self.device)
            bimg = torch.empty(co * cin * taps, dtype=torch.bfloat16, device=self.device)
            self._ok(fn, pack(_p(w), co, cin, 0, _p(f), s))
            self._ok(fn, pack(_p(w), co, cin, 1, _p(bimg), s))
            self.img_f[name], self.img_b[name] = f, bimg

    # ---- helpers ------------------------------------------------------------------------
    def _stream(self):
        if self._s is not None:
            return self._s
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    @staticmethod
    def _ok(fn, rc):
        if rc != 0:
            raise RuntimeError(f"{fn} failed with status {rc}")

    def _act(self, B, S, c, key=None):
        """Activation buffer (B, *S, c): from the arena when one is active (allocated on first use)."""
        shape = (B, *S, c)
        if self._arena is not None and key is not None:
            t = self._arena.get(key)
            if t is None or tuple(t.shape) != shape:
                t = torch.empty(shape, dtype=torch.bfloat16, device=self.device)
                self._arena[key] = t
            return t
        return torch.empty(shape, dtype=torch.bfloat16, device=self.device)

    def _convolve(self, x1, x2, c1, c2, wimg, bias, out1, out2, split, cout, flags, B, S, s):
        if self.dims == 2:
            return self.lib.agx_nn_conv3x3(_p(x1), _p(x2), c1, c2, _p(wimg), _p(bias), _p(out1), _p(out2), split, cout,
                                           flags, B, *S, _p(self.err), s)
        return self.lib.agx_nn_conv3x3x3(_p(x1), _p(x2), c1, c2, _p(wimg), _p(bias), _p(out1), _p(out2), split, cout,
                                         flags, B, *S, _p(self.err), s)

    def _conv(self, name, x1, x2, B, S, loader=None):
        _, c1, c2, co, relu = self._layer(name)
        out = self._act(B, S, co, name)
        flags = relu | (N.AGX_NN_CONST_WEIGHTS if self.const_weights and self._arena is not None else 0)
        lo = self.loader.get(name) if loader is None else loader
        if lo is not None:
            flags |= N.AGX_NN_LOADER(lo)
        rc = self._convolve(x1, x2, c1, c2, self.img_f[name], self.b[name], out, None, co, co, flags, B, S,
                            self._stream())
        self._ok("convolution", rc)
        self.launches += 1
        return out

    def _transfer(self, up, x, out, B, S, c, backward, s):
        """Pooling (up False) or upsampling (up True) of x at spatial size S, one launch."""
        if self.dims == 2:
            fn = self.lib.agx_nn_upsample if up else self.lib.agx_nn_pool
        else:
            fn = self.lib.agx_nn_upsample3d if up else self.lib.agx_nn_pool3d
        self._ok("pooling" if not up else "upsampling", fn(_p(x), _p(out), B, *S, c, self.pool, backward, s))

    def _pool(self, x, B, S, c, key):
        """Average pooling by self.pool in every dimension, one launch."""
        out = self._act(B, tuple(v // self.pool for v in S), c, f"{key}.{self.pool}")
        self._transfer(False, x, out, B, S, c, 0, self._stream())
        self.launches += 1
        return out

    def _up(self, x, B, S, c, key):
        """Nearest upsampling by self.pool of an image of spatial size S, one launch."""
        out = self._act(B, tuple(self.pool * v for v in S), c, f"{key}.{self.pool}")
        self._transfer(True, x, out, B, S, c, 0, self._stream())
        self.launches += 1
        return out

    # ---- forward / backward -------------------------------------------------------------
    def forward(self, x, keep=False, stream=None, arena=None):
        """x: (B, *S, 16) bf16 with every extent of S a multiple of pool^3 -> (B, *S, 16) bf16.

        ``stream``: launch on this CUDA stream (a c_void_p) instead of torch's current one;
        ``arena``: a dict of activation buffers reused across calls (no allocation once warm)."""
        self._s, self._arena = stream, arena
        try:
            return self._forward(x, keep)
        finally:
            self._s, self._arena = None, None

    def _level(self, S0, k):
        return tuple(v // self.pool ** k for v in S0)

    def _forward(self, x, keep):
        B, S0 = x.shape[0], tuple(x.shape[1:-1])
        L = [self._level(S0, k) for k in range(4)]
        h = self.hid
        a = {"x": x}
        a["e0a"] = self._conv("e0a", x, None, B, L[0])
        a["e0b"] = self._conv("e0b", a["e0a"], None, B, L[0])
        a["p0"] = self._pool(a["e0b"], B, L[0], h, "p0")
        a["e1a"] = self._conv("e1a", a["p0"], None, B, L[1])
        a["e1b"] = self._conv("e1b", a["e1a"], None, B, L[1])
        a["p1"] = self._pool(a["e1b"], B, L[1], h, "p1")
        a["e2a"] = self._conv("e2a", a["p1"], None, B, L[2])
        a["e2b"] = self._conv("e2b", a["e2a"], None, B, L[2])
        a["p2"] = self._pool(a["e2b"], B, L[2], h, "p2")
        a["b3a"] = self._conv("b3a", a["p2"], None, B, L[3])
        a["b3b"] = self._conv("b3b", a["b3a"], None, B, L[3])
        a["u2"] = self._up(a["b3b"], B, L[3], h, "u2")
        a["d2a"] = self._conv("d2a", a["u2"], a["e2b"], B, L[2])
        a["d2b"] = self._conv("d2b", a["d2a"], None, B, L[2])
        a["u1"] = self._up(a["d2b"], B, L[2], h, "u1")
        a["d1a"] = self._conv("d1a", a["u1"], a["e1b"], B, L[1])
        a["d1b"] = self._conv("d1b", a["d1a"], None, B, L[1])
        a["u0"] = self._up(a["d1b"], B, L[1], h, "u0")
        a["d0a"] = self._conv("d0a", a["u0"], a["e0b"], B, L[0])
        a["d0b"] = self._conv("d0b", a["d0a"], None, B, L[0])
        out = self._conv("out", a["d0b"], None, B, L[0])
        return (out, a) if keep else out

    def _layer_backward(self, name, g, x1, x2, y, B, S, need_input_grad=True):
        """g: gradient w.r.t. the layer output y (modified in place by the ReLU mask)."""
        _, c1, c2, co, relu = self._layer(name)
        s = self._stream()
        if relu:
            self._ok("agx_nn_relu_backward", self.lib.agx_nn_relu_backward(_p(g), _p(y), g.numel(), s))
        P = B * math.prod(S)
        self._ok("agx_nn_bias_grad", self.lib.agx_nn_bias_grad(_p(g), P, co, _p(self.gb[name]), s))
        taps = 3 ** self.dims
        rows = torch.zeros(taps * (c1 + c2) * co, dtype=torch.float32, device=self.device)
        dw = torch.empty_like(self.w[name])
        if self.dims == 2:
            rc = self.lib.agx_nn_wgrad3x3(_p(x1), _p(x2), c1, c2, _p(g), co, _p(rows), B, *S, _p(self.err), s)
            self._ok("agx_nn_wgrad3x3", rc)
            self._ok("agx_nn_unpack_wgrad", self.lib.agx_nn_unpack_wgrad(_p(rows), co, c1 + c2, _p(dw), s))
        else:
            rc = self.lib.agx_nn_wgrad3x3x3(_p(x1), _p(x2), c1, c2, _p(g), co, _p(rows), B, *S, _p(self.err), s)
            self._ok("agx_nn_wgrad3x3x3", rc)
            self._ok("agx_nn_unpack_wgrad3d", self.lib.agx_nn_unpack_wgrad3d(_p(rows), co, c1 + c2, _p(dw), s))
        self.gw[name] += dw
        if not need_input_grad:
            return None, None
        d1 = self._act(B, S, c1)
        d2 = self._act(B, S, c2) if c2 else None
        rc = self._convolve(g, None, co, 0, self.img_b[name], None, d1, d2, c1, c1 + c2, 0, B, S, s)
        self._ok("convolution (input gradient)", rc)
        return d1, d2

    def backward(self, gout, a):
        """Accumulates parameter gradients into self.gw / self.gb for d(loss)/d(out) = gout."""
        B, S0 = gout.shape[0], tuple(gout.shape[1:-1])
        L = [self._level(S0, k) for k in range(4)]
        h = self.hid
        s = self._stream()
        self.gw = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.gb = {k: torch.zeros_like(v) for k, v in self.b.items()}

        def upb(g, k):  # adjoint of the upsampling from level k + 1 to level k: -> level k + 1
            out = self._act(B, L[k + 1], h)
            self._transfer(True, g, out, B, L[k + 1], h, 1, s)
            return out

        def poolb(g, k):  # adjoint of the pooling from level k to level k + 1: -> level k
            out = self._act(B, L[k], h)
            self._transfer(False, g, out, B, L[k], h, 1, s)
            return out

        def add(x, y):
            self._ok("agx_nn_add", self.lib.agx_nn_add(_p(x), _p(y), x.numel(), s))
            return x

        g = gout.clone()
        g, _ = self._layer_backward("out", g, a["d0b"], None, None, B, L[0])
        g, _ = self._layer_backward("d0b", g, a["d0a"], None, a["d0b"], B, L[0])
        g_u0, g_s0 = self._layer_backward("d0a", g, a["u0"], a["e0b"], a["d0a"], B, L[0])
        g = upb(g_u0, 0)
        g, _ = self._layer_backward("d1b", g, a["d1a"], None, a["d1b"], B, L[1])
        g_u1, g_s1 = self._layer_backward("d1a", g, a["u1"], a["e1b"], a["d1a"], B, L[1])
        g = upb(g_u1, 1)
        g, _ = self._layer_backward("d2b", g, a["d2a"], None, a["d2b"], B, L[2])
        g_u2, g_s2 = self._layer_backward("d2a", g, a["u2"], a["e2b"], a["d2a"], B, L[2])
        g = upb(g_u2, 2)
        g, _ = self._layer_backward("b3b", g, a["b3a"], None, a["b3b"], B, L[3])
        g, _ = self._layer_backward("b3a", g, a["p2"], None, a["b3a"], B, L[3])
        g = add(poolb(g, 2), g_s2)
        g, _ = self._layer_backward("e2b", g, a["e2a"], None, a["e2b"], B, L[2])
        g, _ = self._layer_backward("e2a", g, a["p1"], None, a["e2a"], B, L[2])
        g = add(poolb(g, 1), g_s1)
        g, _ = self._layer_backward("e1b", g, a["e1a"], None, a["e1b"], B, L[1])
        g, _ = self._layer_backward("e1a", g, a["p0"], None, a["e1a"], B, L[1])
        g = add(poolb(g, 0), g_s0)
        g, _ = self._layer_backward("e0b", g, a["e0a"], None, a["e0b"], B, L[0])
        self._layer_backward("e0a", g, a["x"], None, a["e0a"], B, L[0], need_input_grad=False)
        return self.gw, self.gb

    def check(self):
        if int(self.err.item()) != 0:
            raise RuntimeError("a tensor-core kernel timed out waiting for its MMA")

    def autotune(self, x, reps=50, loaders=(0, 1, 2), gain=0.01):
        """Chooses each layer's halo loader (agx_nn_conv3x3's kernel variant: cp.async loop,
        tensor-copy loop, warp-specialised; identical outputs) by what the preconditioner runs: the
        whole forward pass captured into a CUDA graph (programmatic launches overlapping as in the
        FCG graphs) and replayed reps times under CUDA events.  Coordinate descent from the
        default choice (warm-up first): for every layer in turn each variant is tried with the
        others fixed and kept when the pass gets faster by more than `gain`.  Returns
        {"us_per_pass": (before, after), layer: (loader, {loader: us per pass})}.  2-D networks
        only (the 3-D convolution has one variant)."""
        if self.dims != 2:
            return {}
        B, S0 = x.shape[0], tuple(x.shape[1:-1])
        assign = {}
        for name, c1, c2, co, relu in self.layers:
            lv = {"e0": 0, "e1": 1, "e2": 2, "b3": 3, "d2": 2, "d1": 1, "d0": 0, "ou": 0}[name[:2]]
            H, W = self._level(S0, lv)
            assign[name] = 2 if (c2 > 0 and H * W >= 128 * 128) else 1  # the process-wide default
        stream = torch.cuda.Stream(self.device)
        sp = C.c_void_p(stream.cuda_stream)
        arena = {}
        saved_cw, saved_loader = self.const_weights, dict(self.loader)

        def pass_us(trial):
            self.loader = dict(trial)
            with torch.cuda.stream(stream):
                self.forward(x, stream=sp, arena=arena)  # first launches and activations outside the capture
            stream.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                self.forward(x, stream=sp, arena=arena)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                for _ in range(3):
                    g.replay()
                e0.record()
                for _ in range(reps):
                    g.replay()
                e1.record()
            e1.synchronize()
            return e0.elapsed_time(e1) * 1e3 / reps

        chosen = {}
        try:
            self.const_weights = False
            best = pass_us(assign)
            first = best
            for name, *_ in self.layers:
                times = {assign[name]: best}
                for lo in loaders:
                    if lo == assign[name]:
                        continue
                    t = pass_us(dict(assign, **{name: lo}))
                    times[lo] = t
                    if t < best * (1.0 - gain):
                        best, assign[name] = t, lo
                chosen[name] = (assign[name], times)
        except Exception:
            self.loader = saved_loader
            raise
        finally:
            self.const_weights = saved_cw
        self.loader = dict(assign)
        self.check()
        chosen["us_per_pass"] = (first, best)
        return chosen


# The 3-D network: 16 channels at every level, 3x3x3 convolutions, 2 x 2 x 2 average pooling
# (the coarsest level of a 40^3 grid is 5^3), the same encoder-decoder graph as the 2-D one
LAYERS3 = [("e0a", 16, 0, 16, 1), ("e0b", 16, 0, 16, 1), ("e1a", 16, 0, 16, 1), ("e1b", 16, 0, 16, 1),
           ("e2a", 16, 0, 16, 1), ("e2b", 16, 0, 16, 1), ("b3a", 16, 0, 16, 1), ("b3b", 16, 0, 16, 1),
           ("d2a", 16, 16, 16, 1), ("d2b", 16, 0, 16, 1), ("d1a", 16, 16, 16, 1), ("d1b", 16, 0, 16, 1),
           ("d0a", 16, 16, 16, 1), ("d0b", 16, 0, 16, 1), ("out", 16, 0, 16, 0)]
POOL3 = 2


class UNet3D(UNet):
    """The 3-D U-Net on NDHWC tensors (include/autopdex_gb300_nn.h, the 3-D part)."""

    dims = 3
    layers = LAYERS3
    pool = POOL3
    hid = 16


def padded3(n):
    """Grid extent padded to a multiple of POOL3^3 (three poolings)."""
    m = POOL3 ** 3
    return (n + m - 1) // m * m


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


def to_image(lib, r, aux, Hn, Wn, normalize=True, out=None, scale=None, stream=None, nd=1, naux=None):
    """Network input image of a node field r (nd components per node, node-major) and the
    per-node auxiliary features aux (naux per node; 1 when not given)."""
    Hp, Wp = padded(Hn), padded(Wn)
    dev = r.device
    img = out if out is not None else torch.empty((1, Hp, Wp, C_IN), dtype=torch.bfloat16, device=dev)
    sc = scale if scale is not None else torch.empty(1, dtype=torch.float32, device=dev)
    st = stream or C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    if naux is None:
        naux = 0 if aux is None else 1
    rc = lib.agx_nn_grid_from_field(_p(r), nd, _p(aux), naux, Hn, Wn, Hp, Wp, 1 if normalize else 0, _p(sc),
                                    _p(img), st)
    if rc != 0:
        raise RuntimeError("agx_nn_grid_from_field failed")
    return img, sc


OMEGA = 2.0 / 3.0  # damped Jacobi smoothing around the network (preconditioner mode 2)
ITERATES = (0, 2, 5, 10, 20, 40, 80, 160)  # Jacobi-PCG iterations whose residuals are sampled


class TrainingSet:
    """Residual-to-error pairs of the plain solver, reduced to what the loss needs.

    For a Jacobi-PCG iterate x_k of K x = b (solution x*), r = b - K x_k and e = x* - x_k;
    after the damped Jacobi pre-smoothing of the two-level preconditioner the network sees
    r1 = r - w K D^-1 r with error e1 = e - w D^-1 r.  Stored per sample: r1 / rms(r1)
    (float32, on the GPU), its error energy s = (r1, e1) / rms(r1)^2, and the index of its
    problem, whose float32 tangent values (the library's layout) are kept for K y."""

    def __init__(self, n, prob, r1, s, pid, aux, values, free, nd=1, naux=1, factor=1):
        self.n, self.prob, self.factor = n, prob, factor
        self.r1, self.s, self.pid, self.aux, self.values, self.free = r1, s, pid, aux, values, free
        self.nd, self.naux = nd, naux

    def __len__(self):
        return self.r1.shape[0]


def _solve(prob, rhs, x, rtol, maxiter):
    opts = N.SolveOpts()
    opts.method, opts.rtol, opts.atol, opts.maxiter, opts.check_every = N.AGX_PCG, rtol, 0.0, maxiter, 64
    info = N.SolveInfo()
    rc = prob.lib.agx_solve(prob.ctx, C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()), C.byref(opts),
                            C.byref(info))
    if rc not in (N.AGX_OK, N.AGX_NOT_CONVERGED):
        N.check(prob.ctx, "agx_solve", rc)
    return info


def make_training_set(n_problems, n=256, rhs_per_problem=2, seed0=0, iterates=ITERATES, krylov_tol=1e-10,
                      omega=OMEGA, verbose=False):
    """Samples from the plain float64 Jacobi-PCG solver of this backend on heat-conduction
    problems with seeded random conductivity (the 1024^2 heat workload's family at n x n): for every
    problem and right-hand side (constant, then smooth-plus-rough random fields) one solve
    to ``krylov_tol`` gives x*, and the iterates x_k, k in ``iterates``, give the pairs."""
    from . import configs
    from ._problem import get_problem
    w = configs.heat_grf(n=n, seed=seed0)
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    dev = prob.device
    mask = torch.as_tensor(prob.mask.astype(bool), device=dev)
    free = (~mask).float()
    rng = np.random.default_rng(seed0 + 12345)
    nv = prob.nnzb * prob.ndof * prob.ndof
    values = torch.empty((n_problems, nv), dtype=torch.float32, device=dev)
    auxs = torch.empty((n_problems, prob.n_dofs), dtype=torch.float32, device=dev)
    S = n_problems * rhs_per_problem * len(iterates)
    r1s = torch.empty((S, prob.n_dofs), dtype=torch.float32, device=dev)
    ss = torch.empty(S, dtype=torch.float32, device=dev)
    pid = torch.empty(S, dtype=torch.int64)
    x0 = torch.zeros(prob.n_dofs, dtype=torch.float64, device=dev)
    t = torch.empty_like(x0)
    xs = torch.empty_like(x0)
    xk = torch.empty_like(x0)
    z = torch.empty_like(x0)
    j_out = 0
    for i in range(n_problems):
        k = np.exp(configs.gaussian_random_field(n, seed=seed0 + i)).reshape(-1)
        w.settings["conductivity"] = k
        prob.update_models(w.settings)
        prob._call("agx_assemble", C.c_void_p(x0.data_ptr()), None, N.AGX_F64)
        auxs[i] = torch.as_tensor(node_log_conductivity(k, n, n), device=dev)
        for j in range(rhs_per_problem):
            b = _random_rhs(rng, n + 1, dev) if j else torch.ones(prob.n_dofs, dtype=torch.float64, device=dev)
            b = torch.where(mask, torch.zeros_like(b), b)
            info = _solve(prob, b, xs, krylov_tol, 200000)
            for it in iterates:
                if it == 0:
                    xk.zero_()
                else:
                    _solve(prob, b, xk, 0.0, it)
                prob._call("agx_spmv", N.AGX_F64, C.c_void_p(xk.data_ptr()), C.c_void_p(t.data_ptr()))
                r = b - t
                prob._call("agx_jacobi", N.AGX_F64, C.c_void_p(r.data_ptr()), C.c_void_p(z.data_ptr()))
                z.mul_(omega)
                prob._call("agx_spmv", N.AGX_F64, C.c_void_p(z.data_ptr()), C.c_void_p(t.data_ptr()))
                r1 = r - t
                e1 = (xs - xk) - z
                r1[mask] = 0.0
                e1[mask] = 0.0
                rms = r1.pow(2).mean().sqrt().clamp_min(1e-300)
                r1s[j_out] = (r1 / rms).float()
                ss[j_out] = float((r1 @ e1) / (rms * rms))
                pid[j_out] = i
                j_out += 1
        prob._call("agx_assemble", C.c_void_p(x0.data_ptr()), None, N.AGX_F32)
        prob._call("agx_copy_values", N.AGX_F32, C.c_void_p(values[i].data_ptr()))
        if verbose and i % 100 == 0:
            print(f"training problem {i}: {info.iterations} CG iterations to {krylov_tol:g}", flush=True)
    return TrainingSet(n, prob, r1s, ss, pid, auxs, values, free)


def node_features(coords):
    """Per-node features of a membrane's node grid for the network: the coordinates centred and
    scaled to [-1, 1] by the largest extent (n_nodes, 2)."""
    c = np.asarray(coords, dtype=np.float64)
    c = (c - c.mean(0)) / (np.abs(c - c.mean(0)).max() + 1e-300)
    return c.astype(np.float32)


def _direct(prob, rhs, x):
    """x = K^-1 rhs with the banded Cholesky factor of the assembled float64 tangent."""
    opts = N.SolveOpts()
    opts.method, opts.rtol, opts.atol, opts.maxiter, opts.check_every = N.AGX_CHOL_BAND, 1e-6, 0.0, 1, 1
    info = N.SolveInfo()
    rc = prob.lib.agx_solve(prob.ctx, C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()), C.byref(opts),
                            C.byref(info))
    if rc < 0:
        N.check(prob.ctx, "agx_solve", rc)
    if info.status == N.AGX_DIVERGED:
        raise RuntimeError("the banded Cholesky factorization met a non-positive pivot")
    return info


def chebyshev_presmooth(prob, r, dinv, lmax, degree, frac):
    """Residual left by the degree-`degree` Chebyshev smoother for D^-1 K on [frac lmax, lmax]
    started from z = 0 (the pre-smoothing of preconditioner mode 3), in float64."""
    lmin = frac * lmax
    theta, delta = 0.5 * (lmax + lmin), 0.5 * (lmax - lmin)
    sigma = theta / delta
    rho = 1.0 / sigma
    d = dinv * r / theta
    z = d.clone()
    t = torch.empty_like(r)
    for _ in range(1, degree):
        prob._call("agx_spmv", N.AGX_F64, C.c_void_p(z.data_ptr()), C.c_void_p(t.data_ptr()))
        rc = r - t
        rn = 1.0 / (2.0 * sigma - rho)
        d = rn * rho * d + (2.0 * rn / delta) * dinv * rc
        z = z + d
        rho = rn
    prob._call("agx_spmv", N.AGX_F64, C.c_void_p(z.data_ptr()), C.c_void_p(t.data_ptr()))
    return r - t


def gershgorin_lmax(prob):
    """max over rows of sum_j |K_ij| / |K_ii| of the assembled float64 tangent (the bound the
    Chebyshev smoother of the native FCG uses)."""
    b = prob.ndof
    rp = torch.empty(prob.n_nodes + 1, dtype=torch.int32, device=prob.device)
    col = torch.empty(prob.nnzb, dtype=torch.int32, device=prob.device)
    vals = torch.empty((prob.nnzb, b, b), dtype=torch.float64, device=prob.device)
    prob._call("agx_copy_matrix", N.AGX_F64, C.c_void_p(rp.data_ptr()), C.c_void_p(col.data_ptr()),
               C.c_void_p(vals.data_ptr()))
    row_of = torch.repeat_interleave(torch.arange(prob.n_nodes, device=prob.device), (rp[1:] - rp[:-1]).long())
    absrow = torch.zeros((prob.n_nodes, b), dtype=torch.float64, device=prob.device)
    absrow.index_add_(0, row_of, vals.abs().sum(2))
    diag = vals[row_of == col.long()].diagonal(dim1=1, dim2=2).reshape(prob.n_nodes, b)
    return float((absrow / diag.abs().clamp_min(1e-300)).max())


def make_membrane_training_set(n=128, load_steps=(0, 5, 10, 15, 20), rhs_per_state=400, seed=0, degree=3,
                               frac=1.0 / 30.0, factor=1, verbose=False):
    """Samples for the two-level preconditioner of the nearly incompressible Cook membrane
    (plane-strain neo-Hooke, nu = 0.4999; the 512^2 membrane workload's geometry at n x n):
    for the tangents at the converged states of the given load steps (0: the undeformed
    state) and random smooth-plus-rough vector right-hand sides r, the residual r1 that the
    Chebyshev pre-smoothing of the native FCG leaves and its error energy s = (r1, K^-1 r1),
    K^-1 by the banded Cholesky factor of the float64 tangent.  Stored per sample: r1 / rms,
    s / rms^2 and the state index (whose float32 tangent serves K y in training).  With
    ``factor`` f the network is trained on the (n / f + 1)^2 grid through the bilinear transfers,
    the form in which it serves finer meshes."""
    from . import configs, solver
    from ._problem import get_problem
    w = configs.cook_membrane(n=n, solver="lapack")
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    dev = prob.device
    nd = prob.ndof
    mask = torch.as_tensor(prob.mask.astype(bool), device=dev)
    free = (~mask).float()
    rng = np.random.default_rng(seed + 4242)
    wc = w if factor == 1 else configs.cook_membrane(n=n // factor)
    aux = torch.as_tensor(node_features(wc.raw["coords"]).reshape(-1), device=dev)
    states = [np.zeros(w.n_dofs)] if 0 in load_steps else []
    u = np.zeros(w.n_dofs)
    settings = dict(w.settings)
    for k in range(1, max(load_steps) + 1):
        settings = w.steps[k - 1](settings)
        sol, info = solver.solver(u.reshape(-1, nd), settings, w.static_settings, newton_tol=0.0, newton_rtol=1e-7,
                                  maxiter=12)
        u = np.asarray(sol).reshape(-1)
        if k in load_steps:
            states.append(u.copy())
    nv = prob.nnzb * nd * nd
    S = len(states) * rhs_per_state
    values = torch.empty((len(states), nv), dtype=torch.float32, device=dev)
    r1s = torch.empty((S, prob.n_dofs), dtype=torch.float32, device=dev)
    ss = torch.empty(S, dtype=torch.float32, device=dev)
    pid = torch.empty(S, dtype=torch.int64)
    e1 = torch.empty(prob.n_dofs, dtype=torch.float64, device=dev)
    dinv = torch.empty_like(e1)
    ones = torch.ones_like(e1)
    m = n + 1
    j_out = 0
    for i, us in enumerate(states):
        x = torch.as_tensor(us, device=dev)
        prob.update_models(settings)
        prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, N.AGX_F32)
        prob._call("agx_copy_values", N.AGX_F32, C.c_void_p(values[i].data_ptr()))
        prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, N.AGX_F64)
        prob._call("agx_jacobi", N.AGX_F64, C.c_void_p(ones.data_ptr()), C.c_void_p(dinv.data_ptr()))
        lmax = gershgorin_lmax(prob)
        for j in range(rhs_per_state):
            r = torch.stack([_random_rhs(rng, m, dev) for _ in range(nd)], 1).reshape(-1)
            r = torch.where(mask, torch.zeros_like(r), r)
            r1 = chebyshev_presmooth(prob, r, dinv, lmax, degree, frac)
            r1 = torch.where(mask, torch.zeros_like(r1), r1)
            _direct(prob, r1, e1)
            rms = r1.pow(2).mean().sqrt().clamp_min(1e-300)
            r1s[j_out] = (r1 / rms).float()
            ss[j_out] = float((r1 @ e1) / (rms * rms))
            pid[j_out] = i
            j_out += 1
        if verbose:
            print(f"state {i}: {rhs_per_state} samples, lmax {lmax:.3g}", flush=True)
    auxs = aux.reshape(1, -1).expand(len(states), -1).contiguous()
    return TrainingSet(n, prob, r1s, ss, pid, auxs, values, free, nd=nd, naux=2, factor=factor)


def _random_rhs(rng, m, device):
    """Smooth-plus-rough random field on an m x m node grid."""
    f = np.zeros((m, m))
    for scale in (4, 16, 64):
        c = rng.standard_normal((scale, scale))
        f += np.kron(c, np.ones((m // scale + 1, m // scale + 1)))[:m, :m] / math.sqrt(scale)
    f += 0.1 * rng.standard_normal((m, m))
    return torch.as_tensor(f.reshape(-1), dtype=torch.float64, device=device)


SCALE_PENALTY = 1e-3  # weight of (log rms(y))^2, which keeps the output scale near 1


def energy_loss(r1, y, Ky, s):
    """Per-sample loss 1 - (r1, y)^2 / ((y, K y) (r1, e1)) and its gradient with respect to y.

    With the energy-optimal step c = (r1, y) / (y, K y) the error left after z = c y is
    ||e1 - c y||_K^2 = ||e1||_K^2 - (r1, y)^2 / (y, K y), so the loss is the fraction of the
    error energy the correction leaves (0 for y parallel to e1), independent of the scales of
    y and r1.  It is evaluated in float64 on y / rms(y) (for a function homogeneous of degree
    0, grad L(y) = grad L(y / sigma) / sigma); K is symmetric:
    d/dy = -2 a / (b s) (r1 - (a / b) K y), a = (r1, y), b = (y, K y).  A weak penalty
    SCALE_PENALTY (log sigma)^2 keeps sigma = rms(y) near 1: the loss alone is blind to the
    scale, which otherwise drifts.  Samples whose values are not finite get zero gradient."""
    r1, y, Ky, s = r1.double(), y.double(), Ky.double(), s.double()
    n = y.shape[1]
    sig = y.pow(2).mean(1).sqrt().clamp_min(1e-30)
    yn, Kyn = y / sig[:, None], Ky / sig[:, None]
    a = (r1 * yn).sum(1)
    bq = (yn * Kyn).sum(1)
    bq = torch.where(bq.abs() > 1e-30, bq, torch.full_like(bq, 1e-30))
    loss = 1.0 - a * a / (bq * s)
    grad = -(2.0 * a / (bq * s))[:, None] * (r1 - (a / bq)[:, None] * Kyn) / sig[:, None]
    grad = grad + (2.0 * SCALE_PENALTY * torch.log(sig) / (n * sig * sig))[:, None] * y
    ok = torch.isfinite(loss) & torch.isfinite(grad).all(1)
    loss = torch.where(ok, loss, torch.zeros_like(loss))
    grad = torch.where(ok[:, None], grad, torch.zeros_like(grad))
    return loss, grad.float()


def train(net, ts, steps=3000, batch=16, lr=2e-3, seed=0, verbose=False):
    """Adam with a cosine learning-rate schedule on :func:`energy_loss`; every product K y
    runs through agx_spmv_values with the stored tangent of the sample's problem.

    With ``ts.factor`` f > 1 the network works on the grid coarsened by f, as
    :class:`GridPreconditioner` applies it: input P^T r1 (Dirichlet nodes zeroed), output
    y = P y_c on the sample's grid, and the gradient P^T dL/dy for the network."""
    lib = net.lib
    prob = ts.prob
    f = getattr(ts, "factor", 1)
    Hf = ts.n + 1
    Hn = Wn = ts.n // f + 1
    Hp, Wp = padded(Hn), padded(Wn)
    nd = ts.nd
    fixed = torch.as_tensor(prob.mask.astype(np.uint8), device=net.device) if f > 1 else None
    rc_buf = torch.empty((batch, Hn * Wn * nd), dtype=torch.float32, device=net.device)
    y_fine = torch.empty((batch, Hf * Hf * nd), dtype=torch.float32, device=net.device)
    gc_buf = torch.empty((batch, Hn * Wn * nd), dtype=torch.float32, device=net.device)
    params = net.parameters()
    opt = torch.optim.Adam(params, lr=lr)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, steps)
    gen = torch.Generator().manual_seed(seed)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    losses = []
    x = torch.empty((batch, Hp, Wp, C_IN), dtype=torch.bfloat16, device=net.device)
    sc = torch.empty(batch, dtype=torch.float32, device=net.device)
    Ky = torch.empty((batch, prob.n_dofs), dtype=torch.float32, device=net.device)
    g = torch.zeros((batch, Hp, Wp, C_OUT), dtype=torch.float32, device=net.device)
    for step in range(steps):
        idx = torch.randint(0, len(ts), (batch,), generator=gen)
        pids = ts.pid[idx].tolist()
        for b, (i, pi) in enumerate(zip(idx.tolist(), pids)):
            src = ts.r1[i]
            if f > 1:
                rc = lib.agx_nn_restrict_field(_p(ts.r1[i]), _p(fixed), nd, Hn, Wn, f, _p(rc_buf[b]), stream)
                if rc != 0:
                    raise RuntimeError("agx_nn_restrict_field failed")
                src = rc_buf[b]
            to_image(lib, src, ts.aux[pi], Hn, Wn, True, out=x[b:b + 1], scale=sc[b:b + 1], stream=stream,
                     nd=nd, naux=ts.naux)
        out, acts = net.forward(x, keep=True)
        yc = out[..., :nd].float()[:, :Hn, :Wn].reshape(batch, -1).contiguous()
        if f > 1:
            for b in range(batch):
                rc = lib.agx_nn_prolong_field(_p(yc[b]), nd, Hn, Wn, f, _p(y_fine[b]), stream)
                if rc != 0:
                    raise RuntimeError("agx_nn_prolong_field failed")
            y = (y_fine * ts.free).contiguous()
        else:
            y = (yc * ts.free).contiguous()
        for b, pi in enumerate(pids):
            prob._call("agx_spmv_values", N.AGX_F32, C.c_void_p(ts.values[pi].data_ptr()),
                       C.c_void_p(y[b].data_ptr()), C.c_void_p(Ky[b].data_ptr()))
        r1 = ts.r1[idx.to(net.device)]
        loss, grad = energy_loss(r1, y, Ky, ts.s[idx.to(net.device)])
        gy = (grad * ts.free / batch).contiguous()
        if f > 1:  # y = P y_c: dL/dy_c = P^T dL/dy
            for b in range(batch):
                rc = lib.agx_nn_restrict_field(_p(gy[b]), None, nd, Hn, Wn, f, _p(gc_buf[b]), stream)
                if rc != 0:
                    raise RuntimeError("agx_nn_restrict_field failed")
            gy = gc_buf
        g[:, :Hn, :Wn, :nd] = gy.reshape(batch, Hn, Wn, nd)
        # the backward pass is linear in g: run it on g / max|g| (bf16-friendly) and rescale
        gmax = float(g.abs().max().clamp_min(1e-30))
        gw, gb = net.backward((g / gmax).to(torch.bfloat16), acts)
        for name, *_ in net.layers:
            net.w[name].grad = gw[name] * gmax
            net.b[name].grad = gb[name] * gmax
        if bool(torch.stack([torch.isfinite(t.grad).all() for t in params]).all()):
            opt.step()
        sched.step()
        opt.zero_grad(set_to_none=True)
        with torch.no_grad():
            net.w["e0a"][:, net.n_in:] = 0.0
        net.pack()
        losses.append(float(loss.mean()))
        if verbose and step % 100 == 0:
            print(f"step {step}: loss {np.mean(losses[-50:]):.4f}", flush=True)
    net.check()
    return losses


# ---- preconditioner for flexible CG ----------------------------------------------------------
def coarse_log_conductivity(k_elem, nx, ny, f):
    """Node log-conductivity of the grid coarsened by f: k averaged over f x f element blocks,
    then :func:`node_log_conductivity` on the (nx / f) x (ny / f) coarse elements."""
    k = np.asarray(k_elem, dtype=np.float64).reshape(nx, ny)
    kc = k.reshape(nx // f, f, ny // f, f).mean(axis=(1, 3))
    return node_log_conductivity(kc.reshape(-1), nx // f, ny // f)


class GridPreconditioner:
    """The network as the coarse solver of a two-level preconditioner on the node grid of an
    nx x ny structured quad mesh, for a field of ``nd`` components per node (1: heat, the
    network's features the coarse log-conductivity; 2: a plane displacement field, features
    given as ``aux``).

    FCG applies it in a symmetric two-level form: smoothing (damped Jacobi, mode 2, as in
    training, or Chebyshev, mode 3), y = P net(P^T r) with the energy-optimal step, and
    smoothing again.  P is bilinear interpolation from the grid coarsened by ``factor`` (1: the
    network runs on the node grid itself), so a network trained on n x n problems serves
    (factor n) x (factor n) problems on its own resolution.  All buffers are allocated here and the callback only
    enqueues kernels on the stream it is given, so FCG captures it into CUDA graphs."""

    def __init__(self, net, nx, ny, k_elem=None, factor=1, mode=None, omega=None, sweeps=None, fixed=None, nd=1,
                 aux=None, bf16_smoothing=False, autotune=True):
        if nx % factor or ny % factor:
            raise ValueError("the grid must be divisible by the coarsening factor")
        self.net = net
        self.nd = nd
        # the smoothing, residual and step products on a bf16 copy of the tangent's values
        # (AGX_PRECOND_BF16_SMOOTHING)
        self.bf16_smoothing = bool(bf16_smoothing)
        # smoothing around the network, measured on the 1024^2 heat workload to a 1e-10
        # residual: on a coarsened grid (factor 4) the degree-3 Chebyshev smoother on
        # [lmax/30, lmax] (mode 3: 0.070 s; damped Jacobi, mode 2, best at 5 sweeps: 0.093 s);
        # on the network's own grid (256^2, launch-bound) 2 damped Jacobi sweeps (0.026 s;
        # Chebyshev degree 2: 0.031 s)
        if mode is None:
            mode = 2 if factor == 1 else 3
        self.mode = mode
        self.omega = omega if omega is not None else (OMEGA if mode != 3 else 1.0 / 30.0)
        self.sweeps = sweeps if sweeps is not None else (2 if mode != 3 else 3)
        self.factor = factor
        self.nx, self.ny = nx, ny
        self.Hn, self.Wn = nx // factor + 1, ny // factor + 1
        self.Hp, self.Wp = padded(self.Hn), padded(self.Wn)
        dev = net.device
        # per-node features of the network's grid: the coarse log-conductivity (heat), or the
        # caller's (Hn Wn, naux) array
        if aux is None:
            aux = coarse_log_conductivity(k_elem, nx, ny, factor)
        aux = np.asarray(aux, dtype=np.float32).reshape(self.Hn * self.Wn, -1)
        self.naux = aux.shape[1]
        self.aux = torch.as_tensor(np.ascontiguousarray(aux), device=dev)
        self.img = torch.zeros((1, self.Hp, self.Wp, C_IN), dtype=torch.bfloat16, device=dev)
        self.scale = torch.empty(1, dtype=torch.float32, device=dev)
        self.rc = torch.zeros(self.Hn * self.Wn * nd, dtype=torch.float32, device=dev)
        self.yc = torch.zeros(self.Hn * self.Wn * nd, dtype=torch.float32, device=dev)
        self.work = torch.zeros(net.lib.agx_nn_restrict_image_work(), dtype=torch.float64, device=dev)
        self.fixed = None if fixed is None else torch.as_tensor(np.asarray(fixed, dtype=np.uint8), device=dev)
        self.arena = {}
        self.applications = 0
        self.skip_flag = None  # the solve's converged flag once attached to a problem
        # every layer's convolution variant timed on this grid's shapes (before FCG captures them)
        self.loaders = net.autotune(self.img) if autotune else {}
        net.forward(self.img, arena=self.arena)  # allocate the activations once
        torch.cuda.synchronize(dev)
        net.const_weights = True  # packed and synchronised: later forward passes may prefetch them

    def apply_ptr(self, r_ptr, z_ptr, n, stream):
        lib = self.net.lib
        # the network's kernels return at once when the solve has converged (iterations a
        # captured chunk runs past convergence)
        lib.agx_nn_set_skip_flag(self.skip_flag)
        try:
            return self._apply(lib, r_ptr, z_ptr, stream)
        finally:
            lib.agx_nn_set_skip_flag(None)

    def _apply(self, lib, r_ptr, z_ptr, stream):
        st = C.c_void_p(stream)
        f = self.factor
        nd = self.nd
        if f > 1:
            # restriction, 1 / rms and the input image in two launches; the output prolonged
            # straight from the network's image, zero at the prescribed DOFs
            rc = lib.agx_nn_restrict_image(C.c_void_p(r_ptr), _p(self.fixed), nd, _p(self.aux), self.naux, self.Hn,
                                           self.Wn, f, self.Hp, self.Wp, _p(self.rc), _p(self.work), _p(self.scale),
                                           _p(self.img), st)
            if rc != 0:
                return rc
            out = self.net.forward(self.img, stream=st, arena=self.arena)
            rc = lib.agx_nn_prolong_image(_p(out), C_OUT, nd, self.Hn, self.Wn, self.Wp, f, _p(self.fixed),
                                          C.c_void_p(z_ptr), st)
            self.net.launches += 3
        else:
            rc = lib.agx_nn_grid_from_field(C.c_void_p(r_ptr), nd, _p(self.aux), self.naux, self.Hn, self.Wn,
                                            self.Hp, self.Wp, 1, _p(self.scale), _p(self.img), st)
            if rc != 0:
                return rc
            out = self.net.forward(self.img, stream=st, arena=self.arena)
            rc = lib.agx_nn_field_from_grid(_p(out), C_OUT, nd, self.Hn, self.Wn, self.Wp, C.c_void_p(z_ptr), st)
            self.net.launches += 3  # 1 / rms, image, field
        self.applications += 1
        return rc

    def attach(self, prob):
        """Register with a problem's native context (FCG then calls it and captures it)."""
        cb = self.callback(prob)
        prob._precond_cb = cb
        prob._call("agx_set_preconditioner", cb, None)
        flags = N.AGX_PRECOND_CAPTURABLE | (N.AGX_PRECOND_BF16_SMOOTHING if self.bf16_smoothing else 0)
        prob._call("agx_set_preconditioner_mode", int(self.mode), float(self.omega), int(self.sweeps), flags)
        prob.learned = self

    def _grid_dofs(self):
        return (self.nx + 1) * (self.ny + 1) * self.nd

    def callback(self, prob):
        if prob.n_dofs != self._grid_dofs():
            raise ValueError("the learned preconditioner was built for another grid")
        if self.factor > 1 and self.fixed is None:
            self.fixed = torch.as_tensor(prob.mask.astype(np.uint8), device=self.net.device)
        flag = C.c_void_p()
        prob._call("agx_solve_flag", C.byref(flag))
        self.skip_flag = flag

        def fn(user, r, z, n, stream):
            try:
                return self.apply_ptr(r, z, n, stream)
            except Exception:  # noqa: BLE001 -- report through the status code
                return -1
        return N.PRECOND_FN(fn)


# ---- the 3-D variant: structured brick meshes -------------------------------------------------
class BrickPreconditioner(GridPreconditioner):
    """The 3-D network as the coarse solver of the two-level preconditioner on the node grid of
    an n x n x n structured brick mesh (scalar field, ``mesher.structured_mesh`` node order).

    The network works on the grid coarsened by ``factor`` (trilinear P), padded to a multiple
    of 8 voxels a side; its input channels are the restricted residual / rms and a 0/1
    indicator of the coarse grid inside the padding.  Smoothing (damped Jacobi, two sweeps, by
    default), the energy-optimal step and the capture into CUDA graphs are those of
    :class:`GridPreconditioner`."""

    def __init__(self, net, n, factor=4, mode=2, omega=None, sweeps=None, fixed=None):
        if n % factor:
            raise ValueError("the grid must be divisible by the coarsening factor")
        if getattr(net, "dims", 2) != 3:
            raise ValueError("BrickPreconditioner needs a UNet3D")
        self.net, self.nd, self.bf16_smoothing = net, 1, False
        # smoothing measured on the 128^3 workload over 10 time steps (ms per step, mixed
        # Jacobi-PCG 22.2): damped Jacobi (mode 2, the training's smoother) 1 / 2 sweeps 21.2 /
        # 19.7, Chebyshev (mode 3) degree 1 / 2 / 3 22.7 / 25.9 / 24.0
        self.mode = mode
        self.omega = omega if omega is not None else (OMEGA if mode != 3 else 1.0 / 30.0)
        self.sweeps = sweeps if sweeps is not None else (2 if mode != 3 else 3)
        self.factor, self.n = factor, n
        self.nc = n // factor + 1
        self.npad = padded3(self.nc)
        dev = net.device
        self.img = torch.zeros((1, self.npad, self.npad, self.npad, C_IN), dtype=torch.bfloat16, device=dev)
        self.scale = torch.empty(1, dtype=torch.float32, device=dev)
        self.rc = torch.zeros(self.nc ** 3, dtype=torch.float32, device=dev)
        self.work = torch.zeros(net.lib.agx_nn_restrict_image3d_work(), dtype=torch.float64, device=dev)
        self.fixed = None if fixed is None else torch.as_tensor(np.asarray(fixed, dtype=np.uint8), device=dev)
        self.arena = {}
        self.applications = 0
        self.skip_flag = None
        net.forward(self.img, arena=self.arena)
        torch.cuda.synchronize(dev)
        net.const_weights = True

    def _grid_dofs(self):
        return (self.n + 1) ** 3

    def _apply(self, lib, r_ptr, z_ptr, stream):
        st = C.c_void_p(stream)
        nc, npad, f = self.nc, self.npad, self.factor
        rc = lib.agx_nn_restrict_image3d(C.c_void_p(r_ptr), _p(self.fixed), nc, nc, nc, f, npad, npad, npad,
                                         _p(self.rc), _p(self.work), _p(self.scale), _p(self.img), st)
        if rc != 0:
            return rc
        out = self.net.forward(self.img, stream=st, arena=self.arena)
        rc = lib.agx_nn_prolong_image3d(_p(out), C_OUT, nc, nc, nc, npad, npad, f, _p(self.fixed), C.c_void_p(z_ptr),
                                        st)
        self.net.launches += 3
        self.applications += 1
        return rc


ITERATES3 = (0, 2, 5, 10, 20, 40)


def _random_rhs3(rng, m, device):
    """Smooth-plus-rough random field on an m x m x m node grid."""
    f = np.zeros((m, m, m))
    for scale in (4, 16):
        c = rng.standard_normal((scale, scale, scale))
        k = m // scale + 1
        f += np.kron(c, np.ones((k, k, k)))[:m, :m, :m] / math.sqrt(scale)
    f += 0.1 * rng.standard_normal((m, m, m))
    return torch.as_tensor(f.reshape(-1), dtype=torch.float64, device=device)


def make_brick_training_set(n=128, states=2, rhs_per_state=4, seed0=0, iterates=ITERATES3, krylov_tol=1e-10,
                            omega=OMEGA, factor=4, verbose=False):
    """Samples of the 128^3 backward-Euler heat workload's family: for ``states`` seeded random
    temperature fields T (the tangent of the first Newton step of a time step from T, with
    k = 1 + 0.5 T^2) and right-hand sides (the Newton residual at T, then smooth-plus-rough
    random fields), the iterates of the plain float64 Jacobi-PCG solver give (residual, error)
    pairs as in :func:`make_training_set`."""
    from . import configs
    from ._problem import get_problem
    w = configs.heat_transient(n=n, seed=seed0)
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    dev = prob.device
    mask = torch.as_tensor(prob.mask.astype(bool), device=dev)
    free = (~mask).float()
    rng = np.random.default_rng(seed0 + 4321)
    nv = prob.nnzb * prob.ndof * prob.ndof
    values = torch.empty((states, nv), dtype=torch.float32, device=dev)
    S = states * rhs_per_state * len(iterates)
    r1s = torch.empty((S, prob.n_dofs), dtype=torch.float32, device=dev)
    ss = torch.empty(S, dtype=torch.float32, device=dev)
    pid = torch.empty(S, dtype=torch.int64)
    t = torch.empty(prob.n_dofs, dtype=torch.float64, device=dev)
    xs, xk, z, res = (torch.empty_like(t) for _ in range(4))
    j_out = 0
    for i in range(states):
        T = torch.as_tensor(rng.uniform(0.0, 1.0, prob.n_dofs), device=dev)
        T[mask] = 0.0
        w.settings["dofs n"] = {"T": T.cpu().numpy()}
        prob.update_models(w.settings)
        prob._call("agx_assemble", C.c_void_p(T.data_ptr()), C.c_void_p(res.data_ptr()), N.AGX_F64)
        for j in range(rhs_per_state):
            b = -res.clone() if j == 0 else _random_rhs3(rng, n + 1, dev)
            b = torch.where(mask, torch.zeros_like(b), b)
            info = _solve(prob, b, xs, krylov_tol, 200000)
            for it in iterates:
                if it == 0:
                    xk.zero_()
                else:
                    _solve(prob, b, xk, 0.0, it)
                prob._call("agx_spmv", N.AGX_F64, C.c_void_p(xk.data_ptr()), C.c_void_p(t.data_ptr()))
                r = b - t
                prob._call("agx_jacobi", N.AGX_F64, C.c_void_p(r.data_ptr()), C.c_void_p(z.data_ptr()))
                z.mul_(omega)
                prob._call("agx_spmv", N.AGX_F64, C.c_void_p(z.data_ptr()), C.c_void_p(t.data_ptr()))
                r1 = r - t
                e1 = (xs - xk) - z
                r1[mask] = 0.0
                e1[mask] = 0.0
                rms = r1.pow(2).mean().sqrt().clamp_min(1e-300)
                r1s[j_out] = (r1 / rms).float()
                ss[j_out] = float((r1 @ e1) / (rms * rms))
                pid[j_out] = i
                j_out += 1
            if verbose:
                print(f"state {i} rhs {j}: {info.iterations} CG iterations to {krylov_tol:g}", flush=True)
        prob._call("agx_assemble", C.c_void_p(T.data_ptr()), None, N.AGX_F32)
        prob._call("agx_copy_values", N.AGX_F32, C.c_void_p(values[i].data_ptr()))
    return TrainingSet(n, prob, r1s, ss, pid, None, values, free, nd=1, naux=0, factor=factor)


def train3d(net, ts, steps=1000, batch=4, lr=2e-3, seed=0, verbose=False):
    """:func:`train` for the 3-D network: input image restrict_image3d(P^T r1) (as the
    preconditioner builds it), y = P (output channel 0), dL/d(output) = P^T dL/dy."""
    lib = net.lib
    prob = ts.prob
    f = ts.factor
    nc = ts.n // f + 1
    npad = padded3(nc)
    fixed = torch.as_tensor(prob.mask.astype(np.uint8), device=net.device)
    dev = net.device
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    x = torch.zeros((batch, npad, npad, npad, C_IN), dtype=torch.bfloat16, device=dev)
    rc = torch.empty((batch, nc ** 3), dtype=torch.float32, device=dev)
    work = torch.empty(lib.agx_nn_restrict_image3d_work(), dtype=torch.float64, device=dev)
    sc = torch.empty(batch, dtype=torch.float32, device=dev)
    y = torch.empty((batch, prob.n_dofs), dtype=torch.float32, device=dev)
    Ky = torch.empty_like(y)
    gc = torch.empty((batch, nc ** 3), dtype=torch.float32, device=dev)
    g = torch.zeros((batch, npad, npad, npad, C_OUT), dtype=torch.float32, device=dev)
    params = net.parameters()
    opt = torch.optim.Adam(params, lr=lr)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, steps)
    gen = torch.Generator().manual_seed(seed)
    losses = []

    def ok(name, rcode):
        if rcode != 0:
            raise RuntimeError(f"{name} failed with status {rcode}")
    for step in range(steps):
        idx = torch.randint(0, len(ts), (batch,), generator=gen)
        pids = ts.pid[idx].tolist()
        for b, i in enumerate(idx.tolist()):
            ok("agx_nn_restrict_image3d",
               lib.agx_nn_restrict_image3d(_p(ts.r1[i]), _p(fixed), nc, nc, nc, f, npad, npad, npad, _p(rc[b]),
                                           _p(work), _p(sc[b:b + 1]), _p(x[b:b + 1]), stream))
        out, acts = net.forward(x, keep=True)
        for b in range(batch):
            ok("agx_nn_prolong_image3d",
               lib.agx_nn_prolong_image3d(_p(out[b:b + 1]), C_OUT, nc, nc, nc, npad, npad, f, _p(fixed), _p(y[b]),
                                          stream))
        for b, pi in enumerate(pids):
            prob._call("agx_spmv_values", N.AGX_F32, C.c_void_p(ts.values[pi].data_ptr()),
                       C.c_void_p(y[b].data_ptr()), C.c_void_p(Ky[b].data_ptr()))
        r1 = ts.r1[idx.to(dev)]
        loss, grad = energy_loss(r1, y, Ky, ts.s[idx.to(dev)])
        gy = (grad * ts.free / batch).contiguous()
        for b in range(batch):  # y = P y_c, zero at fixed nodes: dL/dy_c = P^T (dL/dy masked)
            ok("agx_nn_restrict3d", lib.agx_nn_restrict3d(_p(gy[b]), None, nc, nc, nc, f, _p(gc[b]), stream))
        g[:, :nc, :nc, :nc, 0] = gc.reshape(batch, nc, nc, nc)
        gmax = float(g.abs().max().clamp_min(1e-30))
        gw, gb = net.backward((g / gmax).to(torch.bfloat16), acts)
        for name, *_ in net.layers:
            net.w[name].grad = gw[name] * gmax
            net.b[name].grad = gb[name] * gmax
        if bool(torch.stack([torch.isfinite(t.grad).all() for t in params]).all()):
            opt.step()
        sched.step()
        opt.zero_grad(set_to_none=True)
        with torch.no_grad():
            net.w["e0a"][:, net.n_in:] = 0.0
        net.pack()
        losses.append(float(loss.mean()))
        if verbose and step % 100 == 0:
            print(f"step {step}: loss {np.mean(losses[-50:]):.4f}", flush=True)
    net.check()
    return losses
