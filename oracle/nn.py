"""Oracle: the learned preconditioner's U-Net in float64 on the CPU (torch) -- TEST ONLY.

Same layers, parameter names and NHWC tensors as ``autopdex_gb300.learned``: 3x3
convolutions with zero padding, 4x4 average pooling, nearest 4x upsampling, channel
concatenation (decoder input first, encoder skip second), ReLU everywhere except the output
layer.  Gradients come from torch autograd in float64, the reference for the GPU's own
forward and backward kernels.
"""
import torch
import torch.nn.functional as F

LAYERS = [("e0a", 16, 0, 32, 1), ("e0b", 32, 0, 32, 1), ("e1a", 32, 0, 32, 1), ("e1b", 32, 0, 32, 1),
          ("e2a", 32, 0, 32, 1), ("e2b", 32, 0, 32, 1), ("b3a", 32, 0, 32, 1), ("b3b", 32, 0, 32, 1),
          ("d2a", 32, 32, 32, 1), ("d2b", 32, 0, 32, 1), ("d1a", 32, 32, 32, 1), ("d1b", 32, 0, 32, 1),
          ("d0a", 32, 32, 32, 1), ("d0b", 32, 0, 32, 1), ("out", 32, 0, 16, 0)]
RELU = {name: relu for name, _, _, _, relu in LAYERS}


def conv(x, w, b, relu):
    """x: (B, H, W, C) -> (B, H, W, Cout); w: (Cout, C, 3, 3)."""
    y = F.conv2d(x.permute(0, 3, 1, 2), w, b, padding=1).permute(0, 2, 3, 1)
    return F.relu(y) if relu else y


POOL = 4


def pool(x):
    return F.avg_pool2d(x.permute(0, 3, 1, 2), POOL).permute(0, 2, 3, 1)


def up(x):
    return F.interpolate(x.permute(0, 3, 1, 2), scale_factor=POOL, mode="nearest").permute(0, 2, 3, 1)


def prolong(c, f):
    """Bilinear interpolation of a coarse node field (Hc, Wc) to the fine node grid
    ((Hc - 1) f + 1, (Wc - 1) f + 1) whose node (f I, f J) is coarse node (I, J)."""
    import numpy as np
    c = np.asarray(c, dtype=np.float64)

    def p1(m):
        P = np.zeros(((m - 1) * f + 1, m))
        for i in range(P.shape[0]):
            I, t = divmod(i, f)
            if I >= m - 1:
                P[i, m - 1] = 1.0
            else:
                P[i, I] += 1.0 - t / f
                P[i, I + 1] += t / f
        return P
    return p1(c.shape[0]) @ c @ p1(c.shape[1]).T


def unet(x, P, masks=None):
    """P: dict name -> (w, b) float64 tensors.  With ``masks`` (name -> 0/1 tensor), ReLU
    layers multiply their pre-activation by the given mask instead of thresholding it."""
    def c(n, t):
        if masks is not None and RELU[n]:
            return conv(t, P[n][0], P[n][1], 0) * masks[n]
        return conv(t, P[n][0], P[n][1], RELU[n])
    s0 = c("e0b", c("e0a", x))
    s1 = c("e1b", c("e1a", pool(s0)))
    s2 = c("e2b", c("e2a", pool(s1)))
    b3 = c("b3b", c("b3a", pool(s2)))
    d2 = c("d2b", c("d2a", torch.cat([up(b3), s2], dim=-1)))
    d1 = c("d1b", c("d1a", torch.cat([up(d2), s1], dim=-1)))
    d0 = c("d0b", c("d0a", torch.cat([up(d1), s0], dim=-1)))
    return c("out", d0)


# ---- the 3-D network (NDHWC tensors) ----------------------------------------------------------
LAYERS3 = [("e0a", 16, 0, 16, 1), ("e0b", 16, 0, 16, 1), ("e1a", 16, 0, 16, 1), ("e1b", 16, 0, 16, 1),
           ("e2a", 16, 0, 16, 1), ("e2b", 16, 0, 16, 1), ("b3a", 16, 0, 16, 1), ("b3b", 16, 0, 16, 1),
           ("d2a", 16, 16, 16, 1), ("d2b", 16, 0, 16, 1), ("d1a", 16, 16, 16, 1), ("d1b", 16, 0, 16, 1),
           ("d0a", 16, 16, 16, 1), ("d0b", 16, 0, 16, 1), ("out", 16, 0, 16, 0)]
RELU3 = {name: relu for name, _, _, _, relu in LAYERS3}
POOL3 = 2


def conv3d(x, w, b, relu):
    """x: (B, D, H, W, C) -> (B, D, H, W, Cout); w: (Cout, C, 3, 3, 3), taps [dz][dy][dx]."""
    y = F.conv3d(x.permute(0, 4, 1, 2, 3), w, b, padding=1).permute(0, 2, 3, 4, 1)
    return F.relu(y) if relu else y


def pool3d(x):
    return F.avg_pool3d(x.permute(0, 4, 1, 2, 3), POOL3).permute(0, 2, 3, 4, 1)


def up3d(x):
    return F.interpolate(x.permute(0, 4, 1, 2, 3), scale_factor=POOL3, mode="nearest").permute(0, 2, 3, 4, 1)


def unet3d(x, P, masks=None):
    """The 3-D U-Net: the same graph as :func:`unet` with 3x3x3 convolutions, 2x2x2 pooling;
    ``masks`` as there."""
    def c(n, t):
        if masks is not None and RELU3[n]:
            return conv3d(t, P[n][0], P[n][1], 0) * masks[n]
        return conv3d(t, P[n][0], P[n][1], RELU3[n])
    s0 = c("e0b", c("e0a", x))
    s1 = c("e1b", c("e1a", pool3d(s0)))
    s2 = c("e2b", c("e2a", pool3d(s1)))
    b3 = c("b3b", c("b3a", pool3d(s2)))
    d2 = c("d2b", c("d2a", torch.cat([up3d(b3), s2], dim=-1)))
    d1 = c("d1b", c("d1a", torch.cat([up3d(d2), s1], dim=-1)))
    d0 = c("d0b", c("d0a", torch.cat([up3d(d1), s0], dim=-1)))
    return c("out", d0)


def _p1(m, f):
    """1-D linear interpolation from m coarse nodes to (m - 1) f + 1 fine nodes."""
    import numpy as np
    P = np.zeros(((m - 1) * f + 1, m))
    for i in range(P.shape[0]):
        I, t = divmod(i, f)
        if I >= m - 1:
            P[i, m - 1] = 1.0
        else:
            P[i, I] += 1.0 - t / f
            P[i, I + 1] += t / f
    return P


def prolong3(c, f):
    """Trilinear interpolation of a coarse node field (Dc, Hc, Wc) to the fine node grid whose
    node (f I, f J, f K) is coarse node (I, J, K)."""
    import numpy as np
    c = np.asarray(c, dtype=np.float64)
    Pz, Py, Px = (_p1(m, f) for m in c.shape)
    return np.einsum("ai,bj,ck,ijk->abc", Pz, Py, Px, c)


def restrict3(r, f, shape_c):
    """P^T of :func:`prolong3`: full weighting of a fine node field onto the coarse grid."""
    import numpy as np
    r = np.asarray(r, dtype=np.float64)
    Pz, Py, Px = (_p1(m, f) for m in shape_c)
    return np.einsum("ai,bj,ck,abc->ijk", Pz, Py, Px, r)
