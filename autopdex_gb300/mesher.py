"""Structured quad/brick meshes with AutoPDEx's numbering (mesher.py:29-205).

Host-side set-up.  Node ``i*(ny+1)+j`` (2-D) / ``i*(ny+1)*(nz+1)+j*(nz+1)+k`` (3-D);
element node order of mesher.py:88-94 and :150-160.
"""
import numpy as np


def structured_mesh(n_elements, vertices, element_type, order=1):
    if order != 1:
        raise NotImplementedError("Only order==1 is implemented at this moment.")
    v = np.asarray(vertices, dtype=np.float64)
    dim = v.shape[1]
    if dim == 2:
        if element_type != "quad":
            raise NotImplementedError("the gb300 backend meshes quads in 2-D")
        nx, ny = n_elements
        S, T = np.meshgrid(np.linspace(-1, 1, nx + 1), np.linspace(-1, 1, ny + 1), indexing="ij")
        s, t = S.reshape(-1, 1), T.reshape(-1, 1)
        coords = ((1 - s) * (1 - t) * v[0] + (1 + s) * (1 - t) * v[1] + (1 + s) * (1 + t) * v[2]
                  + (1 - s) * (1 + t) * v[3]) / 4
        i, j = [a.reshape(-1) for a in np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")]
        n0 = i * (ny + 1) + j
        elems = np.stack([n0, n0 + 1, n0 + ny + 2, n0 + ny + 1], axis=1)
        return coords, elems.astype(np.int64)
    if dim == 3:
        if element_type != "brick":
            raise NotImplementedError("the gb300 backend meshes bricks in 3-D")
        nx, ny, nz = n_elements
        S, T, U = np.meshgrid(np.linspace(-1, 1, nx + 1), np.linspace(-1, 1, ny + 1), np.linspace(-1, 1, nz + 1),
                              indexing="ij")
        s, t, u = S.reshape(-1, 1), T.reshape(-1, 1), U.reshape(-1, 1)
        coords = ((1 - s) * (1 - t) * (1 - u) * v[0] + (1 + s) * (1 - t) * (1 - u) * v[1]
                  + (1 + s) * (1 + t) * (1 - u) * v[2] + (1 - s) * (1 + t) * (1 - u) * v[3]
                  + (1 - s) * (1 - t) * (1 + u) * v[4] + (1 + s) * (1 - t) * (1 + u) * v[5]
                  + (1 + s) * (1 + t) * (1 + u) * v[6] + (1 - s) * (1 + t) * (1 + u) * v[7]) / 8
        i, j, k = [a.reshape(-1) for a in np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")]
        a, b = (ny + 1) * (nz + 1), nz + 1
        n0 = i * a + j * b + k
        elems = np.stack([n0, n0 + a, n0 + a + b, n0 + b, n0 + 1, n0 + a + 1, n0 + a + b + 1, n0 + b + 1], axis=1)
        return coords, elems.astype(np.int64)
    raise NotImplementedError("dimension must be 2 or 3")


def structured_boundary_lines(n_elements, side):
    """2-node boundary lines of a structured quad mesh, ordered counter-clockwise.

    ``side``: 'left' (i = 0), 'right' (i = nx), 'bottom' (j = 0), 'top' (j = ny)."""
    nx, ny = n_elements
    node = lambda i, j: i * (ny + 1) + j
    if side == "right":
        a = [node(nx, j) for j in range(ny)]
        b = [node(nx, j + 1) for j in range(ny)]
    elif side == "left":
        a = [node(0, j + 1) for j in range(ny)]
        b = [node(0, j) for j in range(ny)]
    elif side == "bottom":
        a = [node(i, 0) for i in range(nx)]
        b = [node(i + 1, 0) for i in range(nx)]
    elif side == "top":
        a = [node(i + 1, ny) for i in range(nx)]
        b = [node(i, ny) for i in range(nx)]
    else:
        raise ValueError(side)
    return np.stack([a, b], axis=1).astype(np.int64)
