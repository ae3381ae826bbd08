"""ctypes front end of the oracle's C part (oracle/c/orc.c): closed-form float64 Q1 elements
(neo-Hooke bricks and quads, the Poisson and heat potentials, backward-Euler heat, traction
lines), the element-order scatter and a Jacobi-PCG on CSR.  Test infrastructure only."""
import ctypes as C

import numpy as np

from .build_oracle import build

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P = C.c_void_p
        _lib.orc_neo_hooke_hex8.argtypes = [C.c_int64, P, P, P, C.c_double, C.c_double, P, P]
        _lib.orc_neo_hooke_hex8.restype = None
        _lib.orc_pcg_csr.argtypes = [C.c_int64, P, P, P, P, P, P, P, P, P, P, C.c_int]
        _lib.orc_pcg_csr.restype = C.c_double
        _lib.orc_pcg_csr_tol.argtypes = [C.c_int64, P, P, P, P, P, P, P, P, P, P, C.c_int, C.c_double,
                                         C.POINTER(C.c_int)]
        _lib.orc_pcg_csr_tol.restype = C.c_double
        _lib.orc_threads.restype = C.c_int
        _lib.orc_q1_elements.argtypes = [C.c_int, C.c_int, C.c_int64, P, P, P, P, P, P, C.c_int, P, P]
        _lib.orc_q1_elements.restype = None
        _lib.orc_neumann_lines.argtypes = [C.c_int64, P, P, C.c_double, C.c_double, P]
        _lib.orc_neumann_lines.restype = None
        _lib.orc_scatter.argtypes = [C.c_int64, C.c_int, C.c_int, P, P, P]
        _lib.orc_scatter.restype = None
    return _lib


def threads():
    """Threads of the C oracle's parallel loops."""
    return int(lib().orc_threads())


def _p(a):
    return C.c_void_p(a.ctypes.data)


def neo_hooke_hex8(conn, coords, dofs, E, nu, tangent=True):
    """Element residuals (n_e, 24) and, with ``tangent``, tangents (n_e, 24, 24)."""
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    dofs = np.ascontiguousarray(dofs, dtype=np.float64).reshape(-1, 3)
    n_e = conn.shape[0]
    R = np.empty((n_e, 24))
    K = np.empty((n_e, 24, 24)) if tangent else None
    lib().orc_neo_hooke_hex8(n_e, _p(conn), _p(coords), _p(dofs), float(E), float(nu), _p(R),
                             _p(K) if tangent else None)
    return R, K


def pcg_csr_tol(A, b, rtol, maxiter):
    """Jacobi-PCG from zero on the scipy CSR matrix A until ||r|| <= rtol ||b|| (or maxiter):
    (x, (r, r), iterations)."""
    n = A.shape[0]
    rowptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
    col = np.ascontiguousarray(A.indices, dtype=np.int32)
    val = np.ascontiguousarray(A.data, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    work = [np.empty(n) for _ in range(6)]
    done = C.c_int(0)
    rr = lib().orc_pcg_csr_tol(n, _p(rowptr), _p(col), _p(val), _p(b), *[_p(w) for w in work], int(maxiter),
                               float(rtol), C.byref(done))
    return work[0], rr, int(done.value)


def pcg_csr(A, b, iters):
    """``iters`` Jacobi-PCG iterations from zero on the scipy CSR matrix A; (x, (r, r))."""
    n = A.shape[0]
    rowptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
    col = np.ascontiguousarray(A.indices, dtype=np.int32)
    val = np.ascontiguousarray(A.data, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    work = [np.empty(n) for _ in range(6)]
    rr = lib().orc_pcg_csr(n, _p(rowptr), _p(col), _p(val), _p(b), *[_p(w) for w in work], int(iters))
    return work[0], rr


MODELS = {"poisson": 0, "heat": 1, "neo_hooke": 2, "heat_be": 4}


def q1_elements(model, conn, coords, dofs, params, elem_field=None, node_field=None, accurate=False,
                tangent=True):
    """Element residuals (n_e, m) and, with ``tangent``, tangents (n_e, m, m) of a Q1 quad
    (4 nodes) or brick (8 nodes) set; ``model`` one of MODELS."""
    mid = MODELS[model]
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    dim = coords.shape[1]
    nen = conn.shape[1]
    assert nen == (4 if dim == 2 else 8)
    ndof = dim if mid == 2 else 1
    m = nen * ndof
    dofs = np.ascontiguousarray(dofs, dtype=np.float64).reshape(-1)
    prm = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1))
    ef = None if elem_field is None else np.ascontiguousarray(elem_field, dtype=np.float64).reshape(-1)
    nf = None if node_field is None else np.ascontiguousarray(node_field, dtype=np.float64).reshape(-1)
    n_e = conn.shape[0]
    R = np.empty((n_e, m))
    K = np.empty((n_e, m, m)) if tangent else None
    lib().orc_q1_elements(mid, dim, n_e, _p(conn), _p(coords), _p(dofs), _p(prm),
                          _p(ef) if ef is not None else None, _p(nf) if nf is not None else None, int(bool(accurate)),
                          _p(R), _p(K) if tangent else None)
    return R, K


def neumann_lines(lines, coords, traction):
    """Residuals (n_l, 4) of 2-node traction lines in 2-D."""
    lines = np.ascontiguousarray(lines, dtype=np.int64)
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    R = np.empty((lines.shape[0], 4))
    lib().orc_neumann_lines(lines.shape[0], _p(lines), _p(coords), float(traction[0]), float(traction[1]), _p(R))
    return R


def scatter(conn, ndof, R_e, n_dofs):
    """Global vector from element vectors in element order (serial, as a scatter-add)."""
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    R_e = np.ascontiguousarray(R_e, dtype=np.float64)
    R = np.zeros(n_dofs)
    lib().orc_scatter(conn.shape[0], conn.shape[1], int(ndof), _p(conn), _p(R_e), _p(R))
    return R
