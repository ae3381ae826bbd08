"""ctypes front end of the oracle's C part (oracle/c/orc.c): the closed-form float64 neo-Hooke
brick element and a Jacobi-PCG on CSR.  Test infrastructure only."""
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
        _lib.orc_threads.restype = C.c_int
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
