"""ctypes binding of libautopdex_gb300 (C ABI in include/autopdex_gb300.h).

The library is loaded from the package's ``_lib`` folder.  There is no fallback: if the
shared library is missing or fails to load, every entry point raises.
"""
import ctypes as C
import os
import re

from . import build as _build

AGX_OK = 0
AGX_NOT_CONVERGED = 1
AGX_PRECOND_CAPTURABLE = 1
AGX_PRECOND_BF16_SMOOTHING = 2
AGX_NN_CONST_WEIGHTS = 2
AGX_DIVERGED = 2
AGX_ERR_ARG, AGX_ERR_CUDA, AGX_ERR_UNSUPPORTED, AGX_ERR_STATE = -1, -2, -3, -5


def AGX_NN_LOADER(l):
    """Per-launch halo loader flag of agx_nn_conv3x3 (0 cp.async, 1 tensor copies, 2 warp-specialised)."""
    return (int(l) + 1) << 4


AGX_QUAD4, AGX_HEX8, AGX_LINE2, AGX_QUAD9, AGX_LINE3 = 0, 1, 2, 3, 4
AGX_TRI3, AGX_TRI6, AGX_TET4, AGX_TET10, AGX_HEX27 = 5, 6, 7, 8, 9
AGX_MODEL_POISSON_SINCOS = 0
AGX_MODEL_HEAT_POTENTIAL = 1
AGX_MODEL_NEO_HOOKE = 2
AGX_MODEL_NEUMANN = 3
AGX_MODEL_HEAT_BE = 4
AGX_F64, AGX_F32 = 0, 1
AGX_PCG, AGX_PCG_MIXED, AGX_BICGSTAB, AGX_FCG_MIXED, AGX_CHOL_BAND, AGX_FCG_F64 = 0, 1, 2, 3, 4, 5

AGX_PROF_TANGENT, AGX_PROF_RESIDUAL, AGX_PROF_SPMV, AGX_PROF_VECTOR, AGX_PROF_PRECOND = 0, 1, 2, 3, 4
AGX_PROF_FACTOR, AGX_PROF_SMOOTH = 5, 6
AGX_PROF_CATEGORIES = 8
AGX_NOALLOC_MAX_DOFS = 262144

PRECOND_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p)


class SolveOpts(C.Structure):
    _fields_ = [("method", C.c_int), ("rtol", C.c_double), ("atol", C.c_double), ("maxiter", C.c_int),
                ("check_every", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("rel_residual", C.c_double), ("status", C.c_int)]


class NewtonOpts(C.Structure):
    _fields_ = [("newton_tol", C.c_double), ("newton_rtol", C.c_double), ("maxiter", C.c_int), ("damping", C.c_double),
                ("tangent_dtype", C.c_int), ("krylov", SolveOpts), ("reuse_tangent", C.c_int),
                ("verbose", C.c_int)]


class NewtonInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("res_norm", C.c_double), ("res0", C.c_double), ("diverged", C.c_int),
                ("krylov_iterations", C.c_int), ("n_history", C.c_int),
                ("res_history", C.c_double * 64), ("krylov_history", C.c_int * 64)]


_P = C.c_void_p
_SIGNATURES = {
    "agx_create": (C.c_int, [C.POINTER(_P), _P]),
    "agx_destroy": (C.c_int, [_P]),
    "agx_last_error": (C.c_char_p, [_P]),
    "agx_set_nodes": (C.c_int, [_P, C.c_int64, C.c_int, _P, C.c_int]),
    "agx_add_element_set": (C.c_int, [_P, C.c_int, C.c_int64, C.c_int, _P, C.POINTER(C.c_int)]),
    "agx_set_dirichlet": (C.c_int, [_P, _P]),
    "agx_finalize": (C.c_int, [_P]),
    "agx_set_model": (C.c_int, [_P, C.c_int, C.c_int, _P, C.c_int]),
    "agx_set_element_field": (C.c_int, [_P, C.c_int, _P]),
    "agx_set_node_field": (C.c_int, [_P, C.c_int, _P]),
    "agx_assemble": (C.c_int, [_P, _P, _P, C.c_int]),
    "agx_get_matrix": (C.c_int, [_P, C.c_int, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P), C.POINTER(C.c_int64)]),
    "agx_copy_matrix": (C.c_int, [_P, C.c_int, _P, _P, _P]),
    "agx_copy_values": (C.c_int, [_P, C.c_int, _P]),
    "agx_set_quadrature": (C.c_int, [_P, C.c_int, C.c_int]),
    "agx_set_quadrature_points": (C.c_int, [_P, C.c_int, C.c_int, _P, _P]),
    "agx_spmv_values": (C.c_int, [_P, C.c_int, _P, _P, _P]),
    "agx_jacobi": (C.c_int, [_P, C.c_int, _P, _P]),
    "agx_get_diagonal": (C.c_int, [_P, C.c_int, _P]),
    "agx_spmv": (C.c_int, [_P, C.c_int, _P, _P]),
    "agx_solve": (C.c_int, [_P, _P, _P, C.POINTER(SolveOpts), C.POINTER(SolveInfo)]),
    "agx_newton": (C.c_int, [_P, _P, _P, C.POINTER(NewtonOpts), C.POINTER(NewtonInfo)]),
    "agx_set_preconditioner": (C.c_int, [_P, PRECOND_FN, _P]),
    "agx_set_preconditioner_mode": (C.c_int, [_P, C.c_int, C.c_double, C.c_int, C.c_int]),
    "agx_profile": (C.c_int, [_P, C.c_int]),
    "agx_profile_read": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "agx_autotune": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_float)]),
    "agx_set_tuning": (C.c_int, [_P, C.c_int, C.c_int]),
    "agx_grid_pattern": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "agx_brick_pattern": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "agx_set_pdl": (C.c_int, [C.c_int]),
    "agx_solve_flag": (C.c_int, [_P, C.POINTER(_P)]),
    "agx_nn_set_skip_flag": (C.c_int, [_P]),
    "agx_launch_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
"agx_pcg_noalloc": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int, _P, _P, C.c_double, C.c_int, _P,
                                C.POINTER(SolveInfo), C.c_char_p, C.c_int]),
    "agx_get_sizes": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
    # learned preconditioner (include/autopdex_gb300_nn.h)
    "agx_nn_conv3x3": (C.c_int, [_P, _P, C.c_int, C.c_int, _P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int,
                                 C.c_int, C.c_int, _P, _P]),
    "agx_nn_wgrad3x3": (C.c_int, [_P, _P, C.c_int, C.c_int, _P, C.c_int, _P, C.c_int, C.c_int, C.c_int, _P, _P]),
    "agx_nn_pack_weights": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P]),
    "agx_nn_unpack_wgrad": (C.c_int, [_P, C.c_int, C.c_int, _P, _P]),
    "agx_nn_pool2": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "agx_nn_upsample2": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "agx_nn_pool": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "agx_nn_restrict_image_work": (C.c_int, []),
    "agx_nn_conv3x3x3": (C.c_int, [_P, _P, C.c_int, C.c_int, _P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_int, C.c_int, _P, _P]),
    "agx_nn_wgrad3x3x3": (C.c_int, [_P, _P, C.c_int, C.c_int, _P, C.c_int, _P, C.c_int, C.c_int, C.c_int, C.c_int,
                                    _P, _P]),
    "agx_nn_pack_weights3d": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P]),
    "agx_nn_unpack_wgrad3d": (C.c_int, [_P, C.c_int, C.c_int, _P, _P]),
    "agx_nn_pool3d": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "agx_nn_upsample3d": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "agx_nn_restrict_image3d_work": (C.c_int, []),
    "agx_nn_restrict_image3d": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P,
                                          _P, _P, _P, _P]),
    "agx_nn_restrict3d": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P]),
    "agx_nn_prolong_image3d": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P,
                                         _P]),
    "agx_nn_set_halo_loader": (C.c_int, [C.c_int]),
    "agx_nn_restrict_image": (C.c_int, [_P, _P, C.c_int, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        _P, _P, _P, _P, _P]),
    "agx_nn_prolong_image": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, _P]),
    "agx_nn_upsample": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "agx_nn_relu_backward": (C.c_int, [_P, _P, C.c_int64, _P]),
    "agx_nn_add": (C.c_int, [_P, _P, C.c_int64, _P]),
    "agx_nn_bias_grad": (C.c_int, [_P, C.c_int64, C.c_int, _P, _P]),
    "agx_nn_grid_from_vector": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, _P]),
    "agx_nn_restrict": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, _P, _P]),
    "agx_nn_prolong": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P]),
    "agx_nn_vector_from_grid": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P]),
    "agx_nn_grid_from_field": (C.c_int, [_P, C.c_int, _P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P,
                                         _P, _P]),
    "agx_nn_field_from_grid": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P]),
    "agx_nn_restrict_field": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P]),
    "agx_nn_prolong_field": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P]),
}

_lib = None


def header_symbols():
    """Function names declared in the headers under include/."""
    names = set()
    for f in sorted(os.listdir(_build.INCLUDE)):
        if f.endswith(".h"):
            with open(os.path.join(_build.INCLUDE, f)) as fh:
                txt = fh.read()
            names |= set(re.findall(r"^\s*(?:int|const char\*)\s+(agx_\w+)\s*\(", txt, re.M))
    return sorted(names)


def lib_path():
    return _build.lib_path()


def load(path=None):
    """Load the shared library (building it first when it is absent or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if path is None:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libautopdex_gb300 not found at {path}; run autopdex_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class NativeError(RuntimeError):
    def __init__(self, fn, code, msg):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


def check(ctx, fn, code):
    if code < 0:
        msg = load().agx_last_error(ctx).decode(errors="replace") if ctx else ""
        raise NativeError(fn, code, msg)
    return code
