"""``assembler.assemble_residual`` / ``assemble_tangent`` of AutoPDEx on the GPU.

``assemble_residual(dofs, settings, static_settings)`` mirrors assembler.py:587-637 and
returns the residual with the structure of ``dofs``; ``assemble_tangent_diagonal`` mirrors
assembler.py:639-680 (flat float64 diagonal, the sum over all element sets).  ``assemble_tangent`` mirrors
assembler.py:682-777 but returns the summed node-block CSR matrix (the BCOO of AutoPDEx
keeps the duplicates until scipy_assembling sums them, solver.py:1180-1222) as a
:class:`BlockCSR` of device arrays; with ``eliminate_dirichlet=True`` the prescribed rows
and columns are already removed (identity rows), as the solve uses it.
"""
import ctypes as C

import numpy as np
import torch

from . import _native as N
from ._problem import get_problem
from .solver import _out_like, _backend_check


class BlockCSR:
    """Node-block CSR on the device: ``rowptr`` (n_nodes+1), ``col`` (nnzb) and ``vals``
    (nnzb, b, b) torch tensors; block (p, col[k]) holds the b x b coupling of the DOFs of
    nodes p and col[k]."""

    def __init__(self, rowptr, col, vals, n_nodes, b):
        self.rowptr, self.col, self.vals, self.n_nodes, self.b = rowptr, col, vals, n_nodes, b

    @property
    def shape(self):
        n = self.n_nodes * self.b
        return (n, n)

    def to_scipy(self):
        import scipy.sparse
        rp = self.rowptr.cpu().numpy().astype(np.int64)
        col = self.col.cpu().numpy().astype(np.int64)
        v = self.vals.double().cpu().numpy()
        return scipy.sparse.bsr_matrix((v, col, rp), shape=self.shape).tocsr()


def assemble_residual(dofs, settings, static_settings):
    _backend_check(static_settings)
    prob = get_problem(dofs, settings, static_settings)
    prob.update_models(settings)
    x = prob.to_device(dofs)
    R = torch.empty_like(x)
    prob._call("agx_assemble", C.c_void_p(x.data_ptr()), C.c_void_p(R.data_ptr()), -1)
    return _out_like(R, dofs, prob.key)


def assemble_tangent(dofs, settings, static_settings, dtype="float64", eliminate_dirichlet=False):
    _backend_check(static_settings)
    prob = get_problem(dofs, settings, static_settings)
    prob.update_models(settings)
    x = prob.to_device(dofs)
    dt = N.AGX_F64 if dtype == "float64" else N.AGX_F32
    saved = prob.mask
    if not eliminate_dirichlet:
        prob.set_dirichlet(None)
    try:
        prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, dt)
        nnzb = prob.nnzb
        b = prob.ndof
        tdt = torch.float64 if dt == N.AGX_F64 else torch.float32
        out_rp = torch.empty(prob.n_nodes + 1, dtype=torch.int32, device=prob.device)
        out_col = torch.empty(nnzb, dtype=torch.int32, device=prob.device)
        out_vals = torch.empty((nnzb, b, b), dtype=tdt, device=prob.device)
        prob._call("agx_copy_matrix", dt, C.c_void_p(out_rp.data_ptr()), C.c_void_p(out_col.data_ptr()),
                   C.c_void_p(out_vals.data_ptr()))
    finally:
        if not eliminate_dirichlet:
            mask = saved.copy()
            prob.mask = None
            prob._call("agx_set_dirichlet", mask.ctypes.data)
            prob.mask = mask
    return BlockCSR(out_rp, out_col, out_vals, prob.n_nodes, b)


def assemble_tangent_diagonal(dofs, settings, static_settings, dtype="float64"):
    """Diagonal of the tangent summed over all element sets (assembler.py:639-680, :1090-1113,
    :1216-1306, :1310-1389): a flat float64 vector of length n_dofs, as ``dict_flatten``
    orders the DOFs.  No Dirichlet elimination (the reference's diagonal has none)."""
    _backend_check(static_settings)
    prob = get_problem(dofs, settings, static_settings)
    prob.update_models(settings)
    x = prob.to_device(dofs)
    dt = N.AGX_F64 if dtype == "float64" else N.AGX_F32
    saved = prob.mask
    prob.set_dirichlet(None)
    try:
        prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, dt)
        diag = torch.empty(prob.n_dofs, dtype=torch.float64, device=prob.device)
        prob._call("agx_get_diagonal", dt, C.c_void_p(diag.data_ptr()))
    finally:
        mask = saved.copy()
        prob.mask = None
        prob._call("agx_set_dirichlet", mask.ctypes.data)
        prob.mask = mask
    ref = dofs[prob.key] if isinstance(dofs, dict) else dofs
    if isinstance(ref, np.ndarray) or not hasattr(ref, "shape"):
        return diag.cpu().numpy()
    return diag
