"""Native contexts built from AutoPDEx's ``settings`` / ``static_settings`` dicts.

A context holds one mesh's pattern, scatter maps and work vectors on the GPU; it is built
once per (node coordinates, connectivity tuple, models) and reused across calls, the way
AutoPDEx reuses a jit compilation per static_settings (utility.py:32-80).  Connectivity and
coordinate arrays must not be changed in place between calls (JAX arrays cannot be).
"""
import ctypes as C
import os
from collections import OrderedDict

import numpy as np
import torch

from . import _native as N

_CACHE = OrderedDict()
_CACHE_MAX = 4


def is_foreign(a):
    """An array from another framework (JAX, CuPy, ...) that exports DLPack."""
    return hasattr(a, "__dlpack__") and not isinstance(a, (np.ndarray, torch.Tensor))


def as_torch(a):
    """torch view of a DLPack array (zero-copy on the same device), torch tensors unchanged."""
    return torch.from_dlpack(a) if is_foreign(a) else a


def _np(a, dtype=None):
    a = as_torch(a)
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    a = np.asarray(a)
    return a if dtype is None else np.ascontiguousarray(a, dtype=dtype)


def dof_layout(dofs):
    """(field key or None, n_nodes, ndof) of a single-field dict or an array of DOFs.

    Node-major numbering dof = node * ndof + component, as assembler.py:47-141 and
    :331-436 number a single field.  Several fields in one dict are not supported."""
    if callable(dofs):
        raise NotImplementedError("DOFs given as a function of time are not supported by the gb300 backend")
    key = None
    if isinstance(dofs, dict):
        if len(dofs) != 1:
            raise NotImplementedError("the gb300 backend supports DOF dicts with one field")
        key = next(iter(dofs))
        arr = dofs[key]
    else:
        arr = dofs
    shape = tuple(arr.shape)
    if len(shape) == 1:
        return key, shape[0], 1
    if len(shape) == 2:
        return key, shape[0], shape[1]
    raise ValueError("DOF arrays must be (n_nodes,) or (n_nodes, n_fields)")


def _field(obj, key):
    if isinstance(obj, dict):
        if key is None:
            if len(obj) != 1:
                raise NotImplementedError("one field expected")
            return next(iter(obj.values()))
        return obj[key]
    return obj


def _elem_type(nen, dim, surface=False):
    """Element type of a set: boundary lines (a surface model) or domain elements by their
    node count (3-node triangles and 3-node lines differ only in the model)."""
    if surface:
        if dim == 2 and nen in (2, 3):
            return N.AGX_LINE2 if nen == 2 else N.AGX_LINE3
    else:
        table = {(2, 4): N.AGX_QUAD4, (2, 9): N.AGX_QUAD9, (2, 3): N.AGX_TRI3, (2, 6): N.AGX_TRI6,
                 (3, 8): N.AGX_HEX8, (3, 27): N.AGX_HEX27, (3, 4): N.AGX_TET4, (3, 10): N.AGX_TET10}
        if (dim, nen) in table:
            return table[(dim, nen)]
    raise NotImplementedError(f"{'boundary' if surface else 'domain'} elements with {nen} nodes in {dim}-D are not "
                              "supported by the gb300 backend (Q1/Q2 quads, P1/P2 triangles, Q1/Q2 bricks, P1/P2 "
                              "tetrahedra, 2- and 3-node boundary lines)")


def flatten(values, key):
    """Flattened float64 view of a DOF-shaped structure (utility.dict_flatten order)."""
    return _np(_field(values, key), np.float64).reshape(-1)


class Problem:
    """A native context plus the Python-side state that feeds it."""

    def __init__(self, dofs, settings, static_settings):
        lib = N.load()
        if not torch.cuda.is_available():
            raise RuntimeError("the gb300 backend needs a CUDA device (no CPU fallback)")
        self.lib = lib
        self.key, self.n_nodes, self.ndof = dof_layout(dofs)
        self.n_dofs = self.n_nodes * self.ndof
        modes = tuple(static_settings["assembling mode"])
        self.models = tuple(static_settings["model"])
        if len(modes) != len(self.models):
            raise ValueError("'assembling mode' and 'model' must have one entry per set")
        for m, d in zip(modes, self.models):
            if getattr(d, "mode", None) != m:
                raise NotImplementedError(f"assembling mode {m!r} needs a gb300 model descriptor of that mode")
        self.coords = _np(_field(settings["node coordinates"], self.key), np.float64)
        if self.coords.shape[0] != self.n_nodes:
            raise ValueError("node coordinates and DOFs disagree on the number of nodes")
        self.dim = self.coords.shape[1]
        self.stream = torch.cuda.current_stream()
        self.device = torch.device("cuda", torch.cuda.current_device())
        ctx = C.c_void_p()
        N.check(None, "agx_create", lib.agx_create(C.byref(ctx), C.c_void_p(self.stream.cuda_stream)))
        self.ctx = ctx
        self._call("agx_set_nodes", self.n_nodes, self.dim, self.coords.ctypes.data, self.ndof)
        self.conns = []
        if len(settings["connectivity"]) != len(self.models):
            raise ValueError("settings['connectivity'] must have one entry per set")
        for conn_obj, desc in zip(settings["connectivity"], self.models):
            conn = _np(_field(conn_obj, self.key), np.int64)
            et = _elem_type(conn.shape[1], self.dim, surface=getattr(desc, "dim", None) == 1)
            sid = C.c_int()
            self._call("agx_add_element_set", et, conn.shape[0], conn.shape[1], conn.ctypes.data, C.byref(sid))
            self.conns.append(conn)
            qp = getattr(desc, "qpoints", None)
            if et in (N.AGX_TRI3, N.AGX_TRI6, N.AGX_TET4, N.AGX_TET10):
                if qp is None:
                    raise NotImplementedError("simplex elements need a simplex rule (seeder.int_pts_ref_tri/tet)")
                pts = np.ascontiguousarray(qp, dtype=np.float64)
                w = np.ascontiguousarray(desc.qweights, dtype=np.float64)
                self._call("agx_set_quadrature_points", sid, pts.shape[0], pts.ctypes.data, w.ctypes.data)
            elif qp is not None:
                raise NotImplementedError("a simplex rule was given for a quad/brick/line set")
            else:
                self._call("agx_set_quadrature", sid, int(getattr(desc, "ngauss", 2)))
        self.mask = None
        self.set_dirichlet(settings.get("dirichlet dofs"))
        self._call("agx_finalize")
        n = C.c_int64()
        nnzb = C.c_int64()
        nd = C.c_int()
        self._call("agx_get_sizes", C.byref(n), C.byref(nnzb), C.byref(nd))
        self.nnzb = nnzb.value
        self._elem_field_src = [None] * len(self.models)
        self._node_fields = [None] * len(self.models)
        self.learned = None

    # ---- helpers --------------------------------------------------------------------
    def _call(self, name, *args):
        return N.check(self.ctx, name, getattr(self.lib, name)(self.ctx, *args))

    def __del__(self):
        try:
            if getattr(self, "ctx", None) is not None and self.ctx.value:
                self.lib.agx_destroy(self.ctx)
                self.ctx = None
        except Exception:
            pass

    def set_dirichlet(self, dirichlet_dofs):
        if dirichlet_dofs is None:
            mask = np.zeros(self.n_dofs, dtype=np.uint8)
        else:
            mask = _np(_field(dirichlet_dofs, self.key)).astype(bool).reshape(-1).astype(np.uint8)
            if mask.shape[0] != self.n_dofs:
                raise ValueError("settings['dirichlet dofs'] does not match the DOFs")
        if self.mask is not None and np.array_equal(mask, self.mask):
            return
        self.mask = mask
        self._call("agx_set_dirichlet", mask.ctypes.data)

    def update_models(self, settings):
        """Resolve every descriptor against the current settings (load multiplier, E, ...)."""
        for sid, (desc, conn) in enumerate(zip(self.models, self.conns)):
            model, params, efield, nfield_key = desc.resolve(settings, self.coords, conn)
            p = np.asarray(params, dtype=np.float64)
            self._call("agx_set_model", sid, model, p.ctypes.data, len(p))
            if efield is not None and efield is not self._elem_field_src[sid]:
                f = np.ascontiguousarray(efield, dtype=np.float64)
                self._call("agx_set_element_field", sid, f.ctypes.data)
                self._elem_field_src[sid] = efield
            if nfield_key is not None:
                v = settings[nfield_key]
                if isinstance(v, torch.Tensor) and v.is_cuda and v.dtype == torch.float64:
                    t = v.reshape(-1).contiguous()
                else:
                    t = torch.as_tensor(flatten(v, self.key), device=self.device)
                if t.numel() != self.n_dofs:
                    raise ValueError(f"settings[{nfield_key!r}] does not match the DOFs")
                self._node_fields[sid] = t
                self._call("agx_set_node_field", sid, C.c_void_p(t.data_ptr()))

    def to_device(self, values):
        """Flat float64 device vector of a DOF-shaped structure: torch CUDA tensors and DLPack
        arrays on this device are used in place (no copy when already float64 and
        contiguous), host arrays are copied over (pinned for large ones)."""
        v = as_torch(_field(values, self.key))
        if isinstance(v, torch.Tensor) and v.is_cuda:
            return v.reshape(-1).to(device=self.device, dtype=torch.float64).contiguous()
        host = torch.from_numpy(np.ascontiguousarray(flatten(values, self.key)))
        return host.pin_memory().to(self.device, non_blocking=True) if self.n_dofs > 4096 else host.to(self.device)

    def ensure_tuned(self, dofs_dev, dtype=N.AGX_F32):
        """Lanes per block row of the Krylov product (float32 or float64) from the autotuner,
        cached per GPU model, precision and problem class in autopdex_gb300/_lib/autotune.json."""
        tuned = getattr(self, "_tuned", set())
        if dtype in tuned:
            return
        import json
        from . import build as _b
        path = os.path.join(_b.LIBDIR, "autotune.json")
        gny, brick = C.c_int(), C.c_int()
        self._call("agx_grid_pattern", C.byref(gny))
        self._call("agx_brick_pattern", C.byref(brick))
        key = f"{torch.cuda.get_device_name(self.device)}|{'f32' if dtype == N.AGX_F32 else 'f64'}|" \
              f"ndof={self.ndof}|dim={self.dim}|nnzb=2^{int(np.log2(max(1, self.nnzb)))}" \
              f"{'|grid' if gny.value > 0 else ''}{'|brick' if brick.value > 0 else ''}"
        cache = {}
        try:
            with open(path) as fh:
                cache = json.load(fh)
        except (OSError, ValueError):
            cache = {}
        if key in cache and self.lib.agx_set_tuning(self.ctx, dtype, int(cache[key]["spmv_tpr"])) == N.AGX_OK:
            tpr_v = int(cache[key]["spmv_tpr"])
        else:
            self._call("agx_assemble", C.c_void_p(dofs_dev.data_ptr()), None, dtype)
            tpr = C.c_int()
            ms = C.c_float()
            self._call("agx_autotune", C.byref(tpr), C.byref(ms))
            cache[key] = {"spmv_tpr": int(tpr.value), "spmv_ms": float(ms.value)}
            tpr_v = int(tpr.value)
            try:
                os.makedirs(os.path.dirname(path), exist_ok=True)
                with open(path, "w") as fh:
                    json.dump(cache, fh, indent=1)
            except OSError:
                pass
        if dtype == N.AGX_F32:
            self.spmv_tpr = tpr_v
        else:
            self.spmv_tpr64 = tpr_v
        self._tuned = tuned | {dtype}

    def matrix(self, dtype):
        rp, col, vals = C.c_void_p(), C.c_void_p(), C.c_void_p()
        nnzb = C.c_int64()
        self._call("agx_get_matrix", dtype, C.byref(rp), C.byref(col), C.byref(vals), C.byref(nnzb))
        return rp.value, col.value, vals.value, nnzb.value


def _key(settings, static_settings, dofs):
    objs = [id(_field(settings["node coordinates"], None if not isinstance(settings["node coordinates"], dict)
                      else next(iter(settings["node coordinates"]))))]
    for c in settings["connectivity"]:
        objs.append(id(_field(c, None if not isinstance(c, dict) else next(iter(c)))))
    objs += [id(m) for m in static_settings["model"]]
    key, n_nodes, ndof = dof_layout(dofs)
    return (tuple(objs), n_nodes, ndof, torch.cuda.current_stream().cuda_stream)


def get_problem(dofs, settings, static_settings):
    """Cached context for this mesh/model combination (rebuilt when any object changes)."""
    k = _key(settings, static_settings, dofs)
    ent = _CACHE.get(k)
    if ent is not None:
        prob, refs = ent
        _CACHE.move_to_end(k)
        prob.set_dirichlet(settings.get("dirichlet dofs"))
        return prob
    prob = Problem(dofs, settings, static_settings)
    # keep the keyed objects alive so that their ids stay unique while cached
    refs = (settings["node coordinates"], tuple(settings["connectivity"]), tuple(static_settings["model"]))
    _CACHE[k] = (prob, refs)
    while len(_CACHE) > _CACHE_MAX:
        _CACHE.popitem(last=False)
    return prob


def clear_cache():
    _CACHE.clear()
