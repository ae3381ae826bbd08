"""DOF-dict helpers with AutoPDEx's semantics (utility.py:82-368, :448-462)."""
import numpy as np


def dict_zeros_like(arr, **kw):
    if isinstance(arr, dict):
        return {k: dict_zeros_like(v, **kw) for k, v in arr.items()}
    return np.zeros(np.shape(arr), **kw)


def dict_ones_like(arr, **kw):
    if isinstance(arr, dict):
        return {k: dict_ones_like(v, **kw) for k, v in arr.items()}
    return np.ones(np.shape(arr), **kw)


def dict_flatten(arr):
    """Concatenate the flattened fields in key order (utility.py:104-128)."""
    if isinstance(arr, dict):
        parts = [dict_flatten(arr[k]) for k in arr.keys()]
        return np.concatenate(parts) if parts else np.zeros(0)
    return np.asarray(arr).reshape(-1)


def reshape_as(flat_array, signature_array):
    """Inverse of dict_flatten (utility.py:130-199)."""
    if isinstance(signature_array, dict):
        out, start = {}, 0
        for k, v in signature_array.items():
            size = int(np.size(v))
            out[k] = reshape_as(flat_array[start:start + size], v)
            start += size
        if start != np.size(flat_array):
            raise ValueError("The size of flat_array does not match the total size of signature_array.")
        return out
    if np.size(flat_array) != np.size(signature_array):
        raise ValueError("The size of flat_array does not match the size of signature_array.")
    return np.asarray(flat_array).reshape(np.shape(signature_array))


def dof_select(dirichlet_nodes, selected_fields):
    """Node mask -> DOF mask (utility.py:448-462)."""
    if isinstance(selected_fields, bool):
        return np.asarray(dirichlet_nodes) * selected_fields
    return np.outer(dirichlet_nodes, np.asarray(selected_fields))
