"""Builders of taco_tensor_t structs over numpy (host) or torch CUDA (device) arrays, laid out as
taco's TensorStorage conversion lays them out (src/storage/storage.cpp:127-177): a dense mode
stores its dimension in a one-element int32 array at indices[m][0]; a compressed mode stores
pos at indices[m][0] and crd at indices[m][1]; csize is in bits.

These are the arguments taco's Module passes to a generated assemble/compute
(src/tensor.cpp:779-806), so the same structs drive both libtacogb and taco's own generated
code in the parity tests.
"""
import ctypes

import numpy as np

from . import _native as N

MODE_DENSE, MODE_SPARSE = 0, 1


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


def _csize(a):
    return int(a.itemsize if isinstance(a, np.ndarray) else a.element_size()) * 8


class TacoTensor:
    """Owns a taco_tensor_t and keeps every array it points to alive."""

    def __init__(self, dims, mode_types, vals=None, index_arrays=None, csize=None,
                 mode_ordering=None):
        order = len(dims)
        self._keep = []
        self.dims = (ctypes.c_int32 * order)(*dims)
        self.ordering = (ctypes.c_int32 * order)(*(mode_ordering or range(order)))
        self.types = (ctypes.c_int * order)(*mode_types)
        self.mode_arrays = []
        index_arrays = index_arrays or {}
        per_mode = (ctypes.POINTER(ctypes.c_void_p) * order)()
        for m in range(order):
            if mode_types[m] == MODE_DENSE:
                size_arr = np.array([dims[m]], dtype=np.int32)
                self._keep.append(size_arr)
                slots = (ctypes.c_void_p * 1)(size_arr.ctypes.data)
            else:
                pos, crd = index_arrays[m]
                self._keep += [pos, crd]
                slots = (ctypes.c_void_p * 2)(_ptr(pos), _ptr(crd))
            self.mode_arrays.append(slots)
            per_mode[m] = ctypes.cast(slots, ctypes.POINTER(ctypes.c_void_p))
        self.indices = per_mode
        self.vals_arr = vals
        self.fill = np.zeros(1, dtype=np.float64)
        t = N.TacoTensor()
        t.order = order
        t.dimensions = ctypes.cast(self.dims, ctypes.POINTER(ctypes.c_int32))
        t.csize = csize if csize is not None else (_csize(vals) if vals is not None else 64)
        t.mode_ordering = ctypes.cast(self.ordering, ctypes.POINTER(ctypes.c_int32))
        t.mode_types = ctypes.cast(self.types, ctypes.POINTER(ctypes.c_int))
        t.indices = ctypes.cast(per_mode, ctypes.POINTER(ctypes.POINTER(ctypes.c_void_p)))
        t.vals = _ptr(vals)
        t.fill_value = self.fill.ctypes.data
        t.vals_size = 0
        self.t = t

    @property
    def ptr(self):
        return ctypes.addressof(self.t)

    def index(self, mode, which):
        """Raw pointer stored at indices[mode][which] (e.g. after assemble)."""
        return self.mode_arrays[mode][which]

    @property
    def vals_ptr(self):
        return self.t.vals


def csr(pos, crd, vals, dims):
    return TacoTensor(dims, [MODE_DENSE, MODE_SPARSE], vals=vals, index_arrays={1: (pos, crd)})


def dense(vals, dims):
    return TacoTensor(dims, [MODE_DENSE] * len(dims), vals=vals)


def dense_result(dims, csize=64):
    """A dense result whose vals are allocated by assemble."""
    return TacoTensor(dims, [MODE_DENSE] * len(dims), vals=None, csize=csize)


def csr_result(dims, csize=64):
    """A CSR result whose pos/crd/vals are allocated by assemble."""
    t = TacoTensor(dims, [MODE_DENSE, MODE_SPARSE], vals=None, csize=csize,
                   index_arrays={1: (None, None)})
    return t


def csf3(dims, crd0, pos1, crd1, pos2, crd2, vals, dense0=False):
    """An order-3 {Sparse,Sparse,Sparse} tensor ({Dense,Sparse,Sparse} with dense0, crd0 then
    unused): level 0 pos {0, len(crd0)} and crd0, level 1 pos1/crd1, level 2 pos2/crd2."""
    n0 = (crd0.shape[0] if hasattr(crd0, "shape") else len(crd0))
    pos0 = np.array([0, n0], np.int32)
    types = [MODE_DENSE if dense0 else MODE_SPARSE, MODE_SPARSE, MODE_SPARSE]
    idx = {1: (pos1, crd1), 2: (pos2, crd2)}
    if not dense0:
        idx[0] = (pos0, crd0)
    t = TacoTensor(list(dims), types, vals=vals, index_arrays=idx)
    t._keep.append(pos0)
    return t
