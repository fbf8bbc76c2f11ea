"""taco's own API into the drop-in modules.

The fixtures tests/golden/taco_dropin_<p>.npz hold what genuine taco passed through its kernel
ABI when taco::Tensor<double> statements for SpMV, SpMM and SpGEMM were compiled with
TensorBase::compileSource and the forwarding source of INTEGRATION.md (src/tensor.cpp:905-930),
then assembled and computed (src/tensor.cpp:808-850): the argument packs of the assemble and
the compute calls, as taco built them (tests/cpp/taco_dropin.cpp, made by
tests/golden/make_golden.py dropin_cases), and taco's own result for the statement.  Here the
same packs go into libtacogb_<p>.so's _shim_assemble and _shim_compute in the packed form
ir::Module::callFuncPackedRaw uses (src/codegen/module.cpp:182-218), and the result is compared
with taco's: pos and crd exact, values within 1e-12 normwise (SpGEMM bit for bit).
"""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import taco_gb300 as tg  # noqa: E402
from tests.helpers import arrays_to_taco, normwise  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _module(p):
    L = ctypes.CDLL(os.path.join(os.path.dirname(tg.__file__), "lib", "libtacogb_%s.so" % p))
    for fn in ("_shim_assemble", "_shim_compute"):
        getattr(L, fn).argtypes = [ctypes.c_void_p]
        getattr(L, fn).restype = ctypes.c_int
    return L


def _pack(*tensors):
    return (ctypes.c_void_p * len(tensors))(*[t.ptr for t in tensors])


def _same_operands(g, k):
    keys = [x for x in g.files if x.startswith("a%d_" % k)]
    for key in keys:
        assert np.array_equal(g[key], g["c" + key[1:]]), key


@pytest.mark.parametrize("p", ["spmv", "spmm", "spgemm"])
def test_taco_packs_through_dropin_module(p):
    g = np.load(os.path.join(GOLDEN, "taco_dropin_%s.npz" % p))
    # taco passed the same operands to assemble and compute
    _same_operands(g, 1)
    _same_operands(g, 2)
    R = arrays_to_taco(g, "a0", with_arrays=False)  # the result as taco passes it to assemble
    A, B = arrays_to_taco(g, "a1"), arrays_to_taco(g, "a2")
    L = _module(p)
    assert L._shim_assemble(_pack(R, A, B)) == 0, tg.lib().tacogb_last_error()
    assert L._shim_compute(_pack(R, A, B)) == 0, tg.lib().tacogb_last_error()
    t = R.t
    if p == "spgemm":
        rows = t.dimensions[0]
        pos = np.ctypeslib.as_array(ctypes.cast(R.index(1, 0), ctypes.POINTER(ctypes.c_int32)),
                                    (rows + 1,)).copy()
        nnz = int(pos[-1])
        crd = np.ctypeslib.as_array(ctypes.cast(R.index(1, 1), ctypes.POINTER(ctypes.c_int32)),
                                    (nnz,)).copy()
        vals = np.ctypeslib.as_array(ctypes.cast(t.vals, ctypes.POINTER(ctypes.c_double)),
                                     (nnz,)).copy()
        assert np.array_equal(pos, g["e_pos1"]) and np.array_equal(crd, g["e_crd1"])
        assert np.array_equal(vals, g["e_vals"])
    else:
        count = int(np.prod([t.dimensions[m] for m in range(t.order)]))
        vals = np.ctypeslib.as_array(ctypes.cast(t.vals, ctypes.POINTER(ctypes.c_double)),
                                     (count,)).copy()
        assert normwise(vals, g["e_vals"]) <= 1e-12
