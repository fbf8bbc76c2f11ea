"""ctypes bindings of libtacogb (include/taco_gb300.h) and libtacogb_gen
(include/taco_gb300_gen.h).

The shared objects are built in-tree by taco_gb300.build; loading fails loudly when they are
missing — there is no Python or CPU fallback for any kernel.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")

TACOGB_F64, TACOGB_F32, TACOGB_BF16 = 0, 1, 2
VARIANT_AUTO = -1


class TacoTensor(ctypes.Structure):
    """taco_tensor_t (include/taco/taco_tensor_t.h:13-23 in taco)."""
    _fields_ = [
        ("order", ctypes.c_int32),
        ("dimensions", ctypes.POINTER(ctypes.c_int32)),
        ("csize", ctypes.c_int32),
        ("mode_ordering", ctypes.POINTER(ctypes.c_int32)),
        ("mode_types", ctypes.POINTER(ctypes.c_int)),
        ("indices", ctypes.POINTER(ctypes.POINTER(ctypes.c_void_p))),
        ("vals", ctypes.c_void_p),
        ("fill_value", ctypes.c_void_p),
        ("vals_size", ctypes.c_int32),
    ]


class Csf3(ctypes.Structure):
    """tacogb_csf3: an order-3 {Sparse|Dense,Sparse,Sparse} tensor in device memory."""
    _fields_ = [
        ("dims", ctypes.c_int32 * 3),
        ("n0", ctypes.c_int32),
        ("nfib", ctypes.c_int32),
        ("nnz", ctypes.c_int64),
        ("crd0", ctypes.c_void_p),
        ("pos1", ctypes.c_void_p),
        ("crd1", ctypes.c_void_p),
        ("pos2", ctypes.c_void_p),
        ("crd2", ctypes.c_void_p),
        ("vals", ctypes.c_void_p),
        ("vtype", ctypes.c_int32),
    ]


class Dcsr(ctypes.Structure):
    """tacogb_dcsr: a {Sparse,Sparse} matrix in device memory."""
    _fields_ = [
        ("rows", ctypes.c_int32),
        ("cols", ctypes.c_int32),
        ("n0", ctypes.c_int32),
        ("nnz", ctypes.c_int64),
        ("crd0", ctypes.c_void_p),
        ("pos", ctypes.c_void_p),
        ("crd", ctypes.c_void_p),
        ("vals", ctypes.c_void_p),
        ("vtype", ctypes.c_int32),
    ]


class Csr(ctypes.Structure):
    """tacogb_csr: a CSR matrix in device memory."""
    _fields_ = [
        ("rows", ctypes.c_int32),
        ("cols", ctypes.c_int32),
        ("nnz", ctypes.c_int64),
        ("pos", ctypes.c_void_p),
        ("crd", ctypes.c_void_p),
        ("vals", ctypes.c_void_p),
        ("vtype", ctypes.c_int32),
    ]


class GenSpec(ctypes.Structure):
    """tacogb_gen_spec."""
    _fields_ = [
        ("rows", ctypes.c_int32), ("cols", ctypes.c_int32), ("kind", ctypes.c_int32),
        ("len_lo", ctypes.c_int32), ("len_hi", ctypes.c_int32),
        ("mean", ctypes.c_double), ("len_max", ctypes.c_int32),
        ("band", ctypes.c_int32), ("band_len", ctypes.c_int32), ("grid", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
    ]


_lib = None
_gen = None

P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64

# name -> (restype, argtypes); every symbol declared in include/taco_gb300.h
SIGNATURES = {
    "tacogb_last_error": (ctypes.c_char_p, []),
    "tacogb_version": (ctypes.c_char_p, []),
    "tacogb_device_status": (I32, [ctypes.POINTER(I32)]),
    "tacogb_launch_count": (ctypes.c_longlong, []),
    "tacogb_profile_begin": (None, []),
    "tacogb_profile_end": (I32, [I32, P, P, P]),
    "tacogb_profile_enable": (None, [I32]),
    "tacogb_set_validation": (I32, [I32]),
    "tacogb_validate_level_host": (I32, [I64, I32, P, P, I64]),
    "tacogb_csr_validate": (I32, [P, P]),
    "tacogb_pack_csr": (I32, [I32, I32, I64, P, P, P, I32, P, P, P, P, P]),
    "tacogb_pack_taco": (I32, [P, P, I64]),
    "tacogb_read_rb": (I32, [ctypes.c_char_p, ctypes.POINTER(I32), ctypes.POINTER(I32),
                             ctypes.POINTER(I64), ctypes.POINTER(P), ctypes.POINTER(P),
                             ctypes.POINTER(P)]),
    "tacogb_read_coo": (I32, [ctypes.c_char_p, P, P, P, P, P, P]),
    "tacogb_free_host": (None, [P]),
    "tacogb_spmv": (I32, [ctypes.POINTER(Csr), P, P, I32, P]),
    "tacogb_spmv_variant_count": (I32, []),
    "tacogb_spmv_variant_name": (ctypes.c_char_p, [I32]),
    "tacogb_spmv_auto_variant": (I32, [P, P]),
    "tacogb_spmv_noalloc": (I32, [ctypes.POINTER(Csr), P, P, P]),
    "tacogb_spmv_assemble": (I32, [P, P, P]),
    "tacogb_spmv_compute": (I32, [P, P, P]),
    "tacogb_spmv_evaluate": (I32, [P, P, P]),
    "_shim_tacogb_spmv_assemble": (I32, [P]),
    "_shim_tacogb_spmv_compute": (I32, [P]),
    "_shim_tacogb_spmv_evaluate": (I32, [P]),
    "tacogb_batch_create": (I32, [I32, ctypes.POINTER(Csr), P, P, I32, P, ctypes.POINTER(P)]),
    "tacogb_batch_spmm_create": (I32, [I32, ctypes.POINTER(Csr), I32, P, I32, P, I32,
                                        ctypes.POINTER(P)]),
    "tacogb_batch_run": (I32, [P, P]),
    "tacogb_batch_destroy": (I32, [P]),
    "tacogb_batch_matrix_cycles": (I32, [P, P, P]),
    "tacogb_batch_variant_count": (I32, []),
    "tacogb_batch_variant_name": (ctypes.c_char_p, [I32]),
    "tacogb_mlp_param_count": (I32, []),
    "tacogb_batch_features": (I32, [I32, ctypes.POINTER(Csr), P, P]),
    "tacogb_mlp_predict": (I32, [P, P, P, I32, P, P, P]),
    "tacogb_mlp_grad": (I32, [P, P, P, P, P, I32, P, P, P]),
    "tacogb_mlp_train": (I32, [P, P, P, P, P, I32, I32, I32, ctypes.c_float, P, P, P]),
    "tacogb_batch_autotune": (I32, [I32, ctypes.POINTER(Csr), P, P, I32, I32, P, P, P]),
    "tacogb_batch_select": (I32, [I32, ctypes.POINTER(Csr), P, P, P, P]),
    "tacogb_spmm": (I32, [ctypes.POINTER(Csr), I32, P, I32, P, I32, P]),
    "tacogb_sddmm": (I32, [ctypes.POINTER(Csr), I32, P, P, P, I32, P]),
    "tacogb_sddmm_dense": (I32, [ctypes.POINTER(Csr), I32, P, P, P, I64, I32, P]),
    "tacogb_sddmm_variant_count": (I32, []),
    "tacogb_sddmm_variant_name": (ctypes.c_char_p, [I32]),
    "tacogb_sddmm_assemble": (I32, [P, P, P, P]),
    "tacogb_sddmm_compute": (I32, [P, P, P, P]),
    "tacogb_sddmm_evaluate": (I32, [P, P, P, P]),
    "_shim_tacogb_sddmm_assemble": (I32, [P]),
    "_shim_tacogb_sddmm_compute": (I32, [P]),
    "_shim_tacogb_sddmm_evaluate": (I32, [P]),
    "tacogb_spmv_dcsr": (I32, [ctypes.POINTER(Dcsr), P, P, I32, P]),
    "tacogb_spmm_dcsr": (I32, [ctypes.POINTER(Dcsr), I32, P, P, P]),
    "tacogb_spmv_csc": (I32, [ctypes.POINTER(Csr), P, P, P]),
    "tacogb_csc_to_csr": (I32, [I32, I32, I64, P, P, P, I32, P, P, P, P]),
    "tacogb_densify": (I32, [I32, I64, P, P, I32, P, P]),
    "tacogb_ttv": (I32, [ctypes.POINTER(Csf3), P, P, I32, P]),
    "tacogb_ttv_dense": (I32, [ctypes.POINTER(Csf3), P, P, I32, P]),
    "tacogb_ttm": (I32, [ctypes.POINTER(Csf3), I32, P, P, I32, P]),
    "tacogb_ttm_dense": (I32, [ctypes.POINTER(Csf3), I32, P, P, I32, P]),
    "tacogb_mttkrp": (I32, [ctypes.POINTER(Csf3), I32, P, P, P, I32, P]),
    "tacogb_ttv_assemble": (I32, [P, P, P]),
    "tacogb_ttv_compute": (I32, [P, P, P]),
    "tacogb_ttv_evaluate": (I32, [P, P, P]),
    "tacogb_ttm_assemble": (I32, [P, P, P]),
    "tacogb_ttm_compute": (I32, [P, P, P]),
    "tacogb_ttm_evaluate": (I32, [P, P, P]),
    "tacogb_mttkrp_assemble": (I32, [P, P, P, P]),
    "tacogb_mttkrp_compute": (I32, [P, P, P, P]),
    "tacogb_mttkrp_evaluate": (I32, [P, P, P, P]),
    "_shim_tacogb_ttv_assemble": (I32, [P]),
    "_shim_tacogb_ttv_compute": (I32, [P]),
    "_shim_tacogb_ttv_evaluate": (I32, [P]),
    "_shim_tacogb_ttm_assemble": (I32, [P]),
    "_shim_tacogb_ttm_compute": (I32, [P]),
    "_shim_tacogb_ttm_evaluate": (I32, [P]),
    "_shim_tacogb_mttkrp_assemble": (I32, [P]),
    "_shim_tacogb_mttkrp_compute": (I32, [P]),
    "_shim_tacogb_mttkrp_evaluate": (I32, [P]),
    "tacogb_spmm_variant_count": (I32, []),
    "tacogb_spmm_variant_name": (ctypes.c_char_p, [I32]),
    "tacogb_spmm_assemble": (I32, [P, P, P]),
    "tacogb_spmm_compute": (I32, [P, P, P]),
    "tacogb_spmm_evaluate": (I32, [P, P, P]),
    "_shim_tacogb_spmm_assemble": (I32, [P]),
    "_shim_tacogb_spmm_compute": (I32, [P]),
    "_shim_tacogb_spmm_evaluate": (I32, [P]),
    "tacogb_spgemm_symbolic": (I32, [ctypes.POINTER(Csr), ctypes.POINTER(Csr), P,
                                      ctypes.POINTER(I64), P]),
    "tacogb_spgemm_fill": (I32, [ctypes.POINTER(Csr), ctypes.POINTER(Csr), P, P, P]),
    "tacogb_spgemm_numeric": (I32, [ctypes.POINTER(Csr), ctypes.POINTER(Csr), P, P, P, P]),
    "tacogb_spgemm_onepass": (I32, [ctypes.POINTER(Csr), ctypes.POINTER(Csr), P,
                                    ctypes.POINTER(I64), P]),
    "tacogb_spgemm_onepass_finish": (I32, [P, P, P, P]),
    "tacogb_spgemm_assemble": (I32, [P, P, P]),
    "tacogb_spgemm_compute": (I32, [P, P, P]),
    "tacogb_spgemm_evaluate": (I32, [P, P, P]),
    "_shim_tacogb_spgemm_assemble": (I32, [P]),
    "_shim_tacogb_spgemm_compute": (I32, [P]),
    "_shim_tacogb_spgemm_evaluate": (I32, [P]),
}

GEN_SIGNATURES = {
    "tacogb_gen_pos": (I64, [ctypes.POINTER(GenSpec), P]),
    "tacogb_gen_fill": (I32, [ctypes.POINTER(GenSpec), P, P, P]),
    "tacogb_gen_dense": (None, [ctypes.c_uint64, I64, P]),
    "tacogb_gen_powerlaw_scale": (ctypes.c_double, [ctypes.c_double, I32]),
    "tacogb_gen_batch_spec": (None, [ctypes.c_uint64, I32, I32, I32, ctypes.POINTER(GenSpec)]),
}


def _bind(lib, sigs):
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def lib():
    """The loaded libtacogb (raises if it was not built)."""
    global _lib
    if _lib is None:
        path = os.path.join(LIBDIR, "libtacogb.so")
        if not os.path.exists(path):
            raise RuntimeError("libtacogb.so is not built (run taco_gb300.build.build())")
        _lib = ctypes.CDLL(path)
        _bind(_lib, SIGNATURES)
    return _lib


# include/taco_gb300_probe.h (libtacogb_probe.so, loaded by the benchmark only)
PROBE_SIGNATURES = {
    "tacogb_probe_gather": (I32, [P, I64, P, I64, P, I64, I32, I32, I32, P]),
    "tacogb_probe_wait_timeout": (I32, [P, P, I32, P]),
}
_probe = None


def probe():
    """The random-gather probe library (a measurement the benchmark uses; not libtacogb)."""
    global _probe
    if _probe is None:
        lib()
        _probe = ctypes.CDLL(os.path.join(LIBDIR, "libtacogb_probe.so"))
        _bind(_probe, PROBE_SIGNATURES)
    return _probe


_gen_path = None


def set_generator_library(path):
    """Loads the generators from another build of the same source (the oracle builds its own
    copy, so that a process timing taco's code maps no library of this package)."""
    global _gen, _gen_path
    _gen, _gen_path = None, path


def gen():
    global _gen
    if _gen is None:
        path = _gen_path or os.path.join(LIBDIR, "libtacogb_gen.so")
        if not os.path.exists(path):
            raise RuntimeError("libtacogb_gen.so is not built (run taco_gb300.build.build())")
        _gen = ctypes.CDLL(path)
        _bind(_gen, GEN_SIGNATURES)
    return _gen


class TacoGBError(RuntimeError):
    pass


def check(rc, what=""):
    if rc != 0:
        msg = lib().tacogb_last_error().decode()
        raise TacoGBError("%s failed (code %d): %s" % (what, rc, msg))
    return rc
