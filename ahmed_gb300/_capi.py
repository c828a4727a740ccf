"""ctypes binding of libahx.so (the C ABI declared in include/ahx.h).

The library is required: importing this module without a built libahx.so
raises, so no product call can silently run anything else.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libahx.so")

AHX_OK = 0
AHX_ERR_ARG = 1
AHX_ERR_CUDA = 2
AHX_ERR_STATE = 3
AHX_ERR_NOMEM = 4
AHX_NOT_CONVERGED = 5

TREE_BBX = 0
TREE_PCA = 1
FP64 = 0
FP32 = 1
BF16_FP32 = 2
DF64 = 3

# (name, restype, argtypes) of every exported entry point of include/ahx.h
_vp, _u32, _u64, _i32, _dbl = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_double
SIGNATURES = [
    ("ahx_last_error", C.c_char_p, []),
    ("ahx_version", _i32, []),
    ("ahx_mean_nn", _dbl, [_vp, _u32]),
    ("ahx_min_nn", _dbl, [_vp, _u32]),
    ("ahx_kernel_launches", _u64, []),
    ("ahx_hmat_create", _i32, [_vp, _u32, _i32, _u32, _dbl, _i32, _vp, _vp]),
    ("ahx_hmat_create_sym", _i32, [_vp, _u32, _i32, _u32, _dbl, _i32, _vp, _vp]),
    ("ahx_hmat_symmetric", _i32, [_vp]),
    ("ahx_hmat_destroy", _i32, [_vp]),
    ("ahx_hmat_set_stream", _i32, [_vp, _vp]),
    ("ahx_hmat_stream", _vp, [_vp]),
    ("ahx_hmat_n", _u32, [_vp]),
    ("ahx_hmat_nleaves", _u32, [_vp]),
    ("ahx_hmat_perm", _i32, [_vp, _vp, _vp]),
    ("ahx_hmat_leaves", _i32, [_vp, _vp]),
    ("ahx_assemble", _i32, [_vp, _dbl, _dbl, _u32]),
    ("ahx_hmat_ranks", _i32, [_vp, _vp]),
    ("ahx_hmat_aca_ranks", _i32, [_vp, _vp]),
    ("ahx_hmat_leaf_size", _u64, [_vp, _u32]),
    ("ahx_hmat_get_leaf", _i32, [_vp, _u32, _vp]),
    ("ahx_hmat_set_leaves", _i32, [_vp, _vp, _vp, _vp]),
    ("ahx_hmat_storage_bytes", _u64, [_vp, _i32]),
    ("ahx_hmat_prepare", _i32, [_vp, _i32]),
    ("ahx_hmat_release", _i32, [_vp, _i32]),
    ("ahx_hmat_stream_bytes", _i32, [_vp, _i32, _vp]),
    ("ahx_timing", _i32, [_i32]),
    ("ahx_timing_read", _i32, [_vp, _vp, _i32]),
    ("ahx_matvec", _i32, [_vp, _i32, _dbl, _u32, _vp, _u64, _vp, _u64]),
    ("ahx_gmres", _i32, [_vp, _i32, _u32, _vp, _u64, _vp, _u64, _dbl, _u32, _u32, _vp, _vp]),
    ("ahx_cg", _i32, [_vp, _u32, _vp, _u64, _vp, _u64, _dbl, _u32, _vp, _vp]),
    ("ahx_batch_create", _i32, [_vp, _u32, _i32, _vp]),
    ("ahx_batch_destroy", _i32, [_vp]),
    ("ahx_batch_n", _u64, [_vp]),
    ("ahx_batch_matvec", _i32, [_vp, _dbl, _u32, _vp, _vp]),
    ("ahx_batch_gmres", _i32, [_vp, _vp, _vp, _dbl, _u32, _u32, _vp, _vp]),
    ("ahx_assemble_hinted", _i32, [_vp, _dbl, _dbl, _u32, _vp]),
    ("ahx_hmat_assembly_stats", _i32, [_vp, _vp]),
    ("ahx_hmat_features", _i32, [_vp, _dbl, _dbl, _vp]),
    ("ahx_hmat_autotune", _i32, [_vp, _i32, _u32, _vp]),
    ("ahx_matvec_transposed", _i32, [_vp, _dbl, _u32, _vp, _u64, _vp, _u64]),
    ("ahx_mbls_header", _i32, [C.c_char_p, _vp, _vp, _vp]),
    ("ahx_batch_prepare", _i32, [_vp, _i32]),
    ("ahx_spctrlnrm", _i32, [_vp, _u32, _vp]),
    ("ahx_agglomerate", _i32, [_vp, _dbl, _u32, _vp]),
    ("ahx_hmat_save", _i32, [_vp, _dbl, _u32, C.c_char_p]),
    ("ahx_hmat_load", _i32, [_vp, C.c_char_p, _vp, _vp]),
    ("ahx_hmat_save_stream", _i32, [_vp, _dbl, _u32, _vp, _vp]),
    ("ahx_hmat_load_stream", _i32, [_vp, _vp, _vp, _vp, _vp]),
    ("ahx_helm_aca_ranks", _i32, [_vp, _dbl, _dbl, _dbl, _u32, _vp, _vp]),
    ("ahx_helm_assemble", _i32, [_vp, _dbl, _dbl, _dbl, _u32]),
    ("ahx_helm_ranks", _i32, [_vp, _vp]),
    ("ahx_helm_leaf_size", _u64, [_vp, _u32]),
    ("ahx_helm_get_leaf", _i32, [_vp, _u32, _vp]),
    ("ahx_helm_storage_bytes", _u64, [_vp, _i32]),
    ("ahx_helm_matvec", _i32, [_vp, _i32, _i32, _dbl, _dbl, _u32, _vp, _u64, _vp, _u64]),
    ("ahx_helm_save", _i32, [_vp, _dbl, _u32, C.c_char_p]),
    ("ahx_helm_load", _i32, [_vp, C.c_char_p, _vp, _vp]),
    ("ahx_helm_save_stream", _i32, [_vp, _dbl, _u32, _vp, _vp]),
    ("ahx_helm_load_stream", _i32, [_vp, _vp, _vp, _vp, _vp]),
    ("ahx_helm_agglomerate", _i32, [_vp, _dbl, _u32, _vp]),
    ("ahx_helm_gmres", _i32, [_vp, _i32, _u32, _vp, _u64, _vp, _u64, _dbl, _u32, _u32, _vp, _vp]),
    ("ahx_mlp_nparams", _u32, []),
    ("ahx_mlp_create", _i32, [_i32, _u64, _vp]),
    ("ahx_mlp_destroy", _i32, [_vp]),
    ("ahx_mlp_get_params", _i32, [_vp, _vp]),
    ("ahx_mlp_set_params", _i32, [_vp, _vp]),
    ("ahx_mlp_set_norm", _i32, [_vp, _vp, _vp]),
    ("ahx_mlp_gradients", _i32, [_vp, _vp, _vp, _u32, _vp, _vp]),
    ("ahx_mlp_train", _i32, [_vp, _vp, _vp, _u32, _u32, _u32, C.c_float, _u64, _vp]),
    ("ahx_mlp_predict", _i32, [_vp, _vp, _u32, _vp]),
    ("ahx_aca_block_noalloc", _i32, [_vp, _vp, _vp, _u32, _u32, _u32, _u32, _u32, _dbl, _dbl,
                                     _u32, _vp, _vp, _vp, _vp]),
]

_lib = None


class AhxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ahx error {code}: {msg}")
        self.code = code


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built (python -m ahmed_gb300.build)")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code):
    if code not in (AHX_OK, AHX_NOT_CONVERGED):
        raise AhxError(code, lib().ahx_last_error().decode(errors="replace"))
    return code


def ptr(a):
    """Address of a numpy array or a torch tensor (host or CUDA)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)
