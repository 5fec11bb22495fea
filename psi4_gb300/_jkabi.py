"""ctypes signatures of libgdfjk.so (include/gdfjk.h)."""
import ctypes

P = ctypes.c_void_p
I = ctypes.c_int
D = ctypes.c_double
SZ = ctypes.c_size_t

# name -> (restype, argtypes); the list is the whole exported C ABI of include/gdfjk.h
SIGNATURES = {
    "gdfjk_create": (I, [I, I, I, P, I, ctypes.POINTER(P)]),
    "gdfjk_upload_B": (I, [P, P, I, P, P, P]),
    "gdfjk_upload_B_device": (I, [P, P]),
    "gdfjk_upload_B_block": (I, [P, P, I, I]),
    "gdfjk_upload_B_device_block": (I, [P, P, I, I]),
    "gdfjk_trim": (I, [P]),
    "gdfjk_metric_contract_device": (I, [P, P, P, I, ctypes.c_int64, P, ctypes.c_int64, I]),
    "gdfjk_gemm_device": (I, [P, I, I, I, I, P, ctypes.c_int64, P, ctypes.c_int64, P, ctypes.c_int64, I]),
    "gdfjk_basis_create": (I, [I, I, P, P, P, P, P, P, P, I, ctypes.POINTER(P)]),
    "gdfjk_basis_destroy": (None, [P]),
    "gdfjk_basis_nbf": (I, [P]),
    "gdfjk_three_index_device": (I, [P, P, P, I, I, P, ctypes.c_int64, P, P]),
    "gdfjk_metric_device": (I, [P, I, I, ctypes.c_int64, P, P]),
    "gdfjk_three_index_grad_device": (I, [P, P, P, P, P, ctypes.c_int64, I, P, P]),
    "gdfjk_metric_grad_device": (I, [P, P, ctypes.c_int64, I, P, P]),
    "gdfjk_potential_grad_device": (I, [P, P, I, P, P, P, P]),
    "gdfjk_compute": (I, [P, P, P, I, I, I, P, P, P]),
    "gdfjk_compute_device": (I, [P, P, P, I, I, I, P, P, P]),
    "gdfjk_compute_wK": (I, [P, P, P, P, I, I, I, P]),
    "gdfjk_compute_incremental": (I, [P, P, I, I, P, I, I, I, I, P, P]),
    "gdfjk_compute_incremental_device": (I, [P, P, I, I, P, I, I, I, I, P, P]),
    "gdfjk_backward": (I, [P, P, I, I, P, P, P, P, I]),
    "gdfjk_backward_gamma_device": (I, [P, P, I, I, P, P, P, ctypes.c_int64, P, I]),
    "gdfjk_query_memory": (I, [I, I, I, I, ctypes.POINTER(SZ)]),
    "gdfjk_last_timings": (I, [P, ctypes.POINTER(D), ctypes.POINTER(D), ctypes.POINTER(D)]),
    "gdfjk_synchronize": (I, [P, D]),
    "gdfjk_stream": (P, [P]),
    "gdfjk_coulomb_noalloc": (I, [I, I, P, P, P, P]),
    "gdfjk_debug_refuse_allocations": (I, [I, I]),
    "gdfjk_debug_wait_probe": (I, [P, D]),
    "gdfjk_destroy": (I, [P]),
    "gdfjk_last_error": (ctypes.c_char_p, [P]),
}

GDFJK_OK = 0
GDFJK_ERR_ARG = -1
GDFJK_ERR_CUDA = -2
GDFJK_ERR_OOM = -3
GDFJK_ERR_STATE = -4
GDFJK_ERR_TIMEOUT = -5
GDFJK_ERR_NUMERIC = -6
GDFJK_ERR_DEVICE = -7

B_HOST = 256  # gdfjk_create flag: B in pinned Grace memory, read over NVLink-C2C

LAYOUT_PQQ = 0
LAYOUT_QTRI = 1

DO_J = 1
DO_K = 2
MIXED = 4
INCREMENTAL = 8
RESET = 16
EMULATED = 32

NOALLOC_MAX_NAUX = 65536


def declare(L):
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
