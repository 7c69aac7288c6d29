"""ctypes binding of ``libhh_dmrg.so`` (the C ABI declared in include/hh_dmrg.h).

This is the same binding a Python caller of the reference's hot path would
write; it loads the in-tree library and raises if it is missing: there is no
CPU fallback for any entry point.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhh_dmrg.so")

HH_OK = 0
# status codes (include/hh_dmrg.h)
HH_ERR_INVALID, HH_ERR_CUDA, HH_ERR_NOMEM, HH_ERR_QN = -1, -2, -3, -4
HH_ERR_TIMEOUT, HH_ERR_NUMERIC, HH_ERR_UNSUPPORTED = -5, -6, -7
HH_PREC_FP64 = 0
HH_PREC_BF16X6 = 1  # three BF16 parts, six products: ~2^-24 per product
HH_PREC_BF16X3 = 2  # two BF16 parts, three products: ~2^-16 per product
HH_PREC_FP32 = 3  # FP32 arithmetic: the wave transform's guess only (hh_ctx_set_transform_precision)
HH_PREC_FP32X2 = 4  # double-float on the FP32 pipe (~2^-47): the split Lanczos's restart product
HH_EIG_OWN, HH_EIG_CUSOLVER = 0, 1  # density-matrix eigensolver (hh_ctx_set_eigensolver)
HH_TILE_SHAPES, HH_TUNE_VARIANTS = 4, 16  # stage-2 tile shapes / timings of hh_plan_tune
HH_PLAN_STATS = 24  # doubles written by hh_plan_stats

STATUS = {0: "ok", -1: "invalid argument", -2: "CUDA error", -3: "out of memory",
          -4: "quantum number mismatch", -5: "bounded device wait timed out",
          -6: "numerical failure", -7: "unsupported"}

# term kinds (enum hh_term_kind)
BLOCK_VEC_DIA = 1
VEC_BLOCK_DIA = 2
SITE_VEC_SITE_DIA = 3
SITE_VEC_SITE_NDIA = 4
BLOCK_SITE_VEC_NDIA = 5
VEC_BLOCK_SITE_NDIA = 6
BLOCK_VEC_SITE_NDIA = 7
SITE_VEC_BLOCK_NDIA = 8
BLOCK_VEC_BLOCK_NDIA = 9
BLOCK_SITE_VEC_DIA = 10
VEC_BLOCK_SITE_DIA = 11
BLOCK_VEC_SITE_DIA = 12
SITE_VEC_BLOCK_DIA = 13
BLOCK_VEC_BLOCK_DIA = 14


class HHTerm(C.Structure):
    _fields_ = [("kind", C.c_int), ("flag0", C.c_int), ("flag1", C.c_int),
                ("trans0", C.c_int), ("trans1", C.c_int),
                ("op0", C.c_void_p), ("op1", C.c_void_p),
                ("coef_re", C.c_double), ("coef_im", C.c_double)]


P = C.c_void_p
PP = C.POINTER(C.c_void_p)
I = C.c_int
D = C.c_double
IP = C.POINTER(C.c_int)
DP = C.POINTER(C.c_double)
LLP = C.POINTER(C.c_longlong)
FP = C.POINTER(C.c_float)

# name -> (restype, argtypes); every symbol declared in include/hh_dmrg.h
SIGNATURES = {
    "hh_init": (I, [I, PP]),
    "hh_finalize": (I, [P]),
    "hh_last_error": (C.c_char_p, [P]),
    "hh_status_string": (C.c_char_p, [I]),
    "hh_ctx_stream": (I, [P, PP]),
    "hh_ctx_sync": (I, [P]),
    "hh_version": (I, []),
    "hh_ctx_set_eigensolver": (I, [P, I]),
    "hh_ctx_set_transform_precision": (I, [P, I]),
    "hh_ctx_set_restart_precision": (I, [P, I]),
    "hh_ctx_set_renormalize_precision": (I, [P, I]),
    "hh_ctx_set_krylov_storage": (I, [P, I]),
    "hh_eig_selftest": (I, [P, I, DP, DP, DP]),
    "hh_block_create": (I, [P, I, I, I, I, IP, DP, PP]),
    "hh_block_zeros": (I, [P, I, I, I, I, IP, PP]),
    "hh_block_info": (I, [P, IP, IP, IP, IP, LLP]),
    "hh_block_qn": (I, [P, IP]),
    "hh_block_download": (I, [P, DP]),
    "hh_block_free": (I, [P]),
    "hh_block_add": (I, [P, DP, P]),
    "hh_basis_create": (I, [P, I, I, IP, IP, PP]),
    "hh_basis_free": (I, [P]),
    "hh_wave_create": (I, [P, I, I, I, IP, I, PP]),
    "hh_wave_info": (I, [P, LLP, IP]),
    "hh_wave_upload": (I, [P, DP]),
    "hh_wave_download": (I, [P, DP]),
    "hh_wave_copy": (I, [P, P]),
    "hh_wave_free": (I, [P]),
    "hh_wave_dot": (I, [P, P, DP]),
    "hh_wave_norm": (I, [P, DP]),
    "hh_wave_normalize": (I, [P]),
    "hh_plan_create": (I, [P, P, P, P, I, C.POINTER(HHTerm), PP]),
    "hh_plan_stats": (I, [P, DP]),
    "hh_plan_free": (I, [P]),
    "hh_matvec": (I, [P, P, P, I]),
    "hh_matvec_host": (I, [P, DP, DP, I]),
    "hh_lanczos": (I, [P, P, D, I, I, DP, IP]),
    "hh_plan_tune": (I, [P, I, I, DP, IP]),
    "hh_plan_set_tiles": (I, [P, I]),
    "hh_matvec_async": (I, [P, P, P, I]),
    "hh_plan_check": (I, [P]),
    "hh_matvec_timed": (I, [P, P, P, I, C.POINTER(C.c_float)]),
    "hh_matvec_noalloc": (I, [P, P, P]),
    "hh_tc_selftest": (I, [P, I, I, I, DP, DP, DP, I]),
    "hh_tc_selftest_hold": (I, [P, I]),
    "hh_density_truncate": (I, [P, P, I, I, I, D, PP, IP, DP, DP, DP]),
    "hh_enlarge_operator": (I, [P, I, P, P, I, I, PP]),
    "hh_ham_add_bond": (I, [P, P, P, P, I, P, DP, I, I]),
    "hh_block_product": (I, [P, P, P, I, P, DP, PP]),
    "hh_ham_add_product": (I, [P, P, P, P, DP]),
    "hh_block_copy": (I, [P, P, PP]),
    "hh_wave_random": (I, [P, C.c_ulonglong]),
    "hh_renormalize": (I, [P, P, P, I, PP]),
    "hh_wave_transform": (I, [P, I, P, P, P, P, P, P]),
    "hh_mlp_create": (I, [P, I, C.c_ulonglong, PP]),
    "hh_mlp_free": (I, [P]),
    "hh_mlp_nparams": (I, [P, IP]),
    "hh_mlp_get_params": (I, [P, FP]),
    "hh_mlp_set_params": (I, [P, FP]),
    "hh_mlp_forward": (I, [P, FP, I, FP]),
    "hh_mlp_loss_grad": (I, [P, FP, FP, FP, I, FP, FP]),
    "hh_mlp_train": (I, [P, FP, FP, FP, I, I, C.c_float, FP]),
    "hh_wave_sector_norms": (I, [P, DP]),
    "hh_wave_scale_sectors": (I, [P, DP]),
    "hh_host_alloc": (I, [C.c_longlong, PP]),
    "hh_host_free": (I, [P]),
}

_lib = None


class HHError(RuntimeError):
    def __init__(self, status, msg=""):
        super().__init__(f"{STATUS.get(status, status)} ({status}): {msg}")
        self.status = status


def load(path=LIB_PATH):
    """Load the library once; raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with hofstadter_hubbard_tsc_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, ctx=None):
    if status != HH_OK:
        msg = ""
        if ctx is not None and _lib is not None:
            m = _lib.hh_last_error(ctx)
            msg = m.decode() if m else ""
        raise HHError(status, msg)
