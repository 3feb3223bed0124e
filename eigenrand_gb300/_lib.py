"""ctypes binding to libgpurand.so (include/gpurand.h).

There is no fallback: if the library is missing the import fails with a
message that says how to build it.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgpurand.so")

GR_OK = 0
STATUS_NAMES = {
    0: "GR_OK", 1: "GR_ERR_INVALID", 2: "GR_ERR_CUDA", 3: "GR_ERR_UNSUPPORTED", 4: "GR_ERR_NOMEM",
    5: "GR_ERR_REJECT_LIMIT", 6: "GR_ERR_NOT_PD", 7: "GR_ERR_NAN_WEIGHT", 8: "GR_ERR_CANCELLED",
}

# gr_dtype
F32, F64, I32, U64 = 0, 1, 2, 3

# gr_dist_kind
KINDS = dict(
    UNIFORM_REAL=1, UNIFORM_REAL2=2, BALANCED=3, BALANCED2=4, NORMAL_STD=5, NORMAL=6, LOGNORMAL=7,
    EXPONENTIAL=8, CAUCHY=9, WEIBULL=10, EXTREME_VALUE=11, GAMMA=12, BETA=13, STUDENT_T=14,
    CHI_SQUARED=15, POISSON=16, BINOMIAL=17, DISCRETE=18, RANDBITS=19, BINOMIAL_V=20, BERNOULLI=21,
    GEOMETRIC=22, FISHER_F=23, UNIFORM_INT=24, NEGATIVE_BINOMIAL=25,
)

# exported symbols, as declared in include/gpurand.h
EXPORTS = [
    "gr_engine_create", "gr_engine_destroy", "gr_engine_seed", "gr_engine_state_size", "gr_engine_save",
    "gr_engine_restore", "gr_engine_discard", "gr_engine_sync", "gr_engine_streams", "gr_raw_u64",
    "gr_gen_create", "gr_gen_destroy", "gr_generate", "gr_sample", "gr_sample_batched", "gr_last_error",
    "gr_version", "gr_raw_u64_noalloc", "gr_sample_v", "gr_gen_create_truncated", "gr_sample_truncated",
    "gr_sample_v2", "gr_generate_v",
    "gr_sengine_create", "gr_sengine_destroy", "gr_sengine_raw_u64", "gr_sengine_sample", "gr_sengine_sample_v2",
    "gr_mvnormal_create", "gr_mvnormal_sample", "gr_mvnormal_destroy", "gr_wishart_create", "gr_wishart_sample",
    "gr_wishart_destroy", "gr_dirichlet_create", "gr_dirichlet_sample", "gr_dirichlet_destroy",
    "gr_multinomial_create", "gr_multinomial_sample", "gr_multinomial_destroy",
    "gr_truncmvn_create", "gr_truncmvn_sample", "gr_truncmvn_destroy",
    "gr_server_create", "gr_server_set_mvnormal", "gr_server_submit", "gr_server_progress", "gr_server_read",
    "gr_server_release", "gr_server_cancel", "gr_server_cancel_client", "gr_server_fail_allocs", "gr_server_pending",
    "gr_server_now", "gr_server_destroy",
]

GR_SERVE_MVNORMAL = 64


class Request(ctypes.Structure):
    _fields_ = [
        ("client", ctypes.c_int32),
        ("kind", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("trials", ctypes.c_int32),
        ("a", ctypes.c_double),
        ("b", ctypes.c_double),
        ("count", ctypes.c_uint64),
        ("arrival", ctypes.c_double),
    ]


class Completion(ctypes.Structure):
    _fields_ = [
        ("ticket", ctypes.c_uint64),
        ("status", ctypes.c_int32),
        ("client", ctypes.c_int32),
        ("dev_out", ctypes.c_void_p),
        ("count", ctypes.c_uint64),
        ("bytes", ctypes.c_size_t),
        ("arrival", ctypes.c_double),
        ("admitted", ctypes.c_double),
        ("completed", ctypes.c_double),
    ]


class BatchDesc(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("nsets", ctypes.c_int64),
        ("seed", ctypes.c_uint64),
        ("a", ctypes.c_void_p),
        ("b", ctypes.c_void_p),
        ("trials", ctypes.c_void_p),
        ("counts", ctypes.c_void_p),
        ("offsets", ctypes.c_void_p),
        ("out", ctypes.c_void_p),
    ]


class DistDesc(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("a", ctypes.c_double),
        ("b", ctypes.c_double),
        ("trials", ctypes.c_int32),
        ("nweights", ctypes.c_int32),
        ("weights", ctypes.POINTER(ctypes.c_double)),
    ]


class GrError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_lib = None


def load(path=None):
    """Load libgpurand.so (once)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("GPURAND_LIB", LIB_PATH)
    if not os.path.exists(path):
        raise ImportError(
            f"libgpurand.so not found at {path}; build it with `python eigenrand_gb300/build.py` "
            "(the sampling library has no CPU fallback)")
    lib = ctypes.CDLL(path)
    vp, sz, i32, u64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int32, ctypes.c_uint64
    sig = {
        "gr_engine_create": (i32, [ctypes.POINTER(vp), u64, i32, i32]),
        "gr_engine_destroy": (i32, [vp]),
        "gr_engine_seed": (i32, [vp, u64, vp]),
        "gr_engine_state_size": (sz, [vp]),
        "gr_engine_save": (i32, [vp, vp, sz, vp]),
        "gr_engine_restore": (i32, [vp, vp, sz, vp]),
        "gr_engine_discard": (i32, [vp, u64, vp]),
        "gr_engine_sync": (i32, [vp, vp]),
        "gr_engine_streams": (i32, [vp]),
        "gr_raw_u64": (i32, [vp, vp, sz, vp]),
        "gr_gen_create": (i32, [ctypes.POINTER(vp), ctypes.POINTER(DistDesc)]),
        "gr_gen_destroy": (i32, [vp]),
        "gr_generate": (i32, [vp, vp, vp, sz, vp]),
        "gr_sample": (i32, [vp, ctypes.POINTER(DistDesc), vp, sz, vp]),
        "gr_raw_u64_noalloc": (i32, [vp, vp, sz, vp]),
        "gr_sample_batched": (i32, [vp, ctypes.POINTER(BatchDesc), vp]),
        "gr_sample_v": (i32, [vp, ctypes.POINTER(DistDesc), vp, vp, sz, vp]),
        "gr_sample_v2": (i32, [vp, ctypes.POINTER(DistDesc), vp, vp, vp, sz, vp]),
        "gr_sengine_create": (i32, [ctypes.POINTER(vp), i32, ctypes.c_uint64]),
        "gr_sengine_destroy": (i32, [vp]),
        "gr_sengine_raw_u64": (i32, [vp, vp, sz, vp]),
        "gr_sengine_sample": (i32, [vp, ctypes.POINTER(DistDesc), vp, sz, vp]),
        "gr_sengine_sample_v2": (i32, [vp, ctypes.POINTER(DistDesc), vp, vp, vp, sz, vp]),
        "gr_generate_v": (i32, [vp, vp, vp, vp, vp, sz, vp]),
        "gr_gen_create_truncated": (i32, [ctypes.POINTER(vp), ctypes.POINTER(DistDesc), ctypes.c_double,
                                          ctypes.c_double]),
        "gr_sample_truncated": (i32, [vp, ctypes.POINTER(DistDesc), ctypes.c_double, ctypes.c_double, vp, sz, vp]),
        "gr_mvnormal_create": (i32, [ctypes.POINTER(vp), i32, i32, vp, vp, i32]),
        "gr_mvnormal_sample": (i32, [vp, vp, vp, sz, vp]),
        "gr_mvnormal_destroy": (i32, [vp]),
        "gr_wishart_create": (i32, [ctypes.POINTER(vp), i32, i32, ctypes.c_int64, vp, i32, i32]),
        "gr_wishart_sample": (i32, [vp, vp, vp, sz, vp]),
        "gr_wishart_destroy": (i32, [vp]),
        "gr_dirichlet_create": (i32, [ctypes.POINTER(vp), i32, i32, vp]),
        "gr_dirichlet_sample": (i32, [vp, vp, vp, sz, vp]),
        "gr_dirichlet_destroy": (i32, [vp]),
        "gr_multinomial_create": (i32, [ctypes.POINTER(vp), i32, i32, vp]),
        "gr_multinomial_sample": (i32, [vp, vp, vp, sz, vp]),
        "gr_multinomial_destroy": (i32, [vp]),
        "gr_truncmvn_create": (i32, [ctypes.POINTER(vp), i32, i32, vp, vp, i32, vp, vp, ctypes.c_int64]),
        "gr_truncmvn_sample": (i32, [vp, vp, vp, sz, vp]),
        "gr_truncmvn_destroy": (i32, [vp]),
        "gr_server_create": (i32, [ctypes.POINTER(vp), i32, vp, sz, i32]),
        "gr_server_set_mvnormal": (i32, [vp, i32, vp, vp]),
        "gr_server_submit": (i32, [vp, ctypes.POINTER(Request), ctypes.POINTER(u64)]),
        "gr_server_progress": (i32, [vp, vp, sz, ctypes.POINTER(sz)]),
        "gr_server_read": (i32, [vp, u64, vp, sz]),
        "gr_server_release": (i32, [vp, u64]),
        "gr_server_cancel": (i32, [vp, u64]),
        "gr_server_cancel_client": (i32, [vp, i32]),
        "gr_server_fail_allocs": (i32, [vp, i32]),
        "gr_server_pending": (i32, [vp, ctypes.POINTER(sz), ctypes.POINTER(sz), ctypes.POINTER(sz)]),
        "gr_server_now": (ctypes.c_double, []),
        "gr_server_destroy": (i32, [vp]),
        "gr_last_error": (ctypes.c_char_p, []),
        "gr_version": (ctypes.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != GR_OK:
        msg = _lib.gr_last_error().decode(errors="replace") if _lib else ""
        raise GrError(status, msg)
