"""ctypes binding to the CPU oracle (oracle/_build/liboracle.so).

ORACLE — test infrastructure.  Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use this module; the sampling library never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
PIN = os.path.join(HERE, "_build", "pin_mt")

OR_UNIFORM, OR_BALANCED, OR_NORMAL, OR_LOGNORMAL, OR_EXPONENTIAL, OR_CAUCHY = 1, 2, 3, 4, 5, 6
OR_WEIBULL, OR_EXTREME, OR_GAMMA, OR_BETA, OR_STUDENT_T, OR_CHI_SQUARED, OR_STDNORMAL = 7, 8, 9, 10, 11, 12, 13


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        L.or_vmt_new.restype = vp
        L.or_vmt_new.argtypes = [ctypes.c_uint64, ctypes.c_int]
        L.or_vmt_free.argtypes = [vp]
        L.or_vmt_copy.argtypes = [vp, vp]
        L.or_vmt_sizeof.restype = sz
        L.or_gen_sizeof.restype = sz
        L.or_vmt_raw.argtypes = [vp, vp, sz]
        L.or_vmt_discard.argtypes = [vp, ctypes.c_uint64]
        L.or_vmt_window.argtypes = [vp, vp]
        L.or_gen_real.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, vp, sz]
        L.or_gen_real.restype = ctypes.c_int
        L.or_gen_binomial.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_double, vp, sz]
        L.or_gen_binomial.restype = ctypes.c_int
        L.or_gen_poisson.argtypes = [vp, vp, ctypes.c_double, vp, sz]
        L.or_gen_poisson.restype = ctypes.c_int
        L.or_gen_randbits.argtypes = [vp, vp, sz]
        L.or_gen_randbits.restype = ctypes.c_int
        L.or_discrete_new.restype = vp
        L.or_discrete_new.argtypes = [vp, ctypes.c_int]
        L.or_discrete_free.argtypes = [vp]
        L.or_discrete_table.argtypes = [vp, vp, vp, ctypes.c_int]
        L.or_discrete_table.restype = ctypes.c_int
        L.or_gen_discrete.argtypes = [vp, vp, vp, vp, sz]
        L.or_gen_discrete.restype = ctypes.c_int
        L.or_vop_set.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                 vp, sz]
        L.or_vop_set.restype = ctypes.c_int
        for name in ("or_vec_logf", "or_vec_expf", "or_vec_log", "or_vec_exp"):
            getattr(L, name).argtypes = [vp, vp, sz]
        L.or_vec_sincosf.argtypes = [vp, vp, vp, sz]
        L.or_vec_sincos.argtypes = [vp, vp, vp, sz]
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


class Engine:
    """Vmt19937_64 (4 lanes) emulated on the CPU."""

    def __init__(self, seed, lanes=4):
        self.L = lib()
        self.h = self.L.or_vmt_new(ctypes.c_uint64(seed), lanes)
        self.lanes = lanes

    def __del__(self):
        if getattr(self, "h", None):
            self.L.or_vmt_free(self.h)
            self.h = None

    def raw(self, npackets):
        out = np.empty(npackets * self.lanes, dtype=np.uint64)
        self.L.or_vmt_raw(self.h, _p(out), npackets)
        return out

    def discard(self, npackets):
        self.L.or_vmt_discard(self.h, ctypes.c_uint64(npackets))

    def window(self):
        out = np.empty((self.lanes, 312), dtype=np.uint64)
        self.L.or_vmt_window(self.h, _p(out))
        return out


class Gen:
    """Generator caches (three slots, like a BetaGen with two GammaGens)."""

    def __init__(self):
        self.buf = np.zeros(3 * lib().or_gen_sizeof(), dtype=np.uint8)

    @property
    def ptr(self):
        return _p(self.buf)


REAL = {
    "UNIFORM_REAL": OR_UNIFORM, "UNIFORM_REAL2": OR_UNIFORM, "BALANCED": OR_BALANCED, "BALANCED2": OR_BALANCED,
    "NORMAL_STD": OR_STDNORMAL, "NORMAL": OR_NORMAL, "LOGNORMAL": OR_LOGNORMAL, "EXPONENTIAL": OR_EXPONENTIAL,
    "CAUCHY": OR_CAUCHY, "WEIBULL": OR_WEIBULL, "EXTREME_VALUE": OR_EXTREME, "GAMMA": OR_GAMMA, "BETA": OR_BETA,
    "STUDENT_T": OR_STUDENT_T, "CHI_SQUARED": OR_CHI_SQUARED,
}
DEFAULT_AB = {"UNIFORM_REAL": (0.0, 1.0), "BALANCED": (-1.0, 1.0)}


def generate(eng, gen, kind, n, dtype=np.float32, a=0.0, b=0.0, trials=0, weights=None):
    """Draw n samples of a distribution kind (names as in eigenrand_gb300._lib.KINDS)."""
    L = lib()
    if kind in REAL:
        a, b = DEFAULT_AB.get(kind, (a, b))
        out = np.empty(n, dtype=dtype)
        rc = L.or_gen_real(eng.h, gen.ptr, REAL[kind], 1 if dtype == np.float64 else 0, a, b, _p(out), n)
    elif kind == "BINOMIAL":
        out = np.empty(n, dtype=np.int32)
        rc = L.or_gen_binomial(eng.h, gen.ptr, trials, a, _p(out), n)
    elif kind == "POISSON":
        out = np.empty(n, dtype=np.int32)
        rc = L.or_gen_poisson(eng.h, gen.ptr, a, _p(out), n)
    elif kind == "RANDBITS":
        out = np.empty(n, dtype=np.int32)
        rc = L.or_gen_randbits(eng.h, _p(out), n)
    elif kind == "DISCRETE":
        w = np.asarray(weights, dtype=np.float64)
        d = L.or_discrete_new(_p(w), len(w))
        out = np.empty(n, dtype=np.int32)
        rc = L.or_gen_discrete(eng.h, gen.ptr, d, _p(out), n)
        L.or_discrete_free(d)
    else:
        raise ValueError(kind)
    if rc != 0:
        raise RuntimeError(f"oracle error {rc} for {kind}")
    return out


def vop_set(seed, kind, count, a=0.0, b=1.0, trials=0):
    """One batched set: kind "GAMMA" (float32) or "BINOMIAL_V" (int32)."""
    out = np.empty(max(count, 1), dtype=np.float32 if kind == "GAMMA" else np.int32)
    rc = lib().or_vop_set(ctypes.c_uint64(seed), 0 if kind == "GAMMA" else 1, a, b, trials, _p(out), count)
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return out[:count]


def vec_math(name, x):
    y = np.empty_like(x)
    getattr(lib(), name)(_p(x), _p(y), x.size)
    return y


def pin_engine():
    """Run the libstdc++ / C++-standard pin of the MT19937-64 lane; True if pinned."""
    if not os.path.exists(PIN):
        build()
    r = subprocess.run([PIN], capture_output=True, text=True)
    return r.returncode == 0, r.stdout
