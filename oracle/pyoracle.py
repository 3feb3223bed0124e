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
OR_BERNOULLI, OR_FISHER_F = 14, 15


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
        L.or_gen_negative_binomial.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_double, vp, sz]
        L.or_gen_negative_binomial.restype = ctypes.c_int
        L.or_gen_bernoulli_v_f32.argtypes = [vp, vp, vp, sz]
        L.or_gen_bernoulli_v_f32.restype = ctypes.c_int
        L.or_set_fp_math.argtypes = [ctypes.c_int]
        L.or_set_fp_math.restype = None
        L.or_gen_uniform_int.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int32, vp, sz]
        L.or_gen_uniform_int.restype = ctypes.c_int
        for fn in ("or_gen_bernoulli_i32", "or_gen_geometric"):
            getattr(L, fn).argtypes = [vp, ctypes.c_double, vp, sz]
            getattr(L, fn).restype = ctypes.c_int
        L.or_discrete_new.restype = vp
        L.or_discrete_new.argtypes = [vp, ctypes.c_int]
        L.or_discrete_free.argtypes = [vp]
        L.or_discrete_table.argtypes = [vp, vp, vp, ctypes.c_int]
        L.or_discrete_table.restype = ctypes.c_int
        L.or_gen_discrete.argtypes = [vp, vp, vp, vp, sz]
        L.or_gen_discrete.restype = ctypes.c_int
        L.or_gen_multinomial.argtypes = [vp, vp, vp, ctypes.c_int32, ctypes.c_int32, vp, sz]
        L.or_gen_multinomial.restype = ctypes.c_int
        L.or_gen_multinomial_cond.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int32, vp, sz]
        L.or_gen_multinomial_cond.restype = ctypes.c_int
        L.or_seng_new.restype = vp
        L.or_seng_new.argtypes = [ctypes.c_int, ctypes.c_uint64]
        L.or_seng_free.argtypes = [vp]
        L.or_seng_raw.argtypes = [vp, vp, sz]
        L.or_sgen_real.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, vp, sz]
        L.or_sgen_real.restype = ctypes.c_int
        L.or_sgen_randbits.argtypes = [vp, vp, sz]
        L.or_sgen_randbits.restype = ctypes.c_int
        L.or_gen_truncmvn.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, ctypes.c_int64, vp, sz]
        L.or_gen_truncmvn.restype = ctypes.c_int
        L.or_eigen_sum_avx.argtypes = [vp, ctypes.c_int]
        L.or_eigen_sum_avx.restype = ctypes.c_double
        L.or_vop_set.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                 vp, sz]
        L.or_vop_set.restype = ctypes.c_int
        L.or_gen_real_v.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_double, ctypes.c_double,
                                    vp, sz]
        L.or_gen_real_v.restype = ctypes.c_int
        L.or_gen_binomial_v.argtypes = [vp, vp, vp, ctypes.c_int32, ctypes.c_float, vp, ctypes.c_size_t]
        L.or_gen_binomial_v.restype = ctypes.c_int
        L.or_sgen_binomial_v.argtypes = [vp, vp, vp, ctypes.c_int32, ctypes.c_float, vp, ctypes.c_size_t]
        L.or_sgen_binomial_v.restype = ctypes.c_int
        L.or_sgen_int.argtypes = [vp, ctypes.c_int, ctypes.c_int32, ctypes.c_double, vp, ctypes.c_size_t]
        L.or_sgen_int.restype = ctypes.c_int
        L.or_sgen_discrete.argtypes = [vp, vp, vp, ctypes.c_size_t]
        L.or_sgen_discrete.restype = ctypes.c_int
        L.or_gen_trunc.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, vp, sz]
        L.or_gen_trunc.restype = ctypes.c_int
        for name in ("or_vec_logf", "or_vec_expf", "or_vec_log", "or_vec_exp", "or_vec_erfinvf", "or_vec_erfinv"):
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


class ScalarEngine:
    """A scalar engine as EigenRand's Urng: "mt19937_64" (std::mt19937_64) or
    "p8" (P8_mt19937_64 over Vmt19937_64(seed), Vmt19937_64(seed + 4))."""

    KINDS = {"mt19937_64": 1, "p8": 2}

    def __init__(self, kind, seed):
        self.L = lib()
        self.h = self.L.or_seng_new(self.KINDS[kind], ctypes.c_uint64(seed))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.or_seng_free(self.h)
            self.h = None

    def raw(self, n):
        out = np.empty(n, dtype=np.uint64)
        self.L.or_seng_raw(self.h, _p(out), n)
        return out

    def discrete(self, weights, n):
        """discrete() (a fresh DiscreteGen<int32_t>) through the scalar engine."""
        w = np.asarray(weights, dtype=np.float64)
        d = self.L.or_discrete_new(_p(w), len(w))
        out = np.empty(n, dtype=np.int32)
        rc = self.L.or_sgen_discrete(self.h, d, _p(out), n)
        self.L.or_discrete_free(d)
        if rc:
            raise RuntimeError(f"oracle error {rc}")
        return out

    def binomial_v(self, trials, p):
        """binomial(urng, trials, p) (BinomialVGen<int32_t>) through the scalar engine."""
        ta = np.ascontiguousarray(trials, dtype=np.int32) if isinstance(trials, np.ndarray) else None
        pa = np.ascontiguousarray(p, dtype=np.float32) if isinstance(p, np.ndarray) else None
        n = (ta if ta is not None else pa).size
        out = np.empty(n, dtype=np.int32)
        rc = self.L.or_sgen_binomial_v(self.h, _p(ta) if ta is not None else None, _p(pa) if pa is not None else None,
                                       0 if ta is not None else int(trials), 0.0 if pa is not None else float(p),
                                       _p(out), n)
        if rc:
            raise RuntimeError(f"oracle error {rc}")
        return out

    def generate(self, gen, kind, n, dtype=np.float32, a=0.0, b=0.0, trials=0):
        """Real kinds of generate(), RANDBITS, and the free functions poisson() /
        binomial() (a fresh generator each call), drawn through the scalar engine."""
        if kind in ("POISSON", "BINOMIAL", "UNIFORM_INT", "NEGATIVE_BINOMIAL") or (
                kind in ("BERNOULLI", "GEOMETRIC") and dtype == np.int32):
            out = np.empty(n, dtype=np.int32)
            k = {"POISSON": 0, "BINOMIAL": 1, "UNIFORM_INT": 2, "BERNOULLI": 3, "GEOMETRIC": 4,
                 "NEGATIVE_BINOMIAL": 5}[kind]
            t = int(b) if kind == "UNIFORM_INT" else int(trials)  # UNIFORM_INT: a = min, b = max
            rc = self.L.or_sgen_int(self.h, k, t, float(a), _p(out), n)
        elif kind == "RANDBITS":
            out = np.empty(n, dtype=np.int32)
            rc = self.L.or_sgen_randbits(self.h, _p(out), n)
        else:
            a, b = DEFAULT_AB.get(kind, (a, b))
            out = np.empty(n, dtype=dtype)
            dist = OR_BERNOULLI if kind == "BERNOULLI" else REAL[kind]
            rc = self.L.or_sgen_real(self.h, gen.ptr, dist, 1 if dtype == np.float64 else 0, a, b, _p(out), n)
        if rc != 0:
            raise RuntimeError(f"oracle error {rc} for {kind}")
        return out


class Gen:
    """Generator caches (four slots: a BetaGen with two GammaGens, and a
    TruncGen's carried lanes over any of them)."""

    def __init__(self):
        self.buf = np.zeros(4 * lib().or_gen_sizeof(), dtype=np.uint8)

    @property
    def ptr(self):
        return _p(self.buf)


REAL = {
    "UNIFORM_REAL": OR_UNIFORM, "UNIFORM_REAL2": OR_UNIFORM, "BALANCED": OR_BALANCED, "BALANCED2": OR_BALANCED,
    "NORMAL_STD": OR_STDNORMAL, "NORMAL": OR_NORMAL, "LOGNORMAL": OR_LOGNORMAL, "EXPONENTIAL": OR_EXPONENTIAL,
    "CAUCHY": OR_CAUCHY, "WEIBULL": OR_WEIBULL, "EXTREME_VALUE": OR_EXTREME, "GAMMA": OR_GAMMA, "BETA": OR_BETA,
    "STUDENT_T": OR_STUDENT_T, "CHI_SQUARED": OR_CHI_SQUARED, "FISHER_F": OR_FISHER_F,
}
INT_ONE_PARAM = {"BERNOULLI": "or_gen_bernoulli_i32", "GEOMETRIC": "or_gen_geometric"}
DEFAULT_AB = {"UNIFORM_REAL": (0.0, 1.0), "BALANCED": (-1.0, 1.0)}


def generate(eng, gen, kind, n, dtype=np.float32, a=0.0, b=0.0, trials=0, weights=None):
    """Draw n samples of a distribution kind (names as in eigenrand_gb300._lib.KINDS)."""
    L = lib()
    if kind == "BERNOULLI" and dtype != np.int32:
        out = np.empty(n, dtype=dtype)
        rc = L.or_gen_real(eng.h, gen.ptr, OR_BERNOULLI, 1 if dtype == np.float64 else 0, a, 0.0, _p(out), n)
    elif kind == "NEGATIVE_BINOMIAL":
        out = np.empty(n, dtype=np.int32)
        rc = L.or_gen_negative_binomial(eng.h, gen.ptr, int(trials), a, _p(out), n)
    elif kind == "UNIFORM_INT":
        out = np.empty(n, dtype=np.int32)
        rc = L.or_gen_uniform_int(eng.h, gen.ptr, int(a), int(b), _p(out), n)
    elif kind in INT_ONE_PARAM:
        out = np.empty(n, dtype=np.int32)
        rc = getattr(L, INT_ONE_PARAM[kind])(eng.h, a, _p(out), n)
    elif kind in REAL:
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


def generate_v(eng, gen, kind, a, b=None, dtype=np.float32):
    """A per-element form (*VGen): a / b are arrays of the output's length in
    Eigen's linear order, or scalars."""
    L = lib()
    arrs = [np.ascontiguousarray(x, dtype=dtype) if isinstance(x, np.ndarray) else None for x in (a, b)]
    n = next(x.size for x in arrs if x is not None)
    out = np.empty(n, dtype=dtype)
    sa = 0.0 if arrs[0] is not None else float(a)
    sb = 0.0 if arrs[1] is not None or b is None else float(b)
    rc = L.or_gen_real_v(eng.h, gen.ptr, REAL[kind], 1 if dtype == np.float64 else 0,
                         _p(arrs[0]) if arrs[0] is not None else None,
                         _p(arrs[1]) if arrs[1] is not None else None, sa, sb, _p(out), n)
    if rc != 0:
        raise RuntimeError(f"oracle error {rc} for per-element {kind}")
    return out


def truncated(eng, gen, kind, n, lower, upper, dtype=np.float32, a=0.0, b=0.0):
    """TruncGen<Base>{base, Support(lower, upper)} (Truncated.h): n samples.
    kind names the base as in generate(); the uniform family takes the base's
    own range in (a, b)."""
    L = lib()
    a, b = DEFAULT_AB.get(kind, (a, b))
    out = np.empty(n, dtype=dtype)
    dist = OR_BERNOULLI if kind == "BERNOULLI" else REAL[kind]
    rc = L.or_gen_trunc(eng.h, gen.ptr, dist, 1 if dtype == np.float64 else 0, a, b, lower, upper, _p(out), n)
    if rc != 0:
        raise RuntimeError(f"oracle error {rc} for truncated {kind}")
    return out


def erfinv(x):
    """The oracle's erfinv (Giles' approximation as EigenRand's perfinv evaluates it)."""
    x = np.ascontiguousarray(x)
    y = np.empty_like(x)
    fn = lib().or_vec_erfinvf if x.dtype == np.float32 else lib().or_vec_erfinv
    fn(_p(x), _p(y), x.size)
    return y


def multinomial(eng, gen, weights, trials, samples):
    """MultinomialGen<int32_t>(trials, weights).generate(urng, samples) on the
    per-trial path (Multinomial.h:62-71, 95-118).  Returns (samples, dim):
    row s = column s of the reference's (dim, samples) matrix."""
    L = lib()
    w = np.asarray(weights, dtype=np.float64)
    d = L.or_discrete_new(_p(w), len(w))
    out = np.empty((samples, len(w)), dtype=np.int32)
    rc = L.or_gen_multinomial(eng.h, gen.ptr, d, int(trials), len(w), _p(out), samples)
    L.or_discrete_free(d)
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return out


def binomial_v(eng, trials, p):
    """binomial(urng, trials, p) -> BinomialVGen<int32_t> (Discrete.h:1124-1192,
    1822-1898): int32 trials and float p arrays in Eigen's linear order, or
    one of them a scalar."""
    L = lib()
    ta = np.ascontiguousarray(trials, dtype=np.int32) if isinstance(trials, np.ndarray) else None
    pa = np.ascontiguousarray(p, dtype=np.float32) if isinstance(p, np.ndarray) else None
    n = (ta if ta is not None else pa).size
    out = np.empty(n, dtype=np.int32)
    rc = L.or_gen_binomial_v(eng.h, _p(ta) if ta is not None else None, _p(pa) if pa is not None else None,
                             0 if ta is not None else int(trials), 0.0 if pa is not None else float(p), _p(out), n)
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return out


def multinomial_cond(eng, weights, trials, samples):
    """MultinomialGen<int32_t>(trials, weights).generate(urng, samples) on the
    conditional-binomial path (Multinomial.h:62-87).  Returns (samples, dim)."""
    L = lib()
    w = np.ascontiguousarray(weights, dtype=np.float64)
    out = np.empty((samples, len(w)), dtype=np.int32)
    rc = L.or_gen_multinomial_cond(eng.h, _p(w), len(w), int(trials), _p(out), samples)
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return out


def precision_from_lt(lt):
    """H = L^-T L^-1 from the lower triangle of the factor, FP64."""
    Lt = np.tril(np.asarray(lt, np.float64))
    inv = np.linalg.solve(Lt, np.eye(len(Lt)))
    return inv.T @ inv


def truncmvn(eng, mean, cov, lower, upper, samples, burn_in=0, dtype=np.float32, lower_triangular=False):
    """TruncMvNormalGen(mean, cov | lt, support(lower, upper), burn_in).generate(urng, samples)
    (TruncMvNormal.h:171-209) with the factor of get_lt in FP64.  Returns (samples, dim)."""
    L = lib()
    lt = np.asarray(cov, np.float64) if lower_triangular else get_lt(cov)
    H = np.ascontiguousarray(precision_from_lt(lt).T)  # column-major
    m = np.ascontiguousarray(mean, np.float64)
    lo = np.ascontiguousarray(lower, np.float64)
    hi = np.ascontiguousarray(upper, np.float64)
    out = np.empty((samples, len(m)), dtype=dtype)
    rc = L.or_gen_truncmvn(eng.h, 1 if dtype == np.float64 else 0, len(m), _p(H), _p(m), _p(lo), _p(hi),
                           int(burn_in), _p(out), samples)
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return out


def eigen_sum_avx(v):
    """Eigen 3.4's vectorized sum() order for a double vector (AVX)."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    return lib().or_eigen_sum_avx(_p(v), len(v))


def discrete_table(weights):
    """DiscreteGen's table (Discrete.h:23-207): ("cdf", cdf) or ("alias", prob, alias, bitmask)."""
    L = lib()
    w = np.asarray(weights, dtype=np.float64)
    d = L.or_discrete_new(_p(w), len(w))
    prob = np.zeros(1 << 16, np.int32)
    alias = np.zeros(1 << 16, np.int32)
    ps = L.or_discrete_table(d, _p(prob), _p(alias), len(prob))
    L.or_discrete_free(d)
    if ps < 0:
        return ("cdf", prob[:-ps].astype(np.uint32))
    return ("alias", prob[:ps].copy(), alias[:ps].copy(), ps - 1)


# ---- FP64 restatements of the multivariate assembly (the error oracle) ----
def get_lt(matrix):
    """MvNormal.h:21-38 in FP64: Cholesky of the matrix the lower triangle
    defines, else eigenvectors * sqrt(max(eigenvalues, 0))."""
    a = np.asarray(matrix, dtype=np.float64)
    a = np.tril(a) + np.tril(a, -1).T
    try:
        return np.linalg.cholesky(a)
    except np.linalg.LinAlgError:
        w, v = np.linalg.eigh(a)
        return v * np.sqrt(np.maximum(w, 0.0))


def mvnormal_f64(lt, z, mean):
    """MvNormalGen::generate (MvNormal.h:103-108): lt @ Z + mean, Z (dim, samples)."""
    return np.asarray(lt, np.float64) @ np.asarray(z, np.float64) + np.asarray(mean, np.float64)[:, None]


def bartlett(normals, chis, dim, samples):
    """The per-draw Bartlett matrices of WishartGen::generate (MvNormal.h:236-262):
    strictly-lower normals column by column, sqrt(chi^2) on the diagonal.
    normals: samples * dim (dim-1) / 2 values; chis: (dim, samples)."""
    nper = dim * (dim - 1) // 2
    A = np.zeros((samples, dim, dim))
    nz = np.asarray(normals, np.float64).reshape(samples, nper)
    ptr = 0
    for i in range(dim - 1):
        A[:, i + 1:, i] = nz[:, ptr:ptr + dim - 1 - i]
        ptr += dim - 1 - i
    ch = np.sqrt(np.asarray(chis, np.float64))
    for i in range(dim):
        A[:, i, i] = ch[i]
    return A


def wishart_f64(chol, normals, chis, dim, samples, inverse=False):
    """WishartGen (MvNormal.h:263-276) / InvWishartGen (:427-440) in FP64.
    Returns (dim, dim * samples) like the reference."""
    A = bartlett(normals, chis, dim, samples)
    T = np.asarray(chol, np.float64)[None] @ A
    if inverse:
        U = np.linalg.inv(np.tril(T))
        W = np.transpose(U, (0, 2, 1)) @ U
    else:
        W = T @ np.transpose(T, (0, 2, 1))
    return np.concatenate(list(W), axis=1)


def dirichlet_f64(rows):
    """DirichletGen::generate (Multinomial.h:190-203): column-normalised gamma rows."""
    r = np.asarray(rows, np.float64)
    return r / r.sum(axis=0, keepdims=True)


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


def set_fp_math(on):
    """CPU-baseline timing mode: double log / exp through the C library's FP64
    functions, the speed class of the reference's Eigen plog / pexp (values
    within an ulp of the exact integer versions; never used for parity)."""
    lib().or_set_fp_math(1 if on else 0)


def bernoulli_v(eng, p):
    """BernoulliVGen<float>: one probability per element (float32 array)."""
    p = np.ascontiguousarray(p, dtype=np.float32)
    out = np.empty_like(p)
    rc = lib().or_gen_bernoulli_v_f32(eng.h, _p(p), _p(out), p.size)
    if rc != 0:
        raise RuntimeError(f"oracle error {rc} for bernoulli_v")
    return out
