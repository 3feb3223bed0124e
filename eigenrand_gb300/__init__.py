"""GB300 sampling library with EigenRand's call surface.

Python mirror of the ``Eigen::Rand`` API (bab2min/EigenRand v0.6.0) over the
C ABI in include/gpurand.h.  Engines and generator caches live in HBM; outputs
are CUDA tensors laid out column-major like Eigen arrays (shape (rows, cols),
memory order = Eigen's linear index).  torch is used only for device memory
and the current CUDA stream.

    import eigenrand_gb300 as er
    urng = er.Vmt19937_64(42)                       # Eigen::Rand::Vmt19937_64 urng{42};
    x = er.normal(4096, 4096, urng)                 # Eigen::Rand::normal<ArrayXXf>(4096, 4096, urng)
    g = er.GammaGen(0.5, 1.0, dtype=torch.float64)  # Eigen::Rand::GammaGen<double> g{0.5, 1.0};
    y = g.generate(1024, 1024, urng)

Values are bit-identical to EigenRand built for x86-64 AVX2 with Eigen 3.4
(Vmt19937_64 = 4 lanes, float packets of 8, double 4, int32 4) wherever the
reference's arithmetic is IEEE-exact; log/exp are this library's own <=1-ulp
implementations (see csrc/gr_math.cuh).
"""
import ctypes

import torch

from . import _lib
from ._lib import GrError, KINDS, F32, F64, I32, U64

__all__ = [
    "GrError", "Vmt19937_64", "mt19937_64", "P8_mt19937_64", "raw_u64", "version",
    "uniformReal", "balanced", "normal", "lognormal", "exponential", "cauchy", "weibull", "extremeValue",
    "gamma", "beta", "studentT", "chiSquared", "poisson", "binomial", "discrete", "randBits", "bernoulli",
    "geometric", "fisherF", "uniformInt", "negativeBinomial",
    "StdUniformRealGen", "UniformRealGen", "BalancedGen", "Balanced2Gen", "StdNormalGen", "NormalGen",
    "LognormalGen", "ExponentialGen", "CauchyGen", "WeibullGen", "ExtremeValueGen", "GammaGen", "BetaGen",
    "StudentTGen", "ChiSquaredGen", "PoissonGen", "BinomialGen", "DiscreteGen", "RandbitsGen", "BernoulliGen",
    "GeometricGen", "FisherFGen", "UniformIntGen", "NegativeBinomialGen",
    "UniformRealVGen", "BalancedVGen", "NormalVGen", "LognormalVGen", "ExponentialVGen", "StudentTVGen",
    "WeibullVGen", "ExtremeValueVGen", "CauchyVGen", "BernoulliVGen",
    "Support", "support", "TruncGen", "TruncNormalGen", "truncated", "truncatedLike", "truncatedNormal",
    "truncatedNormalLike",
    "sample_batched",
    "MvNormalGen", "WishartGen", "InvWishartGen", "DirichletGen", "MultinomialGen", "makeMvNormalGen",
    "makeMvNormalGenFromLt", "makeWishartGen", "makeWishartGenFromLt", "makeInvWishartGen",
    "makeInvWishartGenFromIlt", "makeDirichletGen", "makeMultinomialGen",
    "TruncMvNormalGen", "makeTruncMvNormalGen", "makeTruncMvNormalGenFromLt",
]

_lib.load()
_L = _lib._lib


def version():
    return _L.gr_version().decode()


def _stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class Vmt19937_64:
    """Eigen::Rand::Vmt19937_64 (PacketRandomEngine.h:585-599), device resident.

    streams=1: one 4-lane engine, lane l = std::mt19937_64(seed + l).
    streams=K: K independent engines seeded seed + 4k; every call splits its
    output into K contiguous slices, slice k drawn from engine k.
    """

    default_seed = 5489

    def __init__(self, seed=default_seed, streams=1, lanes=4):
        h = ctypes.c_void_p()
        _lib.check(_L.gr_engine_create(ctypes.byref(h), ctypes.c_uint64(seed), lanes, streams))
        self._h = h
        self.streams = streams
        self.lanes = lanes

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _L is not None:
            _L.gr_engine_destroy(h)
            self._h = None

    def seed(self, seed, stream=None):
        _lib.check(_L.gr_engine_seed(self._h, ctypes.c_uint64(seed), _stream_ptr(stream)))

    def discard(self, npackets, stream=None):
        _lib.check(_L.gr_engine_discard(self._h, ctypes.c_uint64(npackets), _stream_ptr(stream)))

    def state_size(self):
        return _L.gr_engine_state_size(self._h)

    def save(self, stream=None):
        buf = ctypes.create_string_buffer(self.state_size())
        _lib.check(_L.gr_engine_save(self._h, buf, len(buf), _stream_ptr(stream)))
        return bytes(buf.raw)

    def restore(self, blob, stream=None):
        buf = ctypes.create_string_buffer(blob, len(blob))
        _lib.check(_L.gr_engine_restore(self._h, buf, len(blob), _stream_ptr(stream)))

    def sync(self, stream=None):
        _lib.check(_L.gr_engine_sync(self._h, _stream_ptr(stream)))


class _ScalarEngine:
    """A scalar engine as the Urng (gr_sengine): its packets come from
    RawbitsMaker<..., scalar_fullbit> over its 64-bit draws.  Fixed-draw
    kinds only (the free functions and cacheless generator objects)."""

    _kind = None

    def __init__(self, seed=5489):
        h = ctypes.c_void_p()
        _lib.check(_L.gr_sengine_create(ctypes.byref(h), self._kind, ctypes.c_uint64(seed)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _L is not None:
            _L.gr_sengine_destroy(h)
            self._h = None

    def raw(self, n, out=None, stream=None):
        """operator()() n times; an int64 tensor of the uint64 bit patterns."""
        o = out if out is not None else torch.empty(n, dtype=torch.int64, device="cuda")
        _lib.check(_L.gr_sengine_raw_u64(self._h, _ptr(o), n, _stream_ptr(stream)))
        return o


class mt19937_64(_ScalarEngine):
    """std::mt19937_64(seed) as EigenRand's Urng."""
    _kind = 1


class P8_mt19937_64(_ScalarEngine):
    """Eigen::Rand::P8_mt19937_64(seed) (PacketRandomEngine.h:600-607)."""
    _kind = 2


def _empty(rows, cols, dtype, out):
    if out is not None:
        return out
    return torch.empty((cols, rows), dtype=dtype, device="cuda").t()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def raw_u64(urng, n, out=None, stream=None):
    """makeUniversalRng<uint64_t>(urng)() repeated n times (PacketRandomEngine.h:468-475).

    Returns an int64 tensor holding the uint64 bit patterns."""
    o = out if out is not None else torch.empty(n, dtype=torch.int64, device="cuda")
    _lib.check(_L.gr_raw_u64(urng._h, _ptr(o), n, _stream_ptr(stream)))
    return o


_DT = {torch.float32: F32, torch.float64: F64, torch.int32: I32}


def _desc(kind, dtype, a=0.0, b=0.0, trials=0, weights=None):
    d = _lib.DistDesc()
    d.kind = KINDS[kind]
    d.dtype = _DT[dtype]
    d.a = float(a)
    d.b = float(b)
    d.trials = int(trials)
    keep = None
    if weights is not None:
        keep = (ctypes.c_double * len(weights))(*[float(w) for w in weights])
        d.nweights = len(weights)
        d.weights = ctypes.cast(keep, ctypes.POINTER(ctypes.c_double))
    return d, keep


class _Gen:
    """One generator object (mirrors a *Gen instance, caches included)."""

    _kind = None

    def __init__(self, dtype, a=0.0, b=0.0, trials=0, weights=None, kind=None):
        self.dtype = dtype
        self._desc, self._keep = _desc(kind or self._kind, dtype, a, b, trials, weights)
        h = ctypes.c_void_p()
        _lib.check(_L.gr_gen_create(ctypes.byref(h), ctypes.byref(self._desc)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _L is not None:
            _L.gr_gen_destroy(h)
            self._h = None

    def generate(self, rows, cols, urng, out=None, stream=None):
        o = _empty(rows, cols, self.dtype, out)
        if isinstance(urng, _ScalarEngine):
            if self._desc.kind in (KINDS["NORMAL_STD"], KINDS["NORMAL"], KINDS["LOGNORMAL"]):
                raise GrError(3, "a generator object with a cache on a scalar engine; use the free function")
            _lib.check(_L.gr_sengine_sample(urng._h, ctypes.byref(self._desc), _ptr(o), rows * cols,
                                            _stream_ptr(stream)))
            return o
        _lib.check(_L.gr_generate(self._h, urng._h, _ptr(o), rows * cols, _stream_ptr(stream)))
        return o

    def generateLike(self, o, urng, stream=None):
        return self.generate(o.shape[0], o.shape[1], urng, stream=stream)


def _sample(kind, rows, cols, urng, dtype, a=0.0, b=0.0, trials=0, weights=None, out=None, stream=None):
    o = _empty(rows, cols, dtype, out)
    d, keep = _desc(kind, dtype, a, b, trials, weights)
    fn = _L.gr_sengine_sample if isinstance(urng, _ScalarEngine) else _L.gr_sample
    _lib.check(fn(urng._h, ctypes.byref(d), _ptr(o), rows * cols, _stream_ptr(stream)))
    del keep
    return o


# ---- generator classes (Dists/*.h) --------------------------------------
class StdUniformRealGen(_Gen):
    _kind = "UNIFORM_REAL"

    def __init__(self, dtype=torch.float32):
        super().__init__(dtype)


class UniformRealGen(_Gen):
    _kind = "UNIFORM_REAL2"

    def __init__(self, min=0.0, max=1.0, dtype=torch.float32):
        super().__init__(dtype, min, max)


class BalancedGen(_Gen):
    _kind = "BALANCED"

    def __init__(self, dtype=torch.float32):
        super().__init__(dtype)


class Balanced2Gen(_Gen):
    _kind = "BALANCED2"

    def __init__(self, a=-1.0, b=1.0, dtype=torch.float32):
        super().__init__(dtype, a, b)


class StdNormalGen(_Gen):
    _kind = "NORMAL_STD"

    def __init__(self, dtype=torch.float32):
        super().__init__(dtype)


class NormalGen(_Gen):
    _kind = "NORMAL"

    def __init__(self, mean=0.0, stdev=1.0, dtype=torch.float32):
        super().__init__(dtype, mean, stdev)


class LognormalGen(_Gen):
    _kind = "LOGNORMAL"

    def __init__(self, mean=0.0, stdev=1.0, dtype=torch.float32):
        super().__init__(dtype, mean, stdev)


class ExponentialGen(_Gen):
    _kind = "EXPONENTIAL"

    def __init__(self, lambda_=1.0, dtype=torch.float32):
        super().__init__(dtype, lambda_)


class CauchyGen(_Gen):
    _kind = "CAUCHY"

    def __init__(self, a=0.0, b=1.0, dtype=torch.float32):
        super().__init__(dtype, a, b)


class WeibullGen(_Gen):
    _kind = "WEIBULL"

    def __init__(self, a=1.0, b=1.0, dtype=torch.float32):
        super().__init__(dtype, a, b)


class ExtremeValueGen(_Gen):
    _kind = "EXTREME_VALUE"

    def __init__(self, a=0.0, b=1.0, dtype=torch.float32):
        super().__init__(dtype, a, b)


class GammaGen(_Gen):
    _kind = "GAMMA"

    def __init__(self, alpha=1.0, beta=1.0, dtype=torch.float32):
        super().__init__(dtype, alpha, beta)


class BetaGen(_Gen):
    _kind = "BETA"

    def __init__(self, a=1.0, b=1.0, dtype=torch.float32):
        super().__init__(dtype, a, b)


class StudentTGen(_Gen):
    _kind = "STUDENT_T"

    def __init__(self, n=1.0, dtype=torch.float32):
        super().__init__(dtype, n)


class ChiSquaredGen(_Gen):
    _kind = "CHI_SQUARED"

    def __init__(self, n=1.0, dtype=torch.float32):
        super().__init__(dtype, n)


class PoissonGen(_Gen):
    _kind = "POISSON"

    def __init__(self, mean=1.0):
        super().__init__(torch.int32, mean)


class BinomialGen(_Gen):
    _kind = "BINOMIAL"

    def __init__(self, trials=1, p=0.5):
        super().__init__(torch.int32, p, trials=trials)


class DiscreteGen(_Gen):
    _kind = "DISCRETE"

    def __init__(self, weights):
        super().__init__(torch.int32, weights=list(weights))


class RandbitsGen(_Gen):
    _kind = "RANDBITS"

    def __init__(self):
        super().__init__(torch.int32)


class BernoulliGen(_Gen):
    """BernoulliGen<Scalar>(p): 1 or 0 in float32, float64 or int32 (Basic.h:669-708)."""
    _kind = "BERNOULLI"

    def __init__(self, p=0.5, dtype=torch.float32):
        super().__init__(dtype, p)


class FisherFGen(_Gen):
    """FisherFGen(m, n) = BetaGen(m/2, n/2) mapped to (n/m) x / (1 - x) (NormalExp.h:984-1023)."""
    _kind = "FISHER_F"

    def __init__(self, m=1.0, n=1.0, dtype=torch.float32):
        super().__init__(dtype, m, n)


class UniformIntGen(_Gen):
    """UniformIntGen<int32_t>(min, max), both ends included (Discrete.h:214-336)."""
    _kind = "UNIFORM_INT"

    def __init__(self, min=0, max=0):
        super().__init__(torch.int32, float(min), float(max))


class NegativeBinomialGen(_Gen):
    """NegativeBinomialGen<int32_t>(trials, p) (GammaPoisson.h:28-98)."""
    _kind = "NEGATIVE_BINOMIAL"

    def __init__(self, trials=1, p=0.5):
        super().__init__(torch.int32, p, trials=trials)


class GeometricGen(_Gen):
    """GeometricGen<int32_t>(p) (Discrete.h:1338-1376)."""
    _kind = "GEOMETRIC"

    def __init__(self, p=0.5):
        super().__init__(torch.int32, p)


# ---- per-element generator classes (*VGen) ----------------------------------
class _VGen:
    """A *VGen object: generate(urng, a[, b]) draws one value per element of
    the parameter tensors; NormalVGen / LognormalVGen keep their StdNormalGen
    cache between calls."""

    _kind = None
    _two = True

    def __init__(self, dtype=torch.float32):
        self.dtype = dtype
        self._desc, self._keep = _desc(self._kind, dtype)
        h = ctypes.c_void_p()
        _lib.check(_L.gr_gen_create(ctypes.byref(h), ctypes.byref(self._desc)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _L is not None:
            _L.gr_gen_destroy(h)
            self._h = None

    def generate(self, urng, a, b=None, out=None, stream=None):
        return _vform(self._kind, urng, a, b, two=self._two, gen=self, out=out, stream=stream)


class UniformRealVGen(_VGen):
    """UniformRealVGen<T> (Basic.h:638-666)."""
    _kind = "UNIFORM_REAL2"


class BalancedVGen(_VGen):
    """BalancedVGen<T> (Basic.h:472-492)."""
    _kind = "BALANCED2"


class NormalVGen(_VGen):
    """NormalVGen<T> (NormalExp.h:139-163)."""
    _kind = "NORMAL"


class LognormalVGen(_VGen):
    """LognormalVGen<T> (NormalExp.h:213-236)."""
    _kind = "LOGNORMAL"


class ExponentialVGen(_VGen):
    """ExponentialVGen<T> (NormalExp.h:402-427)."""
    _kind = "EXPONENTIAL"
    _two = False


class StudentTVGen(_VGen):
    """StudentTVGen<T> (NormalExp.h:305-343)."""
    _kind = "STUDENT_T"
    _two = False


class WeibullVGen(_VGen):
    """WeibullVGen<T> (NormalExp.h:659-686)."""
    _kind = "WEIBULL"


class ExtremeValueVGen(_VGen):
    """ExtremeValueVGen<T> (NormalExp.h:736-765)."""
    _kind = "EXTREME_VALUE"


class CauchyVGen(_VGen):
    """CauchyVGen<T> (NormalExp.h:859-889)."""
    _kind = "CAUCHY"


class BernoulliVGen(_VGen):
    """BernoulliVGen<float> (Basic.h:711-747)."""
    _kind = "BERNOULLI"
    _two = False


# ---- free functions (Dists/*.h tails) -----------------------------------
def _eigen_order(t, dtype):
    """A parameter tensor on the device in Eigen's memory order (column-major
    for 2-D), so that element i of memory is the reference's linear index i."""
    t = t.to(device="cuda", dtype=dtype)
    if t.dim() == 2:
        return t.t().contiguous().t()
    return t.contiguous()


def _vform(kind, urng, a, b=None, two=True, gen=None, out=None, stream=None):
    """The per-element forms: kind(urng, a, b) with a and / or b tensors of
    the output's shape (*VGen, gr_sample_v2 / gr_generate_v)."""
    ten = [x for x in (a, b) if torch.is_tensor(x)]
    if not ten:
        raise TypeError("the per-element form needs a parameter tensor")
    dtype = ten[0].dtype if ten[0].dtype in (torch.float32, torch.float64) else torch.float32
    pa = _eigen_order(a, dtype) if torch.is_tensor(a) else None
    pb = _eigen_order(b, dtype) if torch.is_tensor(b) else None
    if pa is not None and pb is not None and pa.shape != pb.shape:
        raise ValueError("a and b must have the same shape")
    ref = pa if pa is not None else pb
    o = torch.empty_like(ref) if out is None else out
    sa = 0.0 if pa is not None else float(a)
    sb = 0.0 if pb is not None or not two else float(b)
    vp = lambda t: _ptr(t) if t is not None else None
    if gen is not None:
        _lib.check(_L.gr_generate_v(gen._h, urng._h, vp(pa), vp(pb), _ptr(o), o.numel(), _stream_ptr(stream)))
    else:
        d, keep = _desc(kind, dtype, sa, sb)
        fn = _L.gr_sengine_sample_v2 if isinstance(urng, _ScalarEngine) else _L.gr_sample_v2
        _lib.check(fn(urng._h, ctypes.byref(d), vp(pa), vp(pb), _ptr(o), o.numel(), _stream_ptr(stream)))
        del keep
    return o


def _is_v(args):
    return bool(args) and isinstance(args[0], (Vmt19937_64, _ScalarEngine))


def uniformReal(*args, min=None, max=None, dtype=torch.float32, out=None, stream=None):
    """uniformReal(rows, cols, urng[, min, max]); uniformReal(urng, a, b) with
    tensor bounds -> UniformRealVGen (Basic.h:1047-1092)."""
    if _is_v(args):
        return _vform("UNIFORM_REAL2", *args, out=out, stream=stream)
    rows, cols, urng = args[:3]
    if len(args) > 3:
        min = args[3]
    if len(args) > 4:
        max = args[4]
    if min is None and max is None:
        return _sample("UNIFORM_REAL", rows, cols, urng, dtype, out=out, stream=stream)
    return _sample("UNIFORM_REAL2", rows, cols, urng, dtype, 0.0 if min is None else min,
                   1.0 if max is None else max, out=out, stream=stream)


def balanced(*args, a=None, b=None, dtype=torch.float32, out=None, stream=None):
    """balanced(rows, cols, urng[, a, b]); balanced(urng, a, b) -> BalancedVGen (Basic.h:895-939)."""
    if _is_v(args):
        return _vform("BALANCED2", *args, out=out, stream=stream)
    rows, cols, urng = args[:3]
    if len(args) > 3:
        a = args[3]
    if len(args) > 4:
        b = args[4]
    if a is None and b is None:
        return _sample("BALANCED", rows, cols, urng, dtype, out=out, stream=stream)
    return _sample("BALANCED2", rows, cols, urng, dtype, a, b, out=out, stream=stream)


def normal(*args, mean=None, stdev=None, dtype=torch.float32, out=None, stream=None):
    """normal(rows, cols, urng[, mean, stdev]); normal(urng, mean, stdev) with
    tensor operands -> NormalVGen (NormalExp.h:1296-1336)."""
    if _is_v(args):
        return _vform("NORMAL", *args, out=out, stream=stream)
    rows, cols, urng = args[:3]
    if len(args) > 3:
        mean = args[3]
    if len(args) > 4:
        stdev = args[4]
    if mean is None and stdev is None:
        return _sample("NORMAL_STD", rows, cols, urng, dtype, out=out, stream=stream)
    return _sample("NORMAL", rows, cols, urng, dtype, 0.0 if mean is None else mean,
                   1.0 if stdev is None else stdev, out=out, stream=stream)


def _two(kind, defaults):
    def fn(*args, dtype=torch.float32, out=None, stream=None, **kw):
        if _is_v(args):
            return _vform(kind, *args, out=out, stream=stream)
        rows, cols, urng = args[:3]
        vals = list(args[3:]) + [kw.get(k, v) for k, v in list(defaults.items())[len(args) - 3:]]
        return _sample(kind, rows, cols, urng, dtype, *vals[:2], out=out, stream=stream)
    return fn


def _one(kind, name, default):
    def fn(*args, dtype=torch.float32, out=None, stream=None, **kw):
        if _is_v(args):
            return _vform(kind, args[0], args[1], two=False, out=out, stream=stream)
        rows, cols, urng = args[:3]
        v = args[3] if len(args) > 3 else kw.get(name, default)
        return _sample(kind, rows, cols, urng, dtype, v, out=out, stream=stream)
    return fn


lognormal = _two("LOGNORMAL", {"mean": 0.0, "stdev": 1.0})
lognormal.__doc__ = "lognormal(rows, cols, urng[, mean, stdev]); lognormal(urng, mean, stdev) -> LognormalVGen."
exponential = _one("EXPONENTIAL", "lambda_", 1.0)
exponential.__doc__ = "exponential(rows, cols, urng[, lambda]); exponential(urng, lambda) -> ExponentialVGen."
cauchy = _two("CAUCHY", {"a": 0.0, "b": 1.0})
cauchy.__doc__ = "cauchy(rows, cols, urng[, a, b]); cauchy(urng, a, b) -> CauchyVGen."
weibull = _two("WEIBULL", {"a": 1.0, "b": 1.0})
weibull.__doc__ = "weibull(rows, cols, urng[, a, b]); weibull(urng, a, b) -> WeibullVGen."
extremeValue = _two("EXTREME_VALUE", {"a": 0.0, "b": 1.0})
extremeValue.__doc__ = "extremeValue(rows, cols, urng[, a, b]); extremeValue(urng, a, b) -> ExtremeValueVGen."


def gamma(rows, cols, urng, alpha=1.0, beta=1.0, dtype=torch.float32, out=None, stream=None):
    return _sample("GAMMA", rows, cols, urng, dtype, alpha, beta, out=out, stream=stream)


def beta(rows, cols, urng, a=1.0, b=1.0, dtype=torch.float32, out=None, stream=None):
    return _sample("BETA", rows, cols, urng, dtype, a, b, out=out, stream=stream)


studentT = _one("STUDENT_T", "n", 1.0)
studentT.__doc__ = "studentT(rows, cols, urng[, n]); studentT(urng, n) -> StudentTVGen (NormalExp.h:1512-1520)."


def chiSquared(rows, cols, urng, n=1.0, dtype=torch.float32, out=None, stream=None):
    return _sample("CHI_SQUARED", rows, cols, urng, dtype, n, out=out, stream=stream)


def poisson(rows, cols, urng, mean=1.0, out=None, stream=None):
    return _sample("POISSON", rows, cols, urng, torch.int32, mean, out=out, stream=stream)


def binomial(*args, trials=1, p=0.5, out=None, stream=None):
    """binomial(rows, cols, urng[, trials, p]) -> BinomialGen<int32_t>;
    binomial(urng, trials, p) with an int32 trials tensor and / or a float p
    tensor of the output's shape -> BinomialVGen<int32_t> (Discrete.h:1822-1898)."""
    if args and isinstance(args[0], (Vmt19937_64, _ScalarEngine)):
        urng, tr, pv = args[0], args[1], args[2]
        ta = _eigen_order(tr, torch.int32) if torch.is_tensor(tr) else None
        tb = _eigen_order(pv, torch.float32) if torch.is_tensor(pv) else None
        if ta is None and tb is None:
            raise TypeError("the per-element form needs a parameter tensor")
        if ta is not None and tb is not None and ta.shape != tb.shape:
            raise ValueError("trials and p must have the same shape")
        ref = ta if ta is not None else tb
        o = torch.empty_like(ref, dtype=torch.int32) if out is None else out
        d, keep = _desc("BINOMIAL", torch.int32, 0.0 if tb is not None else float(pv),
                        trials=0 if ta is not None else int(tr))
        vp = lambda t: _ptr(t) if t is not None else None
        fn = _L.gr_sengine_sample_v2 if isinstance(urng, _ScalarEngine) else _L.gr_sample_v2
        _lib.check(fn(urng._h, ctypes.byref(d), vp(ta), vp(tb), _ptr(o), o.numel(), _stream_ptr(stream)))
        del keep
        return o
    rows, cols, urng = args[:3]
    if len(args) > 3:
        trials = args[3]
    if len(args) > 4:
        p = args[4]
    return _sample("BINOMIAL", rows, cols, urng, torch.int32, p, trials=trials, out=out, stream=stream)


def discrete(rows, cols, urng, weights, out=None, stream=None):
    return _sample("DISCRETE", rows, cols, urng, torch.int32, weights=list(weights), out=out, stream=stream)


def randBits(rows, cols, urng, out=None, stream=None):
    return _sample("RANDBITS", rows, cols, urng, torch.int32, out=out, stream=stream)


def bernoulli(*args, p=0.5, dtype=torch.float32, out=None, stream=None):
    """bernoulli(rows, cols, urng, p=0.5) -> BernoulliGen; bernoulli(urng, p_tensor)
    -> BernoulliVGen<float>, one probability per element (Basic.h:1105-1153)."""
    if args and isinstance(args[0], Vmt19937_64):
        urng, pv = args[0], args[1]
        pv = _eigen_order(pv, torch.float32)
        o = torch.empty_like(pv) if out is None else out
        d, keep = _desc("BERNOULLI", torch.float32)
        _lib.check(_L.gr_sample_v(urng._h, ctypes.byref(d), _ptr(pv), _ptr(o), pv.numel(), _stream_ptr(stream)))
        del keep
        return o
    rows, cols, urng = args[:3]
    if len(args) > 3:
        p = args[3]
    return _sample("BERNOULLI", rows, cols, urng, dtype, p, out=out, stream=stream)


def fisherF(rows, cols, urng, m=1.0, n=1.0, dtype=torch.float32, out=None, stream=None):
    return _sample("FISHER_F", rows, cols, urng, dtype, m, n, out=out, stream=stream)


def uniformInt(rows, cols, urng, min, max, out=None, stream=None):
    return _sample("UNIFORM_INT", rows, cols, urng, torch.int32, float(min), float(max), out=out, stream=stream)


def negativeBinomial(rows, cols, urng, trials=1, p=0.5, out=None, stream=None):
    return _sample("NEGATIVE_BINOMIAL", rows, cols, urng, torch.int32, p, trials=trials, out=out, stream=stream)


def geometric(rows, cols, urng, p=0.5, out=None, stream=None):
    return _sample("GEOMETRIC", rows, cols, urng, torch.int32, p, out=out, stream=stream)


# ---- truncated distributions (Dists/Truncated.h) ---------------------------
_FINFO = {torch.float32: (-3.4028234663852886e38, 3.4028234663852886e38),
          torch.float64: (-1.7976931348623157e308, 1.7976931348623157e308)}


def _scalar(x, dtype):
    """x rounded to the scalar type, as the reference's Support<Scalar> holds it."""
    return float(torch.tensor(float(x), dtype=dtype).item())


class Support:
    """Support<Ty>{lower, upper} (Truncated.h:157-176)."""

    def __init__(self, lower, upper):
        self.lower = lower
        self.upper = upper

    def intersect(self, other):
        return Support(self.lower if self.lower > other.lower else other.lower,
                       self.upper if self.upper < other.upper else other.upper)


def support(lower, upper):
    """support(lower, upper) (Truncated.h:185-189)."""
    return Support(lower, upper)


def _trunc_args(base, sup):
    """(base generator, support in its scalar type) after merging nested
    TruncGens (TruncGen<TruncGen<B>>, Truncated.h:391-426)."""
    dt = base.dtype
    if sup is None:
        sup = Support(*_FINFO[dt])
    sup = Support(_scalar(sup.lower, dt), _scalar(sup.upper, dt))
    while isinstance(base, TruncGen):
        sup = base.support.intersect(sup)
        base = base.base
    return base, sup


class TruncGen(_Gen):
    """TruncGen<BaseGen>{base, support} (Truncated.h:202-263 and its
    specialisations :342-964).  Bases with a closed-form CDF (normal, standard
    normal, lognormal, exponential, Cauchy, extreme value, Weibull, the
    uniform family) draw by inverse CDF; gamma, beta, Student t, chi-squared,
    Fisher F and Bernoulli by CompressMask rejection over the base's packets
    (single-stream engines; each call synchronises its stream).  The base's
    caches start empty."""

    def __init__(self, base, support=None):
        base, sup = _trunc_args(base, support)
        self.base = base
        self.support = sup
        self.dtype = base.dtype
        self._desc, self._keep = base._desc, base._keep
        h = ctypes.c_void_p()
        _lib.check(_L.gr_gen_create_truncated(ctypes.byref(h), ctypes.byref(self._desc), sup.lower, sup.upper))
        self._h = h

    def getBase(self):
        return self.base

    def getSupport(self):
        return self.support


class TruncNormalGen(TruncGen):
    """TruncNormalGen<T>(mean, stdev, support) (Truncated.h:276-332): inverse
    CDF through erfinv, no rejection."""

    def __init__(self, mean=0.0, stdev=1.0, support=None, dtype=torch.float32):
        super().__init__(NormalGen(mean, stdev, dtype=dtype), support)


def truncated(rows, cols, urng, baseGen, support, out=None, stream=None):
    """truncated<Derived>(rows, cols, urng, baseGen, support) (Truncated.h:984-992)."""
    base, sup = _trunc_args(baseGen, support)
    o = _empty(rows, cols, base.dtype, out)
    _lib.check(_L.gr_sample_truncated(urng._h, ctypes.byref(base._desc), sup.lower, sup.upper, _ptr(o),
                                      rows * cols, _stream_ptr(stream)))
    return o


def truncatedLike(o, urng, baseGen, support, stream=None):
    """truncatedLike(o, urng, baseGen, support) (Truncated.h:1008-1016)."""
    return truncated(o.shape[0], o.shape[1], urng, baseGen, support, stream=stream)


def truncatedNormal(rows, cols, urng, mean, stdev, support, dtype=torch.float32, out=None, stream=None):
    """truncatedNormal<Derived>(rows, cols, urng, mean, stdev, support) (Truncated.h:1036-1045)."""
    return truncated(rows, cols, urng, NormalGen(mean, stdev, dtype=dtype), support, out=out, stream=stream)


def truncatedNormalLike(o, urng, mean, stdev, support, stream=None):
    """truncatedNormalLike(o, urng, mean, stdev, support) (Truncated.h:1061-1070)."""
    return truncatedNormal(o.shape[0], o.shape[1], urng, mean, stdev, support, dtype=o.dtype, stream=stream)


# ---- vectorize-over-params, many sets in one launch ------------------------
def sample_batched(kind, counts, a, b=None, trials=None, seed=5489, urng=None, out=None, offsets=None,
                   stream=None):
    """Draw counts[i] samples for each parameter set i in one launch.

    kind "GAMMA": GammaGen<float>(a[i], b[i]) -> float32.
    kind "BINOMIAL_V": BinomialVGen<int32_t> with (trials[i], p = a[i]) -> int32.
    Set i uses a fresh Vmt19937_64(seed + 4 i).  Returns (out, offsets)."""
    counts = counts.to(device="cuda", dtype=torch.int32).contiguous()
    a = a.to(device="cuda", dtype=torch.float32).contiguous()
    if offsets is None:
        offsets = torch.zeros(counts.numel(), dtype=torch.int64, device="cuda")
        if counts.numel() > 1:
            offsets[1:] = torch.cumsum(counts[:-1].to(torch.int64), 0)
    if out is None:  # sizing reads two values back; pass `out` to stay capturable
        total = int(offsets[-1].item() + counts[-1].item()) if counts.numel() else 0
        out = torch.empty(max(total, 1), dtype=torch.float32 if kind == "GAMMA" else torch.int32, device="cuda")
    bd = _lib.BatchDesc()
    bd.kind = KINDS[kind]
    bd.nsets = counts.numel()
    bd.seed = seed
    bd.a = a.data_ptr()
    keep = [a, counts, offsets]
    if b is not None:
        b = b.to(device="cuda", dtype=torch.float32).contiguous()
        bd.b = b.data_ptr()
        keep.append(b)
    if trials is not None:
        trials = trials.to(device="cuda", dtype=torch.int32).contiguous()
        bd.trials = trials.data_ptr()
        keep.append(trials)
    bd.counts = counts.data_ptr()
    bd.offsets = offsets.data_ptr()
    bd.out = out.data_ptr()
    eng = urng if urng is not None else _status_engine()
    _lib.check(_L.gr_sample_batched(eng._h, ctypes.byref(bd), _stream_ptr(stream)))
    del keep
    return out, offsets


_status_eng = None


def _status_engine():
    global _status_eng
    if _status_eng is None:
        _status_eng = Vmt19937_64(0)
    return _status_eng


# ---- multivariate generators (MvDists/*.h) ---------------------------------
def _host_f64(x, n=None):
    """Column-major float64 host copy of a vector / square matrix (numpy, torch
    or nested lists); returns (ctypes array, keep-alive)."""
    if isinstance(x, torch.Tensor):
        x = x.detach().to("cpu", torch.float64)
        flat = x.t().contiguous().reshape(-1).tolist() if x.dim() == 2 else x.reshape(-1).tolist()
    else:
        import numpy as np

        a = np.asarray(x, dtype=np.float64)
        flat = a.reshape(-1, order="F").tolist()
    if n is not None and len(flat) != n:
        raise ValueError(f"expected {n} values, got {len(flat)}")
    buf = (ctypes.c_double * len(flat))(*flat)
    return buf


class _MvGen:
    _prefix = None

    def _finish(self, h):
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _L is not None:
            getattr(_L, self._prefix + "_destroy")(h)
            self._h = None

    def dims(self):
        return self.dim


class MvNormalGen(_MvGen):
    """Eigen::Rand::MvNormalGen<float|double> (MvNormal.h:56-116).

    MvNormalGen(mean, cov) factors cov by get_lt (FP64 Cholesky on the GPU, or
    V sqrt(max(lambda, 0)) if not positive definite);
    MvNormalGen(mean, lt, lower_triangular=True) takes the factor itself.
    generate(urng, samples) -> (dim, samples) tensor, column-major like the
    Eigen matrix (each sample a contiguous column)."""

    _prefix = "gr_mvnormal"

    def __init__(self, mean, cov, lower_triangular=False, dtype=torch.float32):
        self.dim = len(mean) if not isinstance(mean, torch.Tensor) else mean.numel()
        self.dtype = dtype
        m = _host_f64(mean, self.dim)
        c = _host_f64(cov, self.dim * self.dim)
        h = ctypes.c_void_p()
        _lib.check(_L.gr_mvnormal_create(ctypes.byref(h), _DT[dtype], self.dim, m, c, 1 if lower_triangular else 0))
        self._finish(h)

    def generate(self, urng, samples=1, out=None, stream=None):
        o = out if out is not None else torch.empty((samples, self.dim), dtype=self.dtype, device="cuda").t()
        _lib.check(_L.gr_mvnormal_sample(self._h, urng._h, _ptr(o), samples, _stream_ptr(stream)))
        return o


class WishartGen(_MvGen):
    """Eigen::Rand::WishartGen (MvNormal.h:185-277): WishartGen(df, scale) or
    WishartGen(df, lt, lower_triangular=True).  generate(urng, samples) ->
    (dim, dim * samples) tensor, draw j in columns j*dim .. (j+1)*dim."""

    _prefix = "gr_wishart"
    _inverse = 0

    def __init__(self, df, scale, lower_triangular=False, dtype=torch.float32):
        import math

        self.dim = int(round(math.sqrt(len(_host_f64(scale)))))
        self.dtype = dtype
        self.df = int(df)
        c = _host_f64(scale, self.dim * self.dim)
        h = ctypes.c_void_p()
        _lib.check(_L.gr_wishart_create(ctypes.byref(h), _DT[dtype], self.dim, ctypes.c_int64(self.df), c,
                                        1 if lower_triangular else 0, self._inverse))
        self._finish(h)

    def generate(self, urng, samples=1, out=None, stream=None):
        d = self.dim
        o = out if out is not None else torch.empty((d * samples, d), dtype=self.dtype, device="cuda").t()
        _lib.check(_L.gr_wishart_sample(self._h, urng._h, _ptr(o), samples, _stream_ptr(stream)))
        return o


class InvWishartGen(WishartGen):
    """Eigen::Rand::InvWishartGen (MvNormal.h:347-442): InvWishartGen(df, scale)
    or InvWishartGen(df, ilt, inv_lower_triangular=True)."""

    _inverse = 1

    def __init__(self, df, scale, inv_lower_triangular=False, dtype=torch.float32):
        super().__init__(df, scale, lower_triangular=inv_lower_triangular, dtype=dtype)


class DirichletGen(_MvGen):
    """Eigen::Rand::DirichletGen (Multinomial.h:160-204).  generate(urng,
    samples) -> (dim, samples) tensor."""

    _prefix = "gr_dirichlet"

    def __init__(self, alpha, dtype=torch.float32):
        a = _host_f64(alpha)
        self.dim = len(a)
        self.dtype = dtype
        h = ctypes.c_void_p()
        _lib.check(_L.gr_dirichlet_create(ctypes.byref(h), _DT[dtype], self.dim, a))
        self._finish(h)

    def generate(self, urng, samples=1, out=None, stream=None):
        o = out if out is not None else torch.empty((samples, self.dim), dtype=self.dtype, device="cuda").t()
        _lib.check(_L.gr_dirichlet_sample(self._h, urng._h, _ptr(o), samples, _stream_ptr(stream)))
        return o


class MultinomialGen(_MvGen):
    """Eigen::Rand::MultinomialGen<int32_t> (Multinomial.h:25-118).
    generate(urng, samples) -> int32 (dim, samples) tensor of counts."""

    _prefix = "gr_multinomial"

    def __init__(self, trials, weights):
        w = _host_f64(weights)
        self.dim = len(w)
        self.trials = int(trials)
        self.dtype = torch.int32
        h = ctypes.c_void_p()
        _lib.check(_L.gr_multinomial_create(ctypes.byref(h), self.dim, self.trials, w))
        self._finish(h)

    def generate(self, urng, samples=1, out=None, stream=None):
        o = out if out is not None else torch.empty((samples, self.dim), dtype=torch.int32, device="cuda").t()
        _lib.check(_L.gr_multinomial_sample(self._h, urng._h, _ptr(o), samples, _stream_ptr(stream)))
        return o


class TruncMvNormalGen(_MvGen):
    """Eigen::Rand::TruncMvNormalGen<T> (MvDists/TruncMvNormal.h:31-209):
    TruncMvNormalGen(mean, cov, support(lower, upper), burn_in=0) or, with
    lower_triangular=True, the covariance's factor.  generate(urng, samples)
    -> (dim, samples) tensor; each column is a Gibbs chain of burn_in sweeps
    (0 = 5 * dim)."""

    _prefix = "gr_truncmvn"

    def __init__(self, mean, cov, support, burn_in=0, lower_triangular=False, dtype=torch.float32):
        m = _host_f64(mean)
        self.dim = len(m)
        self.dtype = dtype
        c = _host_f64(cov, self.dim * self.dim)
        lo = _host_f64(support.lower, self.dim)
        hi = _host_f64(support.upper, self.dim)
        h = ctypes.c_void_p()
        _lib.check(_L.gr_truncmvn_create(ctypes.byref(h), _DT[dtype], self.dim, m, c,
                                         1 if lower_triangular else 0, lo, hi, int(burn_in)))
        self._finish(h)

    def generate(self, urng, samples=1, out=None, stream=None):
        o = out if out is not None else torch.empty((samples, self.dim), dtype=self.dtype, device="cuda").t()
        _lib.check(_L.gr_truncmvn_sample(self._h, urng._h, _ptr(o), samples, _stream_ptr(stream)))
        return o


def makeTruncMvNormalGen(mean, cov, support, burn_in=0, dtype=torch.float32):
    return TruncMvNormalGen(mean, cov, support, burn_in, dtype=dtype)


def makeTruncMvNormalGenFromLt(mean, lt, support, burn_in=0, dtype=torch.float32):
    return TruncMvNormalGen(mean, lt, support, burn_in, lower_triangular=True, dtype=dtype)


def makeMvNormalGen(mean, cov, dtype=torch.float32):
    return MvNormalGen(mean, cov, dtype=dtype)


def makeMvNormalGenFromLt(mean, lt, dtype=torch.float32):
    return MvNormalGen(mean, lt, lower_triangular=True, dtype=dtype)


def makeWishartGen(df, scale, dtype=torch.float32):
    return WishartGen(df, scale, dtype=dtype)


def makeWishartGenFromLt(df, lt, dtype=torch.float32):
    return WishartGen(df, lt, lower_triangular=True, dtype=dtype)


def makeInvWishartGen(df, scale, dtype=torch.float32):
    return InvWishartGen(df, scale, dtype=dtype)


def makeInvWishartGenFromIlt(df, ilt, dtype=torch.float32):
    return InvWishartGen(df, ilt, inv_lower_triangular=True, dtype=dtype)


def makeDirichletGen(alpha, dtype=torch.float32):
    return DirichletGen(alpha, dtype=dtype)


def makeMultinomialGen(trials, weights):
    return MultinomialGen(trials, weights)
