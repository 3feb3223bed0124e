"""GPU parity of the truncated family (EigenRand/Dists/Truncated.h) against
the CPU oracle, bit-exact, through the C ABI.

The oracle computes the constructors' constants with this machine's C
library, like the library does, so the comparison runs live here rather than
against fixtures written elsewhere."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

F32MAX = 3.4028234663852886e38
F64MAX = 1.7976931348623157e308


@pytest.fixture(scope="module")
def er(gpulib):
    return gpulib


def mem(t):
    torch.cuda.synchronize()
    if t.dim() == 2:
        t = t.t()
    return t.contiguous().reshape(-1).cpu().numpy()


def npdt(tdt):
    return {torch.float32: np.float32, torch.float64: np.float64}[tdt]


def assert_bits_equal(a, b, msg=""):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    ua = a.view(np.uint64 if a.itemsize == 8 else np.uint32)
    ub = b.view(np.uint64 if b.itemsize == 8 else np.uint32)
    bad = np.nonzero(ua != ub)[0]
    assert bad.size == 0, f"{msg}: {bad.size} mismatches, first at {bad[:5]}: {a[bad[:5]]} vs {b[bad[:5]]}"


def assert_within(x, lo, hi, tdt):
    """Inside [lo, hi] up to the inverse CDF's rounding: evaluated in the
    scalar type it can land just outside a bound, by more in a far tail where
    1 - u keeps few significant bits (the reference's own tests check the
    plain bounds on 64 values).  Where UniformRealGen's value rounds to 1 (or
    1 - 2u to 1) in the scalar type, TruncNormalGen's arithmetic gives
    erfinv(-+1) and an infinity of the opposite sign, as the reference does;
    those lanes are rare and are left out of the check."""
    eps = 1e-4 if tdt == torch.float32 else 1e-9
    x = np.asarray(x, np.float64)
    fin = np.isfinite(x)
    assert fin.mean() > 1 - 1e-3
    x = x[fin]
    assert x.min() >= lo - eps * max(1.0, abs(lo)) and x.max() <= hi + eps * max(1.0, abs(hi)), (x.min(), x.max())


def fmax(tdt):
    return F32MAX if tdt == torch.float32 else F64MAX


# (base kind, a, b, lower, upper); None = the scalar type's lowest() / max()
INVERSE_CDF = [
    ("NORMAL", 0.0, 1.0, -1.0, 1.0),          # truncatedNormalGeneric, test.cpp:1094-1114
    ("NORMAL", 2.0, 3.0, 0.0, 10.0),
    ("NORMAL_STD", 0.0, 0.0, -0.5, 2.0),      # truncatedStdNormalSpecialized
    ("NORMAL", 0.0, 1.0, 0.0, None),          # truncatedNormalOneSided
    ("NORMAL", 0.0, 1.0, None, 0.0),
    ("NORMAL", 0.0, 1.0, 3.5, 6.0),           # erfinv's middle region
    ("NORMAL", 0.0, 1.0, 5.5, 9.0),           # double erfinv's tail region
    ("NORMAL", 0.0, 1.0, -9.0, -5.5),
    ("EXPONENTIAL", 1.0, 0.0, 0.5, 3.0),      # truncatedExponential
    ("EXPONENTIAL", 2.0, 0.0, 0.1, 1.0),
    ("EXPONENTIAL", 1.0, 0.0, -1.0, 2.0),     # lower clamped to 0
    ("CAUCHY", 0.0, 1.0, -2.0, 2.0),          # truncatedCauchySpecialized
    ("CAUCHY", 0.0, 1.0, 0.0, None),
    ("LOGNORMAL", 0.0, 1.0, 0.5, 3.0),        # truncatedLognormalSpecialized
    ("LOGNORMAL", 0.0, 1.0, -1.0, 2.0),       # lower <= 0 -> lowest()
    ("EXTREME_VALUE", 0.0, 1.0, -1.0, 2.0),   # truncatedExtremeValueSpecialized
    ("WEIBULL", 2.0, 1.0, 0.3, 1.5),          # truncatedWeibullSpecialized
    ("WEIBULL", 1.5, 2.0, 0.5, 3.0),
    ("UNIFORM_REAL2", 0.0, 10.0, 2.0, 8.0),   # truncatedUniformSpecialized
    ("UNIFORM_REAL2", 0.0, 10.0, -5.0, 20.0),
    ("UNIFORM_REAL", 0.0, 0.0, 0.2, 0.8),     # truncatedStdUniformSpecialized
    ("BALANCED", 0.0, 0.0, -0.5, 0.5),        # truncatedBalancedSpecialized
    ("BALANCED2", 0.0, 10.0, 2.0, 8.0),       # truncatedBalanced2Specialized
]

REJECT = [
    ("GAMMA", 2.0, 1.0, 0.5, 5.0),            # truncatedGamma, test.cpp:1136-1154
    ("GAMMA", 0.5, 1.0, 0.1, 1.0),
    ("GAMMA", 7.5, 2.0, 10.0, 20.0),
    ("BETA", 2.0, 3.0, 0.2, 0.6),
    ("BETA", 0.5, 0.5, 0.1, 0.9),
    ("STUDENT_T", 5.0, 0.0, -1.0, 1.0),
    ("CHI_SQUARED", 3.0, 0.0, 1.0, 4.0),
    ("FISHER_F", 4.0, 6.0, 0.5, 2.0),
    ("BERNOULLI", 0.3, 0.0, 0.5, 1.0),
]


def _bounds(tdt, lo, hi):
    return (-fmax(tdt) if lo is None else lo), (fmax(tdt) if hi is None else hi)


@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
@pytest.mark.parametrize("case", INVERSE_CDF, ids=lambda c: f"{c[0]}_{c[3]}_{c[4]}")
def test_trunc_inverse_cdf_bit_exact(er, oracle, case, tdt):
    """Inverse-CDF specialisations: consecutive calls of one TruncGen,
    including a long one split into jump-ahead segments, and the free
    function; every value inside the support."""
    kind, a, b, lo, hi = case
    lo, hi = _bounds(tdt, lo, hi)
    P = 8 if tdt == torch.float32 else 4
    u = er.Vmt19937_64(42)
    e = oracle.Engine(42)
    og = oracle.Gen()
    g = er.TruncGen(er._Gen(tdt, a, b, kind=kind), er.support(lo, hi))
    for n in (P, 1000 * P, 1 << 20, 3 * P):
        ref = oracle.truncated(e, og, kind, n, lo, hi, npdt(tdt), a, b)
        got = mem(g.generate(n, 1, u))
        assert_bits_equal(got, ref, f"{kind} [{lo}, {hi}] {tdt} n={n}")
        if not (tdt == torch.float32 and abs(lo) >= 5.5):
            # beyond 5.5 sigma float's 1 - 2u holds almost no bits: the
            # reference's arithmetic gives infinities for most lanes there
            assert_within(got, lo, hi, tdt)
    ref = oracle.truncated(e, oracle.Gen(), kind, 4096, lo, hi, npdt(tdt), a, b)
    got = mem(er.truncated(4096, 1, u, er._Gen(tdt, a, b, kind=kind), er.support(lo, hi)))
    assert_bits_equal(got, ref, f"{kind} free function")


@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
@pytest.mark.parametrize("case", REJECT, ids=lambda c: f"{c[0]}_{c[1]}_{c[3]}_{c[4]}")
def test_trunc_rejection_bit_exact(er, oracle, case, tdt):
    """Generic TruncGen (CompressMask over the base's packets): calls of a
    few packets (pilot chunks), long calls that stop inside a chunk (the
    engine and the base rewind and redraw), lanes carried between calls, and
    the engine state after the last call."""
    kind, a, b, lo, hi = case
    P = 8 if tdt == torch.float32 else 4
    u = er.Vmt19937_64(1234)
    e = oracle.Engine(1234)
    og = oracle.Gen()
    g = er.TruncGen(er._Gen(tdt, a, b, kind=kind), er.support(lo, hi))
    for n in (3 * P, 5000 * P, 1 << 18, P, 77 * P):
        ref = oracle.truncated(e, og, kind, n, lo, hi, npdt(tdt), a, b)
        got = mem(g.generate(n, 1, u))
        assert_bits_equal(got, ref, f"trunc {kind}({a},{b}) [{lo}, {hi}] {tdt} n={n}")
    assert_bits_equal(er.raw_u64(u, 4096).cpu().numpy().view(np.uint64), e.raw(1024), "engine after the calls")


def test_trunc_nested_and_truncnormal(er, oracle):
    """TruncGen<TruncGen<B>> draws as TruncGen<B> over the intersection
    (test.cpp:1196-1234); TruncNormalGen / truncatedNormal are TruncGen of
    NormalGen (:1404-1432)."""
    for tdt in (torch.float32, torch.float64):
        u = er.Vmt19937_64(7)
        e = oracle.Engine(7)
        inner = er.TruncGen(er.NormalGen(0.0, 1.0, dtype=tdt), er.support(-3.0, 3.0))
        g = er.TruncGen(er.TruncGen(inner, er.support(-5.0, 5.0)), er.support(-1.0, 4.0))
        assert (g.support.lower, g.support.upper) == (-1.0, 3.0)
        ref = oracle.truncated(e, oracle.Gen(), "NORMAL", 8192, -1.0, 3.0, npdt(tdt), 0.0, 1.0)
        assert_bits_equal(mem(g.generate(8192, 1, u)), ref, "nested normal")
        inner = er.TruncGen(er.GammaGen(2.0, 1.0, dtype=tdt), er.support(0.5, 5.0))
        g = er.TruncGen(inner, er.support(1.0, 8.0))
        og = oracle.Gen()
        for n in (64, 8192):
            ref = oracle.truncated(e, og, "GAMMA", n, 1.0, 5.0, npdt(tdt), 2.0, 1.0)
            assert_bits_equal(mem(g.generate(n, 1, u)), ref, "nested gamma")
        tn = er.TruncNormalGen(0.0, 1.0, er.support(-1.0, 2.0), dtype=tdt)
        ref = oracle.truncated(e, oracle.Gen(), "NORMAL", 4096, -1.0, 2.0, npdt(tdt), 0.0, 1.0)
        assert_bits_equal(mem(tn.generate(64, 64, u)), ref, "TruncNormalGen")
        ref = oracle.truncated(e, oracle.Gen(), "NORMAL", 4096, -1.0, 2.0, npdt(tdt), 0.0, 1.0)
        assert_bits_equal(mem(er.truncatedNormal(64, 64, u, 0.0, 1.0, er.support(-1.0, 2.0), dtype=tdt)), ref,
                          "truncatedNormal")


def test_trunc_streams_and_errors(er, oracle):
    """Inverse-CDF forms on a multi-stream engine (slice k from engine seed +
    4k); the rejection form needs one stream; ragged sizes are refused."""
    K, per = 4, 8 * 2000
    u = er.Vmt19937_64(99, streams=K)
    x = mem(er.truncated(K * per, 1, u, er.NormalGen(1.0, 2.0), er.support(-1.0, 2.5)))
    for k in range(K):
        ref = oracle.truncated(oracle.Engine(99 + 4 * k), oracle.Gen(), "NORMAL", per, -1.0, 2.5, np.float32,
                               1.0, 2.0)
        assert_bits_equal(x[k * per:(k + 1) * per], ref, f"slice {k}")
    g = er.TruncGen(er.GammaGen(2.0, 1.0), er.support(0.5, 5.0))
    with pytest.raises(er.GrError):
        g.generate(64, 1, u)
    with pytest.raises(er.GrError):
        er.truncated(12, 1, er.Vmt19937_64(1), er.NormalGen(), er.support(-1.0, 1.0))


def test_trunc_bounds_full_size(er):
    """Every value of a 4096 x 4096 draw inside its support, and the
    truncated normal's mean against the closed form."""
    from scipy import stats
    u = er.Vmt19937_64(42)
    x = er.truncatedNormal(4096, 4096, u, 0.0, 1.0, er.support(-1.0, 2.0))
    assert_within(np.array([float(x.min()), float(x.max())]), -1.0, 2.0, torch.float32)
    m = float(x.double().mean())
    assert abs(m - stats.truncnorm(-1.0, 2.0).mean()) < 2e-3
    g = er.TruncGen(er.GammaGen(2.0, 1.0), er.support(0.5, 5.0))
    y = g.generate(4096, 4096, u)
    assert float(y.min()) >= 0.5 and float(y.max()) <= 5.0
