"""GPU parity of scalar engines as the Urng (std::mt19937_64, P8_mt19937_64)
against the CPU oracle, bit-exact, through the C ABI."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def er(gpulib):
    return gpulib


def mem(t):
    torch.cuda.synchronize()
    if t.dim() == 2:
        t = t.t()
    return t.contiguous().reshape(-1).cpu().numpy()


def assert_bits_equal(a, b, msg=""):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    ua = a.view(np.uint64 if a.itemsize == 8 else np.uint32)
    ub = b.view(np.uint64 if b.itemsize == 8 else np.uint32)
    bad = np.nonzero(ua != ub)[0]
    assert bad.size == 0, f"{msg}: {bad.size} mismatches, first at {bad[:5]}: {a[bad[:5]]} vs {b[bad[:5]]}"


ENGINES = [("mt19937_64", "mt19937_64"), ("p8", "P8_mt19937_64")]


def test_mt19937_64_known_answer(er):
    """std::mt19937_64's 10000th output for the default seed, drawn on the GPU."""
    x = er.mt19937_64(5489).raw(10000).cpu().numpy().view(np.uint64)
    assert int(x[-1]) == 9981545732273789042


@pytest.mark.parametrize("okind,cls", ENGINES)
def test_scalar_engine_raw_stream(er, oracle, okind, cls):
    """rng() in calls of odd sizes (P8's eight-lane buffer carried between
    calls) and a long one (jump-ahead segments)."""
    u = getattr(er, cls)(42)
    o = oracle.ScalarEngine(okind, 42)
    for n in (3, 5, 13, 1 << 20, 8, 7, 100001):
        assert_bits_equal(u.raw(n).cpu().numpy().view(np.uint64), o.raw(n), f"{cls} n={n}")


KINDS = [("UNIFORM_REAL", 0, 0), ("UNIFORM_REAL2", -2.0, 3.0), ("BALANCED", 0, 0), ("BALANCED2", -3.0, 5.0),
         ("NORMAL_STD", 0, 0), ("NORMAL", 2.0, 3.0), ("LOGNORMAL", 0.0, 1.0), ("EXPONENTIAL", 1.5, 0),
         ("CAUCHY", 0.0, 1.0), ("WEIBULL", 1.5, 2.0), ("EXTREME_VALUE", 0.0, 1.0), ("GAMMA", 1.0, 2.0),
         ("BERNOULLI", 0.3, 0)]


@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
@pytest.mark.parametrize("kind,a,b", KINDS, ids=[k[0] for k in KINDS])
@pytest.mark.parametrize("okind,cls", ENGINES, ids=["mt", "p8"])
def test_scalar_engine_distributions(er, oracle, okind, cls, kind, a, b, tdt):
    """Fixed-draw kinds through RawbitsMaker<..., scalar_fullbit>: 3 draws per
    float uniform packet (rawbits_34), 4 per double or raw-bits packet, 2 per
    half packet; consecutive free-function calls (fresh generators)."""
    npt = np.float32 if tdt == torch.float32 else np.float64
    P = 8 if tdt == torch.float32 else 4
    u = getattr(er, cls)(1234)
    o = oracle.ScalarEngine(okind, 1234)
    for n in (P, 3 * P, 1 << 20, 5 * P):
        d, keep = er._desc(kind, tdt, a, b)
        out = torch.empty(n, dtype=tdt, device="cuda")
        er._lib.check(er._L.gr_sengine_sample(u._h, er.ctypes.byref(d), er._ptr(out), n, er._stream_ptr()))
        ref = o.generate(oracle.Gen(), kind, n, npt, a, b)
        assert_bits_equal(mem(out), ref, f"{kind} {cls} {tdt} n={n}")


@pytest.mark.parametrize("okind,cls", ENGINES, ids=["mt", "p8"])
def test_scalar_engine_randbits_and_mirror(er, oracle, okind, cls):
    """RandbitsGen<int32_t> (Packet4i rawbits: 2 draws per packet), the Python
    mirror's free functions on a scalar engine, and refused kinds."""
    u = getattr(er, cls)(7)
    o = oracle.ScalarEngine(okind, 7)
    for n in (4, 12, 1 << 18):
        assert_bits_equal(mem(er.randBits(n, 1, u)), o.generate(None, "RANDBITS", n), f"randbits n={n}")
    x = mem(er.normal(64, 64, u, 1.0, 2.0))
    assert_bits_equal(x, o.generate(oracle.Gen(), "NORMAL", 4096, np.float32, 1.0, 2.0), "normal mirror")
    x = mem(er.ExponentialGen(2.0, dtype=torch.float64).generate(32, 32, u))
    assert_bits_equal(x, o.generate(oracle.Gen(), "EXPONENTIAL", 1024, np.float64, 2.0), "object mirror")
    with pytest.raises(er.GrError):
        er.NormalGen().generate(8, 1, u)


@pytest.mark.parametrize("okind,cls", ENGINES)
def test_scalar_engine_binomial_v(er, oracle, okind, cls):
    """binomial(urng, trials, p) with a scalar engine (the reference's own
    binomialV test uses P8_mt19937_64{42}: test.cpp:470-490): its three
    overloads on the test's shapes, a call large enough for several chunks of
    pre-drawn words, and raw draws after each call (the engine stands exactly
    past the words the packets used)."""
    u = getattr(er, cls)(42)
    o = oracle.ScalarEngine(okind, 42)
    a = np.linspace(5, 50, 10).astype(np.int32)
    b = np.linspace(0.1, 1.0, 10).astype(np.float32)
    A = np.tile(a[:, None], (1, 100))
    B = np.tile(b[:, None], (1, 100))
    got = er.binomial(u, torch.from_numpy(A), 0.5)
    assert_bits_equal(mem(got), o.binomial_v(A.T.reshape(-1), 0.5), "trials array, p 0.5")
    got = er.binomial(u, 50, torch.from_numpy(B))
    assert_bits_equal(mem(got), o.binomial_v(50, B.T.reshape(-1)), "trials 50, p array")
    got = er.binomial(u, torch.from_numpy(A), torch.from_numpy(B))
    assert_bits_equal(mem(got), o.binomial_v(A.T.reshape(-1), B.T.reshape(-1)), "both arrays")
    assert_bits_equal(u.raw(5).cpu().numpy().view(np.uint64), o.raw(5), "raw after")
    r = np.random.default_rng(8)
    n = 4 * 30000
    tr = r.choice(np.array([0, 3, 20, 100, 5000], np.int32), n)
    p = r.random(n).astype(np.float32)
    got = er.binomial(u, torch.from_numpy(tr), torch.from_numpy(p))
    assert_bits_equal(mem(got), o.binomial_v(tr, p), "long call")
    assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), "raw after the long call")
    with pytest.raises(er.GrError):
        er.normal(u, torch.ones(8), torch.ones(8))


INT_CASES = [("POISSON", 0.5, 0), ("POISSON", 4.0, 0), ("POISSON", 11.9, 0), ("POISSON", 12.0, 0),
             ("POISSON", 100.0, 0), ("BINOMIAL", 0.3, 10), ("BINOMIAL", 0.8, 24), ("BINOMIAL", 0.005, 100),
             ("BINOMIAL", 0.995, 100), ("BINOMIAL", 0.3, 100), ("BINOMIAL", 0.7, 1000), ("BINOMIAL", 0.5, 0)]


@pytest.mark.parametrize("okind,cls", ENGINES)
def test_scalar_engine_poisson_binomial(er, oracle, okind, cls):
    """poisson() / binomial() (fresh PoissonGen / BinomialGen<int32_t>) with a
    scalar engine: every branch (the trials < 25 sum, the multiplicative
    loop, the tan rejection through CompressMask with lanes carried across
    chunks of pre-drawn words, p > 1/2), calls of several sizes in a row, and
    raw draws after them."""
    u = getattr(er, cls)(2024)
    o = oracle.ScalarEngine(okind, 2024)
    for kind, a, trials in INT_CASES:
        for rows, cols in ((4, 3), (256, 512)):
            if kind == "POISSON":
                got = er.poisson(rows, cols, u, a)
            else:
                got = er.binomial(rows, cols, u, trials, a)
            ref = o.generate(None, kind, rows * cols, np.int32, a, trials=trials)
            assert_bits_equal(mem(got), ref, f"{cls} {kind} {a} {trials} {rows}x{cols}")
        assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), f"{cls} raw after {kind} {a}")


@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
@pytest.mark.parametrize("okind,cls", ENGINES)
def test_scalar_engine_gamma_rejection(er, oracle, okind, cls, tdt):
    """gamma() with a scalar engine on its rejection branches (GS for
    alpha < 1, the tan proposal otherwise; a fresh GammaGen per call):
    candidates of a chunk of trials evaluated at once, CompressMask order
    through the filter, the engine left just past the trial that emitted the
    last output; chiSquared on the same path."""
    npt = np.float32 if tdt == torch.float32 else np.float64
    u = getattr(er, cls)(31)
    o = oracle.ScalarEngine(okind, 31)
    for alpha, beta in ((0.2, 1.0), (0.5, 2.0), (0.93, 1.0), (1.5, 1.0), (2.5, 0.5), (7.3, 1.0)):
        for rows, cols in ((8, 3), (384, 512)):
            got = er.gamma(rows, cols, u, alpha, beta, dtype=tdt)
            ref = o.generate(oracle.Gen(), "GAMMA", rows * cols, npt, alpha, beta)
            assert_bits_equal(mem(got), ref, f"{cls} gamma({alpha}, {beta}) {tdt} {rows}x{cols}")
        assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), f"{cls} raw after gamma({alpha})")
    got = er.chiSquared(64, 64, u, 3.0, dtype=tdt)
    ref = o.generate(oracle.Gen(), "GAMMA", 64 * 64, npt, 1.5, 2.0)
    assert_bits_equal(mem(got), ref, f"{cls} chiSquared(3)")
    # integral alpha < 20: the product of alpha uniforms, and studentT: two
    # uniform packets per output packet
    for alpha, beta in ((2.0, 1.0), (3.0, 0.5), (19.0, 1.0)):
        got = er.gamma(64, 40, u, alpha, beta, dtype=tdt)
        ref = o.generate(oracle.Gen(), "GAMMA", 64 * 40, npt, alpha, beta)
        assert_bits_equal(mem(got), ref, f"{cls} gamma({alpha}, {beta}) {tdt}")
    for nu in (1.0, 4.5):
        got = er.studentT(96, 32, u, nu, dtype=tdt)
        ref = o.generate(oracle.Gen(), "STUDENT_T", 96 * 32, npt, nu)
        assert_bits_equal(mem(got), ref, f"{cls} studentT({nu}) {tdt}")
    assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), f"{cls} raw after the staged kinds")


BETAS = [(0.5, 0.7), (0.2, 0.9), (0.5, 2.0), (2.5, 3.5), (1.0, 2.5), (2.0, 3.0), (0.3, 1.0), (7.3, 0.8)]


@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
@pytest.mark.parametrize("okind,cls", ENGINES, ids=["mt", "p8"])
def test_scalar_engine_beta_fisherf(er, oracle, okind, cls, tdt):
    """beta() and fisherF() with a scalar engine (a fresh BetaGen per call):
    the a, b < 1 rejection loop, and the general branch's GammaGen(a) then
    GammaGen(b) per output packet on every gamma branch (GS, alpha = 1,
    integral alpha, the tan proposal), each with its own carried lanes; the
    engine continues exactly after each call."""
    npt = np.float32 if tdt == torch.float32 else np.float64
    u = getattr(er, cls)(41)
    o = oracle.ScalarEngine(okind, 41)
    for a, b in BETAS:
        for rows, cols in ((8, 1), (256, 96)):
            got = er.beta(rows, cols, u, a, b, dtype=tdt)
            ref = o.generate(oracle.Gen(), "BETA", rows * cols, npt, a, b)
            assert_bits_equal(mem(got), ref, f"{cls} beta({a}, {b}) {tdt} {rows}x{cols}")
        assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), f"{cls} raw after beta({a}, {b})")
    for m, n in ((1.0, 1.5), (5.0, 2.0), (10.0, 12.0)):
        got = er.fisherF(128, 64, u, m, n, dtype=tdt)
        ref = o.generate(oracle.Gen(), "FISHER_F", 128 * 64, npt, m, n)
        assert_bits_equal(mem(got), ref, f"{cls} fisherF({m}, {n}) {tdt}")
    assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), f"{cls} raw after fisherF")


def test_scalar_engine_beta_multichunk(er, oracle):
    """Calls whose chain outruns its first chunk of words: the carried lanes
    of both gammas (and of the a, b < 1 loop) continue into the next chunk."""
    u = er.mt19937_64(6)
    o = oracle.ScalarEngine("mt19937_64", 6)
    for a, b, n in ((0.9, 0.8, 8 * 1_500_000), (0.4, 2.5, 8 * 1_000_000)):  # > 2^24 words each
        got = er.beta(n, 1, u, a, b)
        ref = o.generate(oracle.Gen(), "BETA", n, np.float32, a, b)
        assert_bits_equal(mem(got), ref, f"beta({a}, {b}) multi-chunk")
    assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), "raw after")


def test_scalar_engine_gamma_multichunk(er, oracle):
    """A call needing more trials than one chunk holds: the first chunk runs
    out with lanes carried into the next."""
    u = er.mt19937_64(5)
    o = oracle.ScalarEngine("mt19937_64", 5)
    n = 8 * 4_700_000
    got = er.gamma(n, 1, u, 0.5, 1.0)
    ref = o.generate(oracle.Gen(), "GAMMA", n, np.float32, 0.5, 1.0)
    assert_bits_equal(mem(got), ref, "gamma(0.5) multi-chunk")
    assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), "raw after")


@pytest.mark.parametrize("okind,cls", ENGINES)
def test_scalar_engine_uniform_int(er, oracle, okind, cls):
    """uniformInt() (a fresh UniformIntGen<int32_t>) with a scalar engine:
    constant, masked and rejection ranges (bit slices shifted out of one
    draw, or a new draw per slice), and raw draws after the calls."""
    u = getattr(er, cls)(77)
    o = oracle.ScalarEngine(okind, 77)
    for lo, hi in ((0, 9), (-5, 10), (3, 3), (0, 1000000), (0, 100), (-1000, 1000)):
        for rows, cols in ((4, 5), (300, 200)):
            got = er.uniformInt(rows, cols, u, lo, hi)
            ref = o.generate(None, "UNIFORM_INT", rows * cols, np.int32, lo, hi)
            assert_bits_equal(mem(got), ref, f"{cls} uniformInt({lo}, {hi}) {rows}x{cols}")
    assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), f"{cls} raw after")


@pytest.mark.parametrize("okind,cls", ENGINES)
def test_scalar_engine_bernoulli_geometric_int(er, oracle, okind, cls):
    """BernoulliGen<int32_t> and GeometricGen<int32_t> with a scalar engine:
    one SSE packet of two draws per output packet."""
    u = getattr(er, cls)(13)
    o = oracle.ScalarEngine(okind, 13)
    for p in (0.3, 0.9):
        got = er.bernoulli(200, 40, u, p, dtype=torch.int32)
        assert_bits_equal(mem(got), o.generate(None, "BERNOULLI", 8000, np.int32, p), f"{cls} bernoulli({p})")
        got = er.geometric(200, 40, u, p)
        assert_bits_equal(mem(got), o.generate(None, "GEOMETRIC", 8000, np.int32, p), f"{cls} geometric({p})")
    assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), f"{cls} raw after")


@pytest.mark.parametrize("okind,cls", ENGINES)
def test_scalar_engine_discrete(er, oracle, okind, cls):
    """discrete() (a fresh DiscreteGen<int32_t>) with a scalar engine: the CDF
    (< 16 weights) and alias-table forms, even and odd packet counts (an odd
    last packet draws a whole Packet8i), and raw draws after the calls."""
    u = getattr(er, cls)(21)
    o = oracle.ScalarEngine(okind, 21)
    r = np.random.default_rng(2)
    for nw in (5, 16, 100):
        w = r.uniform(0.1, 2.0, nw)
        for rows, cols in ((4, 3), (256, 130)):
            got = er.discrete(rows, cols, u, w)
            assert_bits_equal(mem(got), o.discrete(w, rows * cols), f"{cls} discrete({nw}) {rows}x{cols}")
        assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), f"{cls} raw after discrete({nw})")


@pytest.mark.parametrize("okind,cls", ENGINES)
def test_scalar_engine_negative_binomial(er, oracle, okind, cls):
    """negativeBinomial() (a fresh NegativeBinomialGen<int32_t>) with a scalar
    engine: the gamma's exponential / product / tan forms, Poisson means below
    and above 12 (the tan rejection sharing the gamma's CompressMask cache),
    and raw draws after the calls."""
    u = getattr(er, cls)(33)
    o = oracle.ScalarEngine(okind, 33)
    for trials, p in ((1, 0.3), (5, 0.5), (25, 0.8), (30, 0.1), (3, 0.05)):
        for rows, cols in ((4, 3), (128, 96)):
            got = er.negativeBinomial(rows, cols, u, trials, p)
            ref = o.generate(None, "NEGATIVE_BINOMIAL", rows * cols, np.int32, p, trials=trials)
            assert_bits_equal(mem(got), ref, f"{cls} negativeBinomial({trials}, {p}) {rows}x{cols}")
    assert_bits_equal(u.raw(3).cpu().numpy().view(np.uint64), o.raw(3), f"{cls} raw after")
