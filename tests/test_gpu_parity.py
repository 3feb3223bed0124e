"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Bit-exact comparisons throughout: the engine is integer work, the uniform
transforms are exact, and the transcendental steps use the same operation
sequence on both sides (csrc/gr_math.cuh, oracle/ormath.c)."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import golden_cases  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def er(gpulib):
    return gpulib


def mem(t):
    """Eigen linear (column-major) order of a (rows, cols) output."""
    torch.cuda.synchronize()
    if t.dim() == 2:
        t = t.t()
    return t.contiguous().reshape(-1).cpu().numpy()


def npdt(tdt):
    return {torch.float32: np.float32, torch.float64: np.float64, torch.int32: np.int32}[tdt]


def assert_bits_equal(a, b, msg=""):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    ua = a.view(np.uint64 if a.itemsize == 8 else np.uint32)
    ub = b.view(np.uint64 if b.itemsize == 8 else np.uint32)
    bad = np.nonzero(ua != ub)[0]
    assert bad.size == 0, f"{msg}: {bad.size} mismatches, first at {bad[:5]}: {a[bad[:5]]} vs {b[bad[:5]]}"


# ---------------------------------------------------------------- engine
def test_raw_stream_config1_2pow24(er, oracle):
    """Vmt19937_64{42}, 2^24 raw uint64 draws: bit-exact (jump-ahead segments)."""
    u = er.Vmt19937_64(42)
    g = er.raw_u64(u, 1 << 24)
    ref = oracle.Engine(42).raw(1 << 22)
    assert_bits_equal(g.cpu().numpy().view(np.uint64), ref, "raw 2^24")


def test_raw_stream_consecutive_calls(er, oracle):
    u = er.Vmt19937_64(7)
    e = oracle.Engine(7)
    for n in (4, 1248, 100000, 4 * 312 * 3, 8, 1 << 20, 40):
        g = er.raw_u64(u, n).cpu().numpy().view(np.uint64)
        assert_bits_equal(g, e.raw(n // 4), f"raw n={n}")


def test_engine_window_after_calls(er, oracle):
    """Engine state in HBM equals the oracle's after mixed calls."""
    u = er.Vmt19937_64(99)
    e = oracle.Engine(99)
    er.raw_u64(u, 4 * 1000)
    e.raw(1000)
    er.raw_u64(u, 1 << 21)
    e.raw(1 << 19)
    blob = u.save()
    win = np.frombuffer(blob[:4 * 312 * 8], dtype=np.uint64).reshape(4, 312)
    np.testing.assert_array_equal(win, e.window())


def test_save_restore_roundtrip(er):
    u = er.Vmt19937_64(5)
    er.raw_u64(u, 4000)
    blob = u.save()
    a = er.raw_u64(u, 40000).cpu()
    u.restore(blob)
    b = er.raw_u64(u, 40000).cpu()
    assert torch.equal(a, b)


def test_discard_matches_draws(er, oracle):
    u = er.Vmt19937_64(11)
    u.discard(12345)
    e = oracle.Engine(11)
    e.discard(12345)
    assert_bits_equal(er.raw_u64(u, 4096).cpu().numpy().view(np.uint64), e.raw(1024), "discard")


def test_long_discard_in_segments(er, oracle):
    """discard(n) of millions of packets (jump-ahead segments), single and
    multi-stream engines."""
    for streams in (1, 3):
        u = er.Vmt19937_64(13, streams=streams)
        u.discard(3_000_017)
        x = er.raw_u64(u, 4096 * streams).cpu().numpy().view(np.uint64)
        for k in range(streams):
            e = oracle.Engine(13 + 4 * k)
            e.discard(3_000_017)
            assert_bits_equal(x[k * 4096:(k + 1) * 4096], e.raw(1024), f"discard stream {k}")


def test_streams_are_independent_engines(er, oracle):
    """streams=K: slice k comes from Vmt19937_64(seed + 4k)."""
    K, per = 8, 8 * 1000
    u = er.Vmt19937_64(1234, streams=K)
    x = mem(er.uniformReal(K * per, 1, u))
    for k in range(K):
        e = oracle.Engine(1234 + 4 * k)
        ref = oracle.generate(e, oracle.Gen(), "UNIFORM_REAL", per, np.float32)
        assert_bits_equal(x[k * per:(k + 1) * per], ref, f"slice {k}")


# ---------------------------------------------------------------- config 1
def test_config1_uniform_and_normal_1024sq(er, oracle):
    for fn, kind in ((er.uniformReal, "UNIFORM_REAL"), (er.normal, "NORMAL_STD")):
        u = er.Vmt19937_64(42)
        x = mem(fn(1024, 1024, u))
        ref = oracle.generate(oracle.Engine(42), oracle.Gen(), kind, 1 << 20, np.float32)
        assert_bits_equal(x, ref, kind)


# ---------------------------------------------------------------- golden fixtures
def _gpu_has(c):
    # truncated cases take their constants from the C library's erfc / exp /
    # atan / pow of the machine that runs them; tests/test_gpu_trunc.py checks
    # them against the oracle run on the same machine
    return not c["trunc"]


SUPPORTED = [name for name, c in golden_cases.CASES.items() if _gpu_has(c)]


@pytest.mark.parametrize("name", SUPPORTED)
def test_golden_fixture(er, name):
    fx = np.load(os.path.join(ROOT, "tests", "golden", "oracle_fixtures.npz"))
    got = golden_cases.run_gpu(er, golden_cases.CASES[name])
    assert_bits_equal(got, fx[name], name)


# ---------------------------------------------------------------- every direct kind, large (jump path)
KINDS = [
    ("UNIFORM_REAL", 0, 0), ("UNIFORM_REAL2", -2.0, 3.0), ("BALANCED", 0, 0), ("BALANCED2", -3.0, 5.0),
    ("NORMAL_STD", 0, 0), ("NORMAL", 2.0, 3.0), ("LOGNORMAL", 0.0, 1.0), ("EXPONENTIAL", 1.5, 0),
    ("CAUCHY", 0.0, 1.0), ("WEIBULL", 1.5, 1.0), ("EXTREME_VALUE", 0.0, 1.0), ("GAMMA", 1.0, 2.0),
    ("BERNOULLI", 0.3, 0),
]


@pytest.mark.parametrize("kind,a,b", KINDS)
@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
def test_kind_bit_exact_large(er, oracle, kind, a, b, tdt):
    n = 1 << 21  # long enough for jump-ahead segments
    u = er.Vmt19937_64(1234)
    d, keep = er._desc(kind, tdt, a, b)
    o = torch.empty(n, dtype=tdt, device="cuda")
    er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), n, er._stream_ptr()))
    got = mem(o)
    ref = oracle.generate(oracle.Engine(1234), oracle.Gen(), kind, n, npdt(tdt), a, b)
    assert_bits_equal(got, ref, f"{kind} {tdt}")


# ---------------------------------------------------------------- multi-packet units (staged kernel)
STAGED = [("GAMMA", 5.0, 1.0, 0), ("GAMMA", 2.0, 3.0, 0), ("GAMMA", 19.0, 1.0, 0), ("CHI_SQUARED", 4.0, 0.0, 0),
          ("CHI_SQUARED", 2.0, 0.0, 0), ("STUDENT_T", 5.0, 0.0, 0)]


@pytest.mark.parametrize("kind,a,b,t", STAGED)
@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
@pytest.mark.parametrize("n", [1 << 12, 1 << 21])
def test_staged_kinds_bit_exact(er, oracle, kind, a, b, t, tdt, n):
    u = er.Vmt19937_64(77)
    e = oracle.Engine(77)
    for rep in range(2):  # second call continues the stream
        d, keep = er._desc(kind, tdt, a, b)
        o = torch.empty(n, dtype=tdt, device="cuda")
        er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), n, er._stream_ptr()))
        ref = oracle.generate(e, oracle.Gen(), kind, n, npdt(tdt), a, b)
        assert_bits_equal(mem(o), ref, f"{kind}({a},{b}) {tdt} n={n} call {rep}")


@pytest.mark.parametrize("trials,p", [(20, 0.3), (1, 0.5), (24, 0.9), (7, 0.01)])
def test_binomial_small_and_half_cache(er, oracle, trials, p):
    """BinomialGen(trials < 25) draws half packets; the half() cache carries
    across calls and across kinds (PacketRandomEngine.h:325-336)."""
    u = er.Vmt19937_64(5)
    e = oracle.Engine(5)
    seq = [("BINOMIAL", 4), ("BINOMIAL", 12), ("RANDBITS", 4), ("BINOMIAL", 4), ("UNIFORM_REAL", 8),
           ("BINOMIAL", 1 << 20), ("BINOMIAL", 4), ("BALANCED", 4), ("BINOMIAL", 1 << 16)]
    for kind, n in seq:
        tdt = torch.float32 if kind == "UNIFORM_REAL" else (torch.float64 if kind == "BALANCED" else torch.int32)
        a = p if kind == "BINOMIAL" else (-1.0 if kind == "BALANCED" else 0.0)
        b = 1.0 if kind == "BALANCED" else 0.0
        d, keep = er._desc(kind, tdt, a, b, trials if kind == "BINOMIAL" else 0)
        o = torch.empty(n, dtype=tdt, device="cuda")
        er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), n, er._stream_ptr()))
        ref = oracle.generate(e, oracle.Gen(), kind, n, npdt(tdt), a, b, trials)
        assert_bits_equal(mem(o), ref, f"{kind} n={n}")


def test_staged_on_many_streams(er, oracle):
    K, per = 6, 8 * 700
    u = er.Vmt19937_64(1234, streams=K)
    x = mem(er.gamma(K * per, 1, u, 5.0, 1.0))
    for k in range(K):
        ref = oracle.generate(oracle.Engine(1234 + 4 * k), oracle.Gen(), "GAMMA", per, np.float32, 5.0, 1.0)
        assert_bits_equal(x[k * per:(k + 1) * per], ref, f"gamma5 slice {k}")


# ---------------------------------------------------------------- rejection samplers (CompressMask automaton)
REJECT = [("GAMMA", 0.5, 1.0, 0), ("GAMMA", 0.2, 3.0, 0), ("GAMMA", 10.5, 1.0, 0), ("GAMMA", 25.0, 2.0, 0),
          ("GAMMA", 1.7, 1.0, 0), ("CHI_SQUARED", 7.0, 0.0, 0), ("BETA", 0.5, 0.7, 0)]


@pytest.mark.parametrize("kind,a,b,t", REJECT)
@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
def test_rejection_kinds_bit_exact(er, oracle, kind, a, b, t, tdt):
    """Consecutive calls with one generator: the carried lanes (rest) and the
    engine position after the completing trial must match the reference."""
    u = er.Vmt19937_64(31)
    e = oracle.Engine(31)
    g = er._Gen(tdt, a, b, kind=kind)
    og = oracle.Gen()
    P = 8 if tdt == torch.float32 else 4
    for n in (P, 3 * P, 1 << 14, 5 * P, 1 << 16):
        got = mem(g.generate(n, 1, u))
        ref = oracle.generate(e, og, kind, n, npdt(tdt), a, b)
        assert_bits_equal(got, ref, f"{kind}({a},{b}) {tdt} n={n}")
    # the engine continues exactly: a raw draw after the rejection calls
    assert_bits_equal(er.raw_u64(u, 64).cpu().numpy().view(np.uint64), e.raw(16), "engine after rejection")


@pytest.mark.parametrize("kind,a,t", [("POISSON", 100.0, 0), ("POISSON", 12.0, 0), ("BINOMIAL", 0.75, 100),
                                      ("BINOMIAL", 0.3, 1000), ("BINOMIAL", 0.1, 30)])
def test_rejection_int_kinds_bit_exact(er, oracle, kind, a, t):
    u = er.Vmt19937_64(32)
    e = oracle.Engine(32)
    g = er._Gen(torch.int32, a, 0.0, trials=t, kind=kind)
    og = oracle.Gen()
    for n in (4, 12, 1 << 14, 8, 1 << 16):
        got = mem(g.generate(n, 1, u))
        ref = oracle.generate(e, og, kind, n, np.int32, a, 0.0, t)
        assert_bits_equal(got, ref, f"{kind}({a},{t}) n={n}")
    # half-packet cache continues into the next half-packet kind
    d, keep = er._desc("RANDBITS", torch.int32)
    o = torch.empty(8, dtype=torch.int32, device="cuda")
    er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), 8, er._stream_ptr()))
    assert_bits_equal(mem(o), oracle.generate(e, oracle.Gen(), "RANDBITS", 8, np.int32), "randbits after")


# ---------------------------------------------------------------- data-dependent consumption (walk kernel)
@pytest.mark.parametrize("kind,a,t", [("POISSON", 4.0, 0), ("POISSON", 0.3, 0), ("POISSON", 11.9, 0),
                                      ("BINOMIAL", 0.01, 50), ("BINOMIAL", 0.995, 100)])
def test_walk_int_kinds_bit_exact(er, oracle, kind, a, t):
    u = er.Vmt19937_64(41)
    e = oracle.Engine(41)
    g = er._Gen(torch.int32, a, 0.0, trials=t, kind=kind)
    og = oracle.Gen()
    for n in (4, 8, 1 << 14, 12, 1 << 16):
        got = mem(g.generate(n, 1, u))
        ref = oracle.generate(e, og, kind, n, np.int32, a, 0.0, t)
        assert_bits_equal(got, ref, f"{kind}({a},{t}) n={n}")
    d, keep = er._desc("RANDBITS", torch.int32)
    o = torch.empty(8, dtype=torch.int32, device="cuda")
    er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), 8, er._stream_ptr()))
    assert_bits_equal(mem(o), oracle.generate(e, oracle.Gen(), "RANDBITS", 8, np.int32), "randbits after")


@pytest.mark.parametrize("scale", [1.0, 0.5, 3.0])
@pytest.mark.parametrize("kind,a,t", [("POISSON", 4.0, 0), ("POISSON", 11.5, 0), ("BINOMIAL", 0.004, 100),
                                      ("BINOMIAL", 0.996, 200)])
def test_walk_segmented_single_engine(er, oracle, monkeypatch, kind, a, t, scale):
    """Long PoissonGen / BinomialGen (mean < 1) calls on one engine run as
    jump-ahead segments (scan, plan, write).  Odd sizes leave the engine's
    half cache set; a plan scale below 1 makes the last segment run on past
    its plan, above 1 ends the call in an earlier segment."""
    monkeypatch.setenv("GR_WALK_PLAN_SCALE", str(scale))
    u = er.Vmt19937_64(77)
    e = oracle.Engine(77)
    g = er._Gen(torch.int32, a, 0.0, trials=t, kind=kind)
    og = oracle.Gen()
    for n in (4, (1 << 18) + 4, 1 << 20, 12, (1 << 16) + 4, 1 << 21):
        got = mem(g.generate(n, 1, u))
        ref = oracle.generate(e, og, kind, n, np.int32, a, 0.0, t)
        assert_bits_equal(got, ref, f"{kind}({a},{t}) n={n} scale={scale}")
    u.sync()
    assert_bits_equal(er.raw_u64(u, 64).cpu().numpy().view(np.uint64), e.raw(16), "engine after segmented walk")


def test_walk_segmented_three_streams(er, oracle):
    K, per = 3, 4 * 300001
    u = er.Vmt19937_64(88, streams=K)
    x = mem(er.poisson(K * per, 1, u, 3.5))
    for k in range(K):
        ref = oracle.generate(oracle.Engine(88 + 4 * k), oracle.Gen(), "POISSON", per, np.int32, 3.5)
        assert_bits_equal(x[k * per:(k + 1) * per], ref, f"poisson3.5 slice {k}")


@pytest.mark.parametrize("a,b", [(0.5, 2.0), (2.0, 0.5), (1.0, 3.0), (2.5, 4.0), (0.3, 1.0), (22.0, 1.5)])
@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
def test_beta_general_bit_exact(er, oracle, a, b, tdt):
    u = er.Vmt19937_64(43)
    e = oracle.Engine(43)
    g = er.BetaGen(a, b, dtype=tdt)
    og = oracle.Gen()
    P = 8 if tdt == torch.float32 else 4
    for n in (P, 3 * P, 1 << 13, 5 * P, 1 << 15):
        got = mem(g.generate(n, 1, u))
        ref = oracle.generate(e, og, "BETA", n, npdt(tdt), a, b)
        assert_bits_equal(got, ref, f"beta({a},{b}) {tdt} n={n}")
    assert_bits_equal(er.raw_u64(u, 64).cpu().numpy().view(np.uint64), e.raw(16), "engine after beta")


@pytest.mark.parametrize("kind,a,b,t,tdt", [
    ("GAMMA", 0.5, 1.0, 0, torch.float32), ("GAMMA", 3.3, 2.0, 0, torch.float64), ("BETA", 0.4, 0.6, 0, torch.float32),
    ("POISSON", 50.0, 0.0, 0, torch.int32), ("BINOMIAL", 0.4, 0.0, 500, torch.int32),
    ("BINOMIAL", 0.8, 0.0, 60, torch.int32), ("GAMMA", 25.0, 1.0, 0, torch.float32)])
def test_segmented_rejection_large_and_short_plan(er, oracle, kind, a, b, t, tdt, monkeypatch):
    """Long single-engine calls run as jump-ahead segments (count, scan,
    write, gather).  A plan scaled down to 30% of the needed trials makes the
    last segment run on past its end; both must equal the single stream."""
    u = er.Vmt19937_64(2718)
    e = oracle.Engine(2718)
    g = er._Gen(tdt, a, b, trials=t, kind=kind)
    og = oracle.Gen()
    for n, scale in ((1 << 21, None), (24, None), (1 << 19, "0.3"), (1 << 18, None)):
        if scale:
            monkeypatch.setenv("GR_REJECT_PLAN_SCALE", scale)
        else:
            monkeypatch.delenv("GR_REJECT_PLAN_SCALE", raising=False)
        got = mem(g.generate(n, 1, u))
        ref = oracle.generate(e, og, kind, n, npdt(tdt), a, b, t)
        assert_bits_equal(got, ref, f"{kind}({a},{b},{t}) {tdt} n={n} scale={scale}")
    monkeypatch.delenv("GR_REJECT_PLAN_SCALE", raising=False)
    u.sync()
    assert_bits_equal(er.raw_u64(u, 64).cpu().numpy().view(np.uint64), e.raw(16), "engine after segmented calls")


def test_segmented_rejection_few_streams(er, oracle):
    K, per = 3, 8 * 40000
    u = er.Vmt19937_64(55, streams=K)
    x = mem(er.gamma(K * per, 1, u, 0.7, 1.0))
    for k in range(K):
        ref = oracle.generate(oracle.Engine(55 + 4 * k), oracle.Gen(), "GAMMA", per, np.float32, 0.7, 1.0)
        assert_bits_equal(x[k * per:(k + 1) * per], ref, f"gamma0.7 slice {k}")


def test_rejection_on_many_streams(er, oracle):
    K, per = 5, 8 * 512
    u = er.Vmt19937_64(99, streams=K)
    x = mem(er.gamma(K * per, 1, u, 0.5, 1.0))
    for k in range(K):
        ref = oracle.generate(oracle.Engine(99 + 4 * k), oracle.Gen(), "GAMMA", per, np.float32, 0.5, 1.0)
        assert_bits_equal(x[k * per:(k + 1) * per], ref, f"gamma0.5 slice {k}")


# ---------------------------------------------------------------- caches carried between calls
def test_normal_gen_cache_carry(er, oracle):
    """StdNormalGen caches the cos half across generate() calls."""
    for tdt, P in ((torch.float32, 8), (torch.float64, 4)):
        u = er.Vmt19937_64(3)
        g = er.NormalGen(0.5, 2.0, dtype=tdt)
        e = oracle.Engine(3)
        og = oracle.Gen()
        for n in (P, 3 * P, 5 * P, 2 * P, P, 7 * P, 1 << 18):
            got = mem(g.generate(n, 1, u))
            ref = oracle.generate(e, og, "NORMAL", n, npdt(tdt), 0.5, 2.0)
            assert_bits_equal(got, ref, f"normal cache {tdt} n={n}")


def test_half_packet_cache_between_kinds(er, oracle):
    """rng.half() cache survives full-packet draws (PacketRandomEngine.h:325-336)."""
    u = er.Vmt19937_64(8)
    e = oracle.Engine(8)
    seq = [("BALANCED", torch.float64, 4), ("UNIFORM_REAL", torch.float32, 16), ("RANDBITS", torch.int32, 4),
           ("BALANCED", torch.float64, 12), ("RANDBITS", torch.int32, 8), ("BALANCED", torch.float64, 1 << 16),
           ("RANDBITS", torch.int32, 4)]
    for kind, tdt, n in seq:
        d, keep = er._desc(kind, tdt)
        o = torch.empty(n, dtype=tdt, device="cuda")
        er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), n, er._stream_ptr()))
        ref = oracle.generate(e, oracle.Gen(), kind, n, npdt(tdt), *((-1.0, 1.0) if kind == "BALANCED" else (0.0, 0.0)))
        assert_bits_equal(mem(o), ref, f"{kind} n={n}")


@pytest.mark.parametrize("ab", [(0.5, 2.0), (2.0, 1.0), (3.0, 1.5)])
@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
def test_beta_walk_call_ends_everywhere(er, oracle, tdt, ab):
    """Many BetaGen calls of random sizes on one engine: each call ends at a
    different point of the engine blocks it generated (including inside the
    oldest one resident, whose predecessor the kernel recovers by untwisting),
    and the engine continues exactly (checked by the next call and by a final
    raw draw).  (2, 1) has no rejection component (the walk runs ahead of its
    evaluated positions only by its record buffer); (3, 1.5) two tan-proposal
    components."""
    P = 8 if tdt == torch.float32 else 4
    rng = np.random.default_rng(71)
    u = er.Vmt19937_64(33)
    e = oracle.Engine(33)
    g = er.BetaGen(*ab, dtype=tdt)
    og = oracle.Gen()
    for _ in range(60):
        n = int(rng.integers(1, 700)) * P
        ref = oracle.generate(e, og, "BETA", n, npdt(tdt), *ab)
        assert_bits_equal(mem(g.generate(n, 1, u)), ref, f"beta{ab} {tdt} n={n}")
    d, keep = er._desc("RANDBITS", torch.int32)
    o = torch.empty(16, dtype=torch.int32, device="cuda")
    er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), 16, er._stream_ptr()))
    assert_bits_equal(mem(o), oracle.generate(e, oracle.Gen(), "RANDBITS", 16, np.int32), "randbits after")


@pytest.mark.parametrize("m,n", [(1.0, 1.0), (1.0, 1.6), (5.0, 5.0), (1.0, 5.0), (4.0, 2.0), (10.0, 3.0)])
@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
def test_fisher_f_bit_exact(er, oracle, m, n, tdt):
    """FisherFGen = BetaGen(m/2, n/2) (both branches: a, b < 1 rejection with
    its segmented form on one engine, and the two-gamma walk) followed by
    (b/a) x / (1 - x) on every output, including lanes carried between calls."""
    P = 8 if tdt == torch.float32 else 4
    u = er.Vmt19937_64(44)
    e = oracle.Engine(44)
    g = er.FisherFGen(m, n, dtype=tdt)
    og = oracle.Gen()
    for cnt in (P, 3 * P, 1 << 20, 5 * P, 1 << 14):
        ref = oracle.generate(e, og, "FISHER_F", cnt, npdt(tdt), m, n)
        assert_bits_equal(mem(g.generate(cnt, 1, u)), ref, f"fisherF({m},{n}) {tdt} n={cnt}")


@pytest.mark.parametrize("kind,a", [("BERNOULLI", 0.7), ("BERNOULLI", 1.0), ("BERNOULLI", 0.0),
                                    ("GEOMETRIC", 0.25), ("GEOMETRIC", 0.9), ("GEOMETRIC", 0.0),
                                    ("GEOMETRIC", 1.0)])
def test_half_word_int_kinds_bit_exact(er, oracle, kind, a):
    """int32 BernoulliGen / GeometricGen over rng.half() words, large calls
    (jump segments) and odd half-packet counts that leave the half() cache
    full; p = 1 gives 0 on the packet path (signed compare with 2^31), and
    GeometricGen(0) converts NaN / inf lanes to INT_MIN like cvttps2dq."""
    u = er.Vmt19937_64(31)
    e = oracle.Engine(31)
    for n in (4, 12, 1 << 21, 8, 4 + (1 << 20)):
        d, keep = er._desc(kind, torch.int32, a)
        o = torch.empty(n, dtype=torch.int32, device="cuda")
        er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), n, er._stream_ptr()))
        ref = oracle.generate(e, oracle.Gen(), kind, n, np.int32, a)
        assert_bits_equal(mem(o), ref, f"{kind}({a}) n={n}")


UNIFORM_INT_RANGES = [(0, 9), (-5, 5), (1, 6), (0, 2), (0, 7), (7, 7), (-1000, 100000), (0, 65536),
                      (-2 ** 31, 2 ** 31 - 1), (0, 2 ** 31 - 2), (10, 5)]


@pytest.mark.parametrize("lo,hi", UNIFORM_INT_RANGES)
def test_uniform_int_bit_exact(er, oracle, lo, hi):
    """UniformIntGen<int32_t>: bit-slice rejection through CompressMask with
    the carried lanes and the half() cache continuing across calls; power-of-two
    ranges mask; a one-value range draws nothing; min > max follows the
    reference's size_t arithmetic."""
    u = er.Vmt19937_64(17)
    e = oracle.Engine(17)
    g = er.UniformIntGen(lo, hi)
    og = oracle.Gen()
    for n in (4, 8, 12, 1 << 20, 4, (1 << 16) + 4, 8):
        ref = oracle.generate(e, og, "UNIFORM_INT", n, np.int32, lo, hi)
        assert_bits_equal(mem(g.generate(n, 1, u)), ref, f"uniformInt[{lo},{hi}] n={n}")
    # the engine continues exactly where the oracle's does
    d, keep = er._desc("RANDBITS", torch.int32)
    o = torch.empty(12, dtype=torch.int32, device="cuda")
    er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), 12, er._stream_ptr()))
    assert_bits_equal(mem(o), oracle.generate(e, oracle.Gen(), "RANDBITS", 12, np.int32), "randbits after")


@pytest.mark.parametrize("trials,p", [(5, 0.3), (1, 0.5), (3, 0.9), (25, 0.5), (2, 0.05), (19, 0.6), (40, 0.2)])
def test_negative_binomial_bit_exact(er, oracle, trials, p):
    """NegativeBinomialGen<int32_t>: gamma draw (exponential, product or tan
    rejection), then the Poisson loop or tan rejection through the shared
    CompressMask carry; the carry and the half() cache continue across calls."""
    u = er.Vmt19937_64(19)
    e = oracle.Engine(19)
    g = er.NegativeBinomialGen(trials, p)
    og = oracle.Gen()
    for n in (4, 8, 1 << 17, 12, (1 << 14) + 4):
        ref = oracle.generate(e, og, "NEGATIVE_BINOMIAL", n, np.int32, p, trials=trials)
        assert_bits_equal(mem(g.generate(n, 1, u)), ref, f"negbin({trials},{p}) n={n}")
    d, keep = er._desc("RANDBITS", torch.int32)
    o = torch.empty(12, dtype=torch.int32, device="cuda")
    er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), 12, er._stream_ptr()))
    assert_bits_equal(mem(o), oracle.generate(e, oracle.Gen(), "RANDBITS", 12, np.int32), "randbits after")


def test_negative_binomial_many_streams(er, oracle):
    K, per = 9, 4 * 1500
    u = er.Vmt19937_64(29, streams=K)
    x = mem(er.negativeBinomial(K * per, 1, u, 4, 0.35))
    for k in range(K):
        ref = oracle.generate(oracle.Engine(29 + 4 * k), oracle.Gen(), "NEGATIVE_BINOMIAL", per, np.int32, 0.35,
                              trials=4)
        assert_bits_equal(x[k * per:(k + 1) * per], ref, f"negbin slice {k}")


def test_uniform_int_many_streams(er, oracle):
    K, per = 6, 4 * 3000
    u = er.Vmt19937_64(23, streams=K)
    x = mem(er.uniformInt(K * per, 1, u, -3, 20))
    for k in range(K):
        ref = oracle.generate(oracle.Engine(23 + 4 * k), oracle.Gen(), "UNIFORM_INT", per, np.int32, -3, 20)
        assert_bits_equal(x[k * per:(k + 1) * per], ref, f"uniformInt slice {k}")


def test_half_cache_shared_by_int_kinds(er, oracle):
    """RandbitsGen, BernoulliGen<int32_t> and GeometricGen all draw through
    rng.half(): a cached half left by one is used by the next."""
    u = er.Vmt19937_64(12)
    e = oracle.Engine(12)
    seq = [("BERNOULLI", 0.4, 4), ("GEOMETRIC", 0.3, 12), ("RANDBITS", 0.0, 4), ("BERNOULLI", 0.4, 1 << 16 | 4),
           ("GEOMETRIC", 0.3, 4), ("UNIFORM_REAL", 0.0, 8), ("GEOMETRIC", 0.3, 4), ("BERNOULLI", 0.9, 8)]
    for kind, a, n in seq:
        tdt = torch.float32 if kind == "UNIFORM_REAL" else torch.int32
        d, keep = er._desc(kind, tdt, a)
        o = torch.empty(n, dtype=tdt, device="cuda")
        er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), n, er._stream_ptr()))
        ref = oracle.generate(e, oracle.Gen(), kind, n, npdt(tdt), a)
        assert_bits_equal(mem(o), ref, f"{kind} n={n}")


def test_bernoulli_per_element(er, oracle):
    """BernoulliVGen<float> (bernoulli(urng, ArrayXf p)): one probability per
    element, including 0, 1 (which the packet path turns into 0) and tiny
    values; long calls run as jump segments; K streams split the array."""
    rng = np.random.default_rng(5)
    pv = rng.uniform(0, 1, 1 << 20).astype(np.float32)
    pv[:8] = [0.0, 1.0, 1e-9, 0.5, 0.999999, 2 ** -31, 0.25, 0.75]
    for streams in (1, 5):
        u = er.Vmt19937_64(61, streams=streams)
        got = er.bernoulli(u, torch.from_numpy(pv)).cpu().numpy()
        # slices of whole packets, the first (granules mod K) one packet longer
        g, r = divmod(pv.size // 8, streams)
        lo = 0
        for k in range(streams):
            hi = lo + 8 * (g + (1 if k < r else 0))
            ref = oracle.bernoulli_v(oracle.Engine(61 + 4 * k), pv[lo:hi])
            assert_bits_equal(got[lo:hi], ref, f"bernoulliV streams={streams} slice {k}")
            lo = hi
    u = er.Vmt19937_64(62)
    e = oracle.Engine(62)
    for n in (8, 64, 8):  # consecutive calls continue the stream
        q = rng.uniform(0, 1, n).astype(np.float32)
        assert_bits_equal(er.bernoulli(u, torch.from_numpy(q)).cpu().numpy(), oracle.bernoulli_v(e, q), f"n={n}")
    with pytest.raises(er.GrError):
        d, keep = er._desc("BERNOULLI", torch.float64)
        t = torch.zeros(8, dtype=torch.float64, device="cuda")
        er._lib.check(er._L.gr_sample_v(u._h, er.ctypes.byref(d), er._ptr(t), er._ptr(t), 8, er._stream_ptr()))


def test_bernoulli_real_generator_and_invalid_p(er, oracle):
    for tdt in (torch.float32, torch.float64):
        u = er.Vmt19937_64(3)
        e = oracle.Engine(3)
        g = er.BernoulliGen(0.25, dtype=tdt)
        for n in (8, 1 << 20, 16):
            ref = oracle.generate(e, oracle.Gen(), "BERNOULLI", n, npdt(tdt), 0.25)
            assert_bits_equal(mem(g.generate(n, 1, u)), ref, f"bernoulli {tdt} n={n}")
    with pytest.raises(er.GrError):
        er.bernoulli(8, 1, er.Vmt19937_64(1), p=1.5)


@pytest.mark.parametrize("weights", [golden_cases.W16, golden_cases.W5, list(range(1, 41))])
def test_discrete_gen_cache(er, oracle, weights):
    u = er.Vmt19937_64(21)
    g = er.DiscreteGen(weights)
    e = oracle.Engine(21)
    og = oracle.Gen()
    for n in (4, 8, 12, 4, 1 << 16, 4):
        got = mem(g.generate(n, 1, u))
        ref = oracle.generate(e, og, "DISCRETE", n, np.int32, weights=weights)
        assert_bits_equal(got, ref, f"discrete n={n}")


# ---------------------------------------------------------------- errors
def test_size_not_multiple_of_packet_is_rejected(er):
    """A partial last packet goes through the generator's scalar operator();
    kinds whose scalar form is not exact bit arithmetic refuse it (the
    exact ones are in test_gpu_tail.py)."""
    u = er.Vmt19937_64(1)
    with pytest.raises(er.GrError):
        er.normal(5, 3, u)
    with pytest.raises(er.GrError):
        er.gamma(3, 3, u, 0.5, 1.0)


def test_nan_weight_sum_is_rejected(er):
    u = er.Vmt19937_64(1)
    with pytest.raises(er.GrError):
        er.discrete(16, 1, u, [float("nan")] + [1.0] * 20)
