"""GPU parity of the per-element forms (*VGen: parameter arrays of the
output's shape) against the CPU oracle, bit-exact, through the C ABI."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def er(gpulib):
    return gpulib


def assert_bits_equal(a, b, msg=""):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    ua = a.view(np.uint64 if a.itemsize == 8 else np.uint32)
    ub = b.view(np.uint64 if b.itemsize == 8 else np.uint32)
    bad = np.nonzero(ua != ub)[0]
    assert bad.size == 0, f"{msg}: {bad.size} mismatches, first at {bad[:5]}: {a[bad[:5]]} vs {b[bad[:5]]}"


def eigen_mem(t):
    """Eigen linear order of a (rows, cols) tensor."""
    torch.cuda.synchronize()
    if t.dim() == 2:
        t = t.t()
    return t.contiguous().reshape(-1).cpu().numpy()


# kind, python free function, parameter generators (a, b) as functions of (rng, n)
def _pos(lo, hi):
    return lambda r, n: r.uniform(lo, hi, n)


VKINDS = [
    ("UNIFORM_REAL2", "uniformReal", _pos(-3, 0), _pos(0.5, 4)),
    ("BALANCED2", "balanced", _pos(-3, 0), _pos(0.5, 4)),
    ("NORMAL", "normal", _pos(-2, 2), _pos(0.1, 3)),
    ("LOGNORMAL", "lognormal", _pos(-1, 1), _pos(0.1, 1)),
    ("EXPONENTIAL", "exponential", _pos(0.2, 5), None),
    ("STUDENT_T", "studentT", _pos(0.5, 20), None),
    ("WEIBULL", "weibull", _pos(0.5, 4), _pos(0.5, 3)),
    ("EXTREME_VALUE", "extremeValue", _pos(-2, 2), _pos(0.2, 3)),
    ("CAUCHY", "cauchy", _pos(-2, 2), _pos(0.2, 3)),
]


@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
@pytest.mark.parametrize("kind,fn,ga,gb", VKINDS, ids=[v[0] for v in VKINDS])
def test_vgen_free_function_bit_exact(er, oracle, kind, fn, ga, gb, tdt):
    """kind(urng, a, b): both operands arrays, one array and one scalar, a 2-D
    (column-major) call, and a long call split into jump-ahead segments."""
    npt = np.float32 if tdt == torch.float32 else np.float64
    r = np.random.default_rng(3)
    u = er.Vmt19937_64(42)
    e = oracle.Engine(42)
    f = getattr(er, fn)
    for n in (64, 1 << 20, 8):
        a = ga(r, n).astype(npt)
        b = gb(r, n).astype(npt) if gb else None
        got = f(u, torch.from_numpy(a), torch.from_numpy(b)) if gb else f(u, torch.from_numpy(a))
        ref = oracle.generate_v(e, oracle.Gen(), kind, a, b, npt)
        assert_bits_equal(eigen_mem(got), ref, f"{kind} {tdt} n={n}")
    if gb:
        a = ga(r, 4096).astype(npt)
        got = f(u, torch.from_numpy(a), 1.5)
        ref = oracle.generate_v(e, oracle.Gen(), kind, a, 1.5, npt)
        assert_bits_equal(eigen_mem(got), ref, f"{kind} scalar b")
        b = gb(r, 4096).astype(npt)
        got = f(u, 0.25, torch.from_numpy(b))
        ref = oracle.generate_v(e, oracle.Gen(), kind, 0.25, b, npt)
        assert_bits_equal(eigen_mem(got), ref, f"{kind} scalar a")
    A = ga(r, 32 * 48).astype(npt).reshape(32, 48)
    B = gb(r, 32 * 48).astype(npt).reshape(32, 48) if gb else None
    tA = torch.from_numpy(A)
    got = f(u, tA, torch.from_numpy(B)) if gb else f(u, tA)
    assert tuple(got.shape) == (32, 48)
    ref = oracle.generate_v(e, oracle.Gen(), kind, A.T.reshape(-1), B.T.reshape(-1) if gb else None, npt)
    assert_bits_equal(eigen_mem(got), ref, f"{kind} 2-D")


@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
def test_vgen_objects_keep_their_cache(er, oracle, tdt):
    """NormalVGen / LognormalVGen objects carry the StdNormalGen half-pair
    between calls (odd packet counts), like the reference's generate()."""
    npt = np.float32 if tdt == torch.float32 else np.float64
    P = 8 if tdt == torch.float32 else 4
    r = np.random.default_rng(5)
    for cls, kind in ((er.NormalVGen, "NORMAL"), (er.LognormalVGen, "LOGNORMAL")):
        u = er.Vmt19937_64(9)
        e = oracle.Engine(9)
        g = cls(dtype=tdt)
        og = oracle.Gen()
        for n in (P, 3 * P, (1 << 19) + P, 5 * P):
            a = r.uniform(-1, 1, n).astype(npt)
            b = r.uniform(0.2, 1, n).astype(npt)
            got = g.generate(u, torch.from_numpy(a), torch.from_numpy(b))
            ref = oracle.generate_v(e, og, kind, a, b, npt)
            assert_bits_equal(eigen_mem(got), ref, f"{kind} object {tdt} n={n}")
    g = er.ExponentialVGen(dtype=tdt)
    u = er.Vmt19937_64(9)
    a = r.uniform(0.5, 2, 4096).astype(npt)
    ref = oracle.generate_v(oracle.Engine(9), oracle.Gen(), "EXPONENTIAL", a, None, npt)
    assert_bits_equal(eigen_mem(g.generate(u, torch.from_numpy(a))), ref, "ExponentialVGen")


def test_vgen_matches_scalar_generator_and_streams(er, oracle):
    """Constant parameter arrays give the scalar generator's values; slices of
    a multi-stream engine come from engines seed + 4k."""
    u1, u2 = er.Vmt19937_64(77), er.Vmt19937_64(77)
    x = er.cauchy(1024, 1, u1, 0.5, 2.0)
    y = er.cauchy(u2, torch.full((1024,), 0.5), torch.full((1024,), 2.0))
    assert_bits_equal(eigen_mem(x), eigen_mem(y), "cauchy scalar vs per-element")
    K, per = 4, 8 * 1000
    u = er.Vmt19937_64(1234, streams=K)
    r = np.random.default_rng(1)
    a = r.uniform(-1, 1, K * per).astype(np.float32)
    b = r.uniform(0.5, 2, K * per).astype(np.float32)
    got = eigen_mem(er.normal(u, torch.from_numpy(a), torch.from_numpy(b)))
    for k in range(K):
        sl = slice(k * per, (k + 1) * per)
        ref = oracle.generate_v(oracle.Engine(1234 + 4 * k), oracle.Gen(), "NORMAL", a[sl], b[sl], np.float32)
        assert_bits_equal(got[sl], ref, f"slice {k}")
    with pytest.raises(er.GrError):
        er._vform("GAMMA", er.Vmt19937_64(1), torch.ones(8), torch.ones(8))
    with pytest.raises(er.GrError):
        er.normal(er.Vmt19937_64(1), torch.ones(12), torch.ones(12))


def _binom_params(r, n):
    tr = r.choice(np.array([0, 1, 3, 20, 50, 100, 1000, 40000], np.int32), n)
    p = r.choice(np.array([0.0, 0.01, 0.2, 0.5, 0.75, 0.99, 1.0], np.float32), n)
    p = np.where(r.random(n) < 0.5, p, r.random(n).astype(np.float32))
    return tr.astype(np.int32), p.astype(np.float32)


def test_binomial_v_bit_exact(er, oracle):
    """binomial(urng, trials, p) -> BinomialVGen<int32_t>: both operands
    arrays, one scalar, a 2-D (column-major) call, and calls that continue
    the same engine (the half-packet cache and the window carried between
    calls, and into and out of the uniform-parameter BinomialGen)."""
    r = np.random.default_rng(17)
    u = er.Vmt19937_64(2024)
    e = oracle.Engine(2024)
    for n in (4, 64, 1 << 18, 12):
        tr, p = _binom_params(r, n)
        got = er.binomial(u, torch.from_numpy(tr), torch.from_numpy(p))
        assert got.dtype == torch.int32
        assert_bits_equal(eigen_mem(got), oracle.binomial_v(e, tr, p), f"binomialV n={n}")
    tr, _ = _binom_params(r, 4096)
    assert_bits_equal(eigen_mem(er.binomial(u, torch.from_numpy(tr), 0.5)), oracle.binomial_v(e, tr, 0.5),
                      "scalar p")
    _, p = _binom_params(r, 4096)
    assert_bits_equal(eigen_mem(er.binomial(u, 50, torch.from_numpy(p))), oracle.binomial_v(e, 50, p), "scalar trials")
    got = er.binomial(8, 6, u, 10, 0.3)
    ref = oracle.generate(e, oracle.Gen(), "BINOMIAL", 48, np.int32, 0.3, 0.0, trials=10)
    assert_bits_equal(eigen_mem(got), ref, "BinomialGen between per-element calls")
    T = np.linspace(5, 50, 10).astype(np.int32).repeat(100).reshape(10, 100)
    P = np.tile(np.linspace(0.1, 1.0, 10).astype(np.float32)[:, None], (1, 100))
    got = er.binomial(u, torch.from_numpy(T), torch.from_numpy(P))
    assert tuple(got.shape) == (10, 100)
    ref = oracle.binomial_v(e, T.T.reshape(-1), P.T.reshape(-1))
    assert_bits_equal(eigen_mem(got), ref, "2-D")


def test_binomial_v_streams_and_errors(er, oracle):
    """Slices of a multi-stream engine come from engines seed + 4k; constant
    operands give the batched (VoP) binomial's values; sizes not a multiple
    of 4 and mismatched shapes are rejected."""
    K, per = 6, 4 * 333
    u = er.Vmt19937_64(99, streams=K)
    r = np.random.default_rng(4)
    tr, p = _binom_params(r, K * per)
    got = eigen_mem(er.binomial(u, torch.from_numpy(tr), torch.from_numpy(p)))
    for k in range(K):
        sl = slice(k * per, (k + 1) * per)
        assert_bits_equal(got[sl], oracle.binomial_v(oracle.Engine(99 + 4 * k), tr[sl], p[sl]), f"slice {k}")
    u1 = er.Vmt19937_64(321)
    got = er.binomial(u1, torch.full((1000,), 25, dtype=torch.int32), 0.4)
    assert_bits_equal(eigen_mem(got), oracle.vop_set(321, "BINOMIAL", 1000, 0.4, 1.0, 25), "VoP constant")
    with pytest.raises(er.GrError):
        er.binomial(er.Vmt19937_64(1), torch.ones(10, dtype=torch.int32), 0.5)
    with pytest.raises(ValueError):
        er.binomial(er.Vmt19937_64(1), torch.ones(8, dtype=torch.int32), torch.ones(12))


def test_binomial_v_many_streams(er, oracle):
    """More streams than 7 CTAs per SM take the kernel form that tempers each
    half packet as it reads it: every slice of a 1500-stream engine, the
    engines' half caches and windows (next draws), against the oracle."""
    K, per = 1500, 4 * 7
    u = er.Vmt19937_64(55, streams=K)
    r = np.random.default_rng(12)
    tr, p = _binom_params(r, K * per)
    got = eigen_mem(er.binomial(u, torch.from_numpy(tr), torch.from_numpy(p)))
    nxt = eigen_mem(er.binomial(u, 30, torch.full((4 * K,), 0.4)))
    for k in range(K):
        e = oracle.Engine(55 + 4 * k)
        sl = slice(k * per, (k + 1) * per)
        assert_bits_equal(got[sl], oracle.binomial_v(e, tr[sl], p[sl]), f"stream {k}")
        assert_bits_equal(nxt[4 * k:4 * k + 4], oracle.binomial_v(e, 30, np.full(4, 0.4, np.float32)),
                          f"stream {k} next")
