"""GPU checks of the multivariate generators through the C ABI.

MultinomialGen is integer work: bit-exact against the oracle.  MvNormalGen,
WishartGen, InvWishartGen and DirichletGen draw their normal / chi-squared /
gamma streams bit-exactly (the oracle reproduces them); the linear algebra
after the draws is compared with an FP64 evaluation of the reference's
formulas on the same draws, with the tolerances written in each test:
  MvNormal float (3xTF32 tensor-core L Z):  max |X - X64| / (|L| |Z| + |mean|) <= 1e-5
  Wishart float (3xTF32 Bartlett products): max |W - W64| / max |W64|         <= 1e-5
  InvWishart float:                                                           <= 1e-4
  Dirichlet float:                          max relative error                 <= 1e-5
  every double object:                                                        <= 1e-12
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def er(gpulib):
    return gpulib


def rows(t):
    """(dim, samples) column-major result -> numpy (samples, dim)."""
    torch.cuda.synchronize()
    return t.t().contiguous().cpu().numpy()


def spd(d, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((d, d))
    return a @ a.T + d * np.eye(d), rng.standard_normal(d)


NPD = {torch.float32: np.float32, torch.float64: np.float64}


# ------------------------------------------------------------------ Multinomial
@pytest.mark.parametrize("dim,trials,samples", [
    (100, 1000, 64), (5, 17, 37), (20, 18, 40), (20, 5, 33), (64, 100, 48), (3, 4, 9), (16, 1, 8), (100, 2399, 5),
])
def test_multinomial_bit_exact(er, oracle, dim, trials, samples):
    rng = np.random.default_rng(dim + trials)
    w = rng.dirichlet(np.ones(dim))
    g = er.MultinomialGen(trials, w)
    u = er.Vmt19937_64(2024)
    a = rows(g.generate(u, samples))
    b = rows(g.generate(u, samples + 3))  # the DiscreteGen cache carries over
    e, og = oracle.Engine(2024), oracle.Gen()
    np.testing.assert_array_equal(a, oracle.multinomial(e, og, w, trials, samples))
    np.testing.assert_array_equal(b, oracle.multinomial(e, og, w, trials, samples + 3))
    # engine position: the next raw draws agree
    np.testing.assert_array_equal(er.raw_u64(u, 8).cpu().numpy().view(np.uint64), e.raw(2))


@pytest.mark.parametrize("trials,samples", [(1000, 4096), (5, 1 << 17), (18, 1 << 16)])
def test_multinomial_jump_segments(er, oracle, trials, samples):
    """Long single-engine calls run as jump-ahead segments; the first call
    leaves the cache full when trials / 4 is odd, so segments then start in
    the cached state and rebuild the cache from the jumped window."""
    dim = 100
    w = np.random.default_rng(trials).dirichlet(np.ones(dim))
    g = er.MultinomialGen(trials, w)
    u = er.Vmt19937_64(11)
    e, og = oracle.Engine(11), oracle.Gen()
    a0 = rows(g.generate(u, 1))
    np.testing.assert_array_equal(a0, oracle.multinomial(e, og, w, trials, 1))
    a = rows(g.generate(u, samples))
    np.testing.assert_array_equal(a, oracle.multinomial(e, og, w, trials, samples))
    np.testing.assert_array_equal(er.raw_u64(u, 8).cpu().numpy().view(np.uint64), e.raw(2))


def test_multinomial_streams(er, oracle):
    K, samples, dim, trials = 5, 103, 100, 1000
    w = np.random.default_rng(4).dirichlet(np.ones(dim))
    g = er.MultinomialGen(trials, w)
    u = er.Vmt19937_64(77, streams=K)
    a = rows(g.generate(u, samples))
    off = 0
    for k in range(K):
        n = samples // K + (1 if k < samples % K else 0)
        ref = oracle.multinomial(oracle.Engine(77 + 4 * k), oracle.Gen(), w, trials, n)
        np.testing.assert_array_equal(a[off:off + n], ref)
        off += n


def test_multinomial_counts_chi2(er):
    """Distribution check at the headline shape (K=100, trials=1000)."""
    dim, trials, samples = 100, 1000, 1 << 15
    p = np.random.default_rng(8).dirichlet(np.ones(dim))
    g = er.MultinomialGen(trials, p)
    a = rows(g.generate(er.Vmt19937_64(3, streams=64), samples))
    assert (a.sum(axis=1) == trials).all()
    tot = a.sum(axis=0).astype(np.float64)
    exp = p * trials * samples
    chi2 = ((tot - exp) ** 2 / exp).sum()
    from scipy.stats import chi2 as c2
    assert c2.sf(chi2, dim - 1) > 1e-3, chi2


def test_multinomial_errors(er):
    g = er.MultinomialGen(100000, np.ones(10))  # conditional-binomial path: packets of 8 samples
    with pytest.raises(er.GrError, match="INVALID"):
        g.generate(er.Vmt19937_64(1), 12)
    with pytest.raises(er.GrError, match="INVALID"):
        er.MultinomialGen(10, [1.0, -1.0, 2.0])


@pytest.mark.parametrize("dim,trials", [(10, 1000), (2, 500), (1, 200), (5, 100000), (100, 5000), (7, 180)])
def test_multinomial_conditional_path_bit_exact(er, oracle, dim, trials):
    """trials >= max(30 (dim - 1), 100): BinomialVGen<float> row by row
    (Multinomial.h:62-87), single-stream calls in a row (engine state carried)
    and a multi-stream engine (slice k from engine seed + 4k)."""
    w = np.random.default_rng(dim).uniform(0.0, 2.0, dim)
    if dim > 3:
        w[1] = 0.0
    g = er.MultinomialGen(trials, w)
    u = er.Vmt19937_64(77)
    e = oracle.Engine(77)
    for samples in (8, 4096, 24):
        a = rows(g.generate(u, samples))
        ref = oracle.multinomial_cond(e, w, trials, samples)
        np.testing.assert_array_equal(a, ref)
    np.testing.assert_array_equal(er.raw_u64(u, 64).cpu().numpy().view(np.uint64), e.raw(16))
    K, samples = 3, 8 * 1001
    a = rows(g.generate(er.Vmt19937_64(77, streams=K), samples))
    gran, off = samples // 8, 0
    for k in range(K):
        n = 8 * (gran // K + (1 if k < gran % K else 0))
        np.testing.assert_array_equal(a[off:off + n], oracle.multinomial_cond(oracle.Engine(77 + 4 * k), w, trials, n))
        off += n
    if dim > 1:
        assert (a.sum(axis=1) == trials).all()


# ------------------------------------------------------------------ MvNormal
def mvn_case(er, oracle, d, n, tdt, seed=5, lower=False):
    cov, mean = spd(d, seed)
    L64 = oracle.get_lt(cov)
    g = er.MvNormalGen(mean, L64 if lower else cov, lower_triangular=lower, dtype=tdt)
    u = er.Vmt19937_64(1234)
    x = rows(g.generate(u, n)).astype(np.float64)
    e, og = oracle.Engine(1234), oracle.Gen()
    z = oracle.generate(e, og, "NORMAL_STD", d * n, dtype=NPD[tdt]).astype(np.float64).reshape(n, d).T
    x64 = oracle.mvnormal_f64(L64, z, mean).T
    scale = (np.abs(L64) @ np.abs(z)).T + np.abs(mean)[None, :]
    return np.max(np.abs(x - x64) / scale)


@pytest.mark.parametrize("d", [3, 16, 20, 64, 256])
def test_mvnormal_f32_vs_fp64_oracle(er, oracle, d):
    n = 1000 if d < 256 else 512
    err = mvn_case(er, oracle, d, n, torch.float32)
    print(f"MvNormal d={d} float: max error / (|L||Z| + |mean|) = {err:.3g}")
    assert err <= 1e-5


@pytest.mark.parametrize("d,n", [(4, 776), (36, 136), (100, 1002), (132, 258), (200, 257), (256, 300),
                                 (5, 776), (33, 136)])
def test_mvnormal_f32_tensor_memory_shapes(er, oracle, d, n, monkeypatch):
    """The tcgen05 product (dim a multiple of 4, <= 256; forced with the
    GR_MVN_PRODUCT test hook below the default threshold) at shapes that pad
    every dimension: zero-padded N (dim to a multiple of 16) and K (to 32,
    all-zero K steps left out), one and two 128-column passes, the factor
    resident in shared memory (dim <= 160) or streamed per slice (200, 256),
    and sample counts that leave a partial 128-sample tile.  dim 5 and 33
    take the mma.sync form."""
    monkeypatch.setenv("GR_MVN_PRODUCT", "tcgen05")
    err = mvn_case(er, oracle, d, n, torch.float32, seed=d)
    print(f"MvNormal d={d} n={n} float: max error / (|L||Z| + |mean|) = {err:.3g}")
    assert err <= 1e-5


@pytest.mark.parametrize("d", [16, 64, 256])
def test_mvnormal_f32_mma_sync_form(er, oracle, d, monkeypatch):
    """The mma.sync form of the product (the default below dim 20, and for
    dims that are not a multiple of 4), forced at dims that default to tcgen05."""
    monkeypatch.setenv("GR_MVN_PRODUCT", "mma_sync")
    assert mvn_case(er, oracle, d, 520, torch.float32, seed=d + 2) <= 1e-5


@pytest.mark.parametrize("d,n", [(20, 300), (64, 500), (128, 260), (136, 300), (256, 200)])
def test_mvnormal_f32_full_form_products(er, oracle, d, n, monkeypatch):
    """The full-matrix form of the products (every block of L, as for the
    eigen-form factor of a singular covariance), forced on a Cholesky factor
    with the GR_MVN_FULL_FORM test hook so that the FP64 check still holds."""
    monkeypatch.setenv("GR_MVN_FULL_FORM", "1")
    err = mvn_case(er, oracle, d, n, torch.float32, seed=d + 1)
    assert err <= 1e-5


def test_mvnormal_f32_many_tiles_per_cta(er, oracle):
    """More tiles than twice the SM count: every ring (raw slots, A stages,
    both accumulators) wraps many times."""
    d, n = 64, 152 * 128 * 5 + 77
    err = mvn_case(er, oracle, d, n, torch.float32, seed=3)
    assert err <= 1e-5


def test_misaligned_outputs_refused(er):
    """A device output that is not 16-byte aligned is refused on the host
    (GR_ERR_INVALID) before anything is launched."""
    import ctypes
    buf = torch.zeros(4096 + 4, dtype=torch.float32, device="cuda")
    bad = ctypes.c_void_p(buf.data_ptr() + 4)
    u = er.Vmt19937_64(1)
    d, keep = er._desc("NORMAL_STD", torch.float32)
    assert er._L.gr_sample(u._h, ctypes.byref(d), bad, 64, er._stream_ptr()) == 1
    assert "aligned" in er._L.gr_last_error().decode()
    assert er._L.gr_raw_u64(u._h, bad, 64, er._stream_ptr()) == 1
    g = er.MvNormalGen(np.zeros(4), np.eye(4))
    assert er._L.gr_mvnormal_sample(g._h, u._h, bad, 16, er._stream_ptr()) == 1
    torch.cuda.synchronize()
    assert float(buf.abs().sum()) == 0.0  # nothing was written


@pytest.mark.parametrize("d", [3, 16, 64])
def test_mvnormal_f64_vs_fp64_oracle(er, oracle, d):
    err = mvn_case(er, oracle, d, 400, torch.float64)
    assert err <= 1e-12


def test_mvnormal_lower_triangular_form(er, oracle):
    assert mvn_case(er, oracle, 24, 200, torch.float32, lower=True) <= 1e-5


def test_mvnormal_cache_carry_and_streams(er, oracle):
    d = 3  # 3 x 8 normals: one and a half Box-Muller blocks per call
    cov, mean = spd(d, 9)
    L64 = oracle.get_lt(cov)
    g = er.MvNormalGen(mean, cov)
    u = er.Vmt19937_64(5)
    x1 = rows(g.generate(u, 8)).astype(np.float64)
    x2 = rows(g.generate(u, 8)).astype(np.float64)
    e, og = oracle.Engine(5), oracle.Gen()
    for x in (x1, x2):
        z = oracle.generate(e, og, "NORMAL_STD", d * 8).astype(np.float64).reshape(8, d).T
        assert np.max(np.abs(x - oracle.mvnormal_f64(L64, z, mean).T)) < 1e-5 * 10
    # K streams: normals split into K contiguous slices, slice k from engine seed + 4k
    K, n = 3, 64
    gk = er.MvNormalGen(mean, cov)
    xk = rows(gk.generate(er.Vmt19937_64(21, streams=K), n)).astype(np.float64)
    tot = d * n // 8
    zs = []
    for k in range(K):
        cnt = (tot // K + (1 if k < tot % K else 0)) * 8
        zs.append(oracle.generate(oracle.Engine(21 + 4 * k), oracle.Gen(), "NORMAL_STD", cnt))
    z = np.concatenate(zs).astype(np.float64).reshape(n, d).T
    assert np.max(np.abs(xk - oracle.mvnormal_f64(L64, z, mean).T)) < 1e-4


def test_mvnormal_psd_singular_uses_eigen_form(er):
    """Rank-deficient covariance: Cholesky fails, get_lt falls back to
    V sqrt(max(lambda, 0)); samples then stay in the covariance's range."""
    rng = np.random.default_rng(2)
    b = rng.standard_normal((8, 3))
    cov = b @ b.T
    mean = rng.standard_normal(8)
    g = er.MvNormalGen(mean, cov)
    x = rows(g.generate(er.Vmt19937_64(9, streams=16), 1 << 15)).astype(np.float64) - mean
    w, v = np.linalg.eigh(cov)
    null = v[:, w < 1e-9 * w.max()]
    assert null.shape[1] == 5
    assert np.max(np.abs(x @ null)) < 1e-4 * np.sqrt(w.max())
    emp = x.T @ x / x.shape[0]
    assert np.max(np.abs(emp - cov)) < 0.05 * np.max(np.abs(cov))


def test_mvnormal_indefinite_clamps_eigenvalues(er):
    """Indefinite matrix: get_lt's eigen form V sqrt(max(lambda, 0)) gives the
    covariance V max(lambda, 0) V^T."""
    rng = np.random.default_rng(3)
    v, _ = np.linalg.qr(rng.standard_normal((8, 8)))
    lam = np.array([3.0, 2.0, 1.0, 0.5, -0.2, -1.0, 0.0, 0.0])
    cov = (v * lam) @ v.T
    plus = (v * np.maximum(lam, 0)) @ v.T
    g = er.MvNormalGen(np.zeros(8), cov)
    x = rows(g.generate(er.Vmt19937_64(13, streams=16), 1 << 15)).astype(np.float64)
    assert np.max(np.abs(x @ v[:, 4:])) < 1e-4
    emp = x.T @ x / x.shape[0]
    assert np.max(np.abs(emp - plus)) < 0.05 * np.max(np.abs(plus))


def test_mvnormal_moments_headline_dims(er):
    for d in (16, 64):
        cov, mean = spd(d, d)
        g = er.MvNormalGen(mean, cov)
        x = rows(g.generate(er.Vmt19937_64(1, streams=64), 1 << 16)).astype(np.float64)
        sd = np.sqrt(np.diag(cov))
        assert np.max(np.abs(x.mean(0) - mean) / sd) < 0.03
        emp = np.cov(x.T)
        assert np.max(np.abs(emp - cov) / np.outer(sd, sd)) < 0.05


def test_mvnormal_errors(er):
    cov, mean = spd(4, 1)
    with pytest.raises(er.GrError, match="INVALID"):
        er.MvNormalGen(mean, np.full((4, 4), np.nan))
    g = er.MvNormalGen(mean[:3], cov[:3, :3])
    with pytest.raises(er.GrError, match="INVALID"):
        g.generate(er.Vmt19937_64(1), 3)  # 9 values: not a multiple of 8


# ------------------------------------------------------------------ Wishart
def wishart_case(er, oracle, d, df, n, tdt, inverse=False):
    scale, _ = spd(d, 100 + d)
    G = er.InvWishartGen if inverse else er.WishartGen
    g = G(df, scale, dtype=tdt)
    u = er.Vmt19937_64(31)
    w = g.generate(u, n)
    torch.cuda.synchronize()
    W = w.cpu().numpy().astype(np.float64)  # (d, d * n) in the reference's layout
    e = oracle.Engine(31)
    nt = NPD[tdt]
    normals = oracle.generate(e, oracle.Gen(), "NORMAL_STD", n * d * (d - 1) // 2, dtype=nt) if d > 1 else []
    chis = np.stack([oracle.generate(e, oracle.Gen(), "CHI_SQUARED", n, dtype=nt, a=float(df - i))
                     for i in range(d)])
    chol = oracle.get_lt(np.linalg.inv(scale) if inverse else scale)
    W64 = oracle.wishart_f64(chol, normals, chis, d, n, inverse=inverse)
    return np.max(np.abs(W - W64)) / np.max(np.abs(W64))


@pytest.mark.parametrize("d,df,n", [(4, 6, 64), (32, 40, 64), (5, 5, 16), (130, 140, 8)])
def test_wishart_f32_vs_fp64_oracle(er, oracle, d, df, n):
    err = wishart_case(er, oracle, d, df, n, torch.float32)
    print(f"Wishart d={d} float: max |W - W64| / max |W64| = {err:.3g}")
    assert err <= 1e-5


@pytest.mark.parametrize("d,df,n", [(1, 3, 16), (3, 5, 40), (16, 20, 24), (17, 20, 40), (33, 40, 40), (64, 70, 24),
                                    (32, 40, 152 * 4 * 3 + 8)])
def test_wishart_f32_tensor_memory_shapes(er, oracle, d, df, n):
    """The tcgen05 Bartlett products (float, dim <= 64): draws stacked 8 / 4 /
    2 to a 128-row tile for padded dims 16 / 32 / 64, partial last tiles,
    zero-padded rows and columns, and more tiles than SMs."""
    err = wishart_case(er, oracle, d, df, n, torch.float32)
    print(f"Wishart d={d} n={n} float (tcgen05): max |W - W64| / max |W64| = {err:.3g}")
    assert err <= 1e-5


@pytest.mark.parametrize("d,df,n", [(4, 6, 64), (32, 40, 64)])
def test_wishart_f32_mma_sync_form(er, oracle, d, df, n, monkeypatch):
    """The mma.sync products (InvWishart, dims above 64), forced with the
    GR_WISHART_PRODUCT test hook at dims that default to tcgen05."""
    monkeypatch.setenv("GR_WISHART_PRODUCT", "mma_sync")
    assert wishart_case(er, oracle, d, df, n, torch.float32) <= 1e-5


@pytest.mark.parametrize("d,df,n", [(4, 6, 64), (32, 40, 32)])
def test_invwishart_f32_vs_fp64_oracle(er, oracle, d, df, n):
    err = wishart_case(er, oracle, d, df, n, torch.float32, inverse=True)
    print(f"InvWishart d={d} float: relative error {err:.3g}")
    assert err <= 1e-4


@pytest.mark.parametrize("inverse", [False, True])
def test_wishart_f64_vs_fp64_oracle(er, oracle, inverse):
    assert wishart_case(er, oracle, 5, 9, 16, torch.float64, inverse=inverse) <= 1e-12


def test_wishart_mean(er):
    d, df, n = 32, 40, 1 << 12
    scale, _ = spd(d, 3)
    g = er.WishartGen(df, scale)
    w = g.generate(er.Vmt19937_64(8, streams=32), n)
    torch.cuda.synchronize()
    W = w.cpu().numpy().astype(np.float64).reshape(d, n, d)  # [row, draw, col]
    m = W.mean(axis=1)
    sd = np.sqrt(df * (scale ** 2 + np.outer(np.diag(scale), np.diag(scale))) / n)
    assert np.max(np.abs(m - df * scale) / sd) < 6


def test_wishart_errors(er):
    scale, _ = spd(4, 1)
    with pytest.raises(er.GrError, match="INVALID"):
        er.WishartGen(3, scale)  # df must exceed dim - 1
    g = er.WishartGen(6, scale)
    with pytest.raises(er.GrError, match="INVALID"):
        g.generate(er.Vmt19937_64(1), 5)


# ------------------------------------------------------------------ Dirichlet
@pytest.mark.parametrize("tdt,tol", [(torch.float32, 1e-5), (torch.float64, 1e-12)])
def test_dirichlet_vs_fp64_oracle(er, oracle, tdt, tol):
    K, n = 64, 1024
    alpha = np.random.default_rng(6).uniform(0.1, 2.0, K)
    g = er.DirichletGen(alpha, dtype=tdt)
    u = er.Vmt19937_64(17)
    x = rows(g.generate(u, n)).astype(np.float64)
    x2 = rows(g.generate(u, n)).astype(np.float64)  # gamma carries (compress_append) persist
    e = oracle.Engine(17)
    gens = [oracle.Gen() for _ in range(K)]
    for xx in (x, x2):
        rws = np.stack([oracle.generate(e, gens[i], "GAMMA", n, dtype=NPD[tdt], a=alpha[i], b=1.0) for i in range(K)])
        ref = oracle.dirichlet_f64(rws).T
        floor = 1e-30 if tdt == torch.float32 else 1e-300  # gamma draws may underflow
        assert np.all(np.abs(xx - ref) <= tol * ref + floor)


def test_dirichlet_moments(er):
    K, n = 64, 1 << 16
    alpha = np.random.default_rng(12).uniform(0.1, 2.0, K)
    x = rows(er.DirichletGen(alpha).generate(er.Vmt19937_64(4, streams=64), n)).astype(np.float64)
    assert np.allclose(x.sum(axis=1), 1.0, atol=1e-5)
    a0 = alpha.sum()
    m = alpha / a0
    sd = np.sqrt(m * (1 - m) / (a0 + 1) / n)
    assert np.max(np.abs(x.mean(axis=0) - m) / sd) < 6


# ------------------------------------------------------------------ TruncMvNormal
TMVN_CASES = {
    # test_mv.cpp:224-256 / :392-434 (truncMvNormal, truncMvNormalFromLt)
    "basic": ([1, 2, 3], [[1.0, 0.3, 0.1], [0.3, 1.2, 0.2], [0.1, 0.2, 0.8]], [-1, 0, 1], [5, 5, 6], 0),
    # :258-303 (truncMvNormalTight, 50 sweeps)
    "tight": ([0, 0, 0], [[1.0, 0.5, 0.0], [0.5, 1.0, 0.5], [0.0, 0.5, 1.0]], [0.5] * 3, [1.5] * 3, 50),
    # :305-353 (truncMvNormalOneSided)
    "one_sided": ([0, 0, 0], [[1.0, 0.3, 0.0], [0.3, 1.0, 0.3], [0.0, 0.3, 1.0]], [0] * 3, [100] * 3, 0),
}


def _highdim_case():
    """test_mv.cpp:355-390 (truncMvNormalHighDim)."""
    c = np.zeros((9, 9))
    c[0, 1], c[2, 7], c[3, 1] = 0.5, 0.5, 0.7
    c[np.diag_indices(9)] = [1, 1.2, 1.4, 1.6, 1.8, 1.6, 1.4, 1.2, 1]
    return ([-1, 0, 1, 2, 3, 2, 1, 0, -1], c @ c.T, [-4, -3, -2, -1, 0, -1, -2, -3, -4], [4, 5, 6, 7, 8, 7, 6, 5, 4], 0)


TMVN_CASES["high_dim"] = _highdim_case()


@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
@pytest.mark.parametrize("name", sorted(TMVN_CASES))
def test_truncmvn_matches_oracle(er, oracle, name, tdt):
    """Gibbs chains against the oracle on the same draws: every value within
    the support, and within the rounding of erfc and of the dot products
    (CUDA's erfc here, the C library's in the oracle: |diff| <= 1e-3 (1+|x|)
    float, 1e-7 (1+|x|) double, median far below); consecutive calls carry the
    engine; a multi-stream engine gives engine seed + 4k to slice k."""
    mean, cov, lo, hi, burn = TMVN_CASES[name]
    npt = NPD[tdt]
    tol = 1e-3 if tdt == torch.float32 else 1e-7
    g = er.TruncMvNormalGen(mean, cov, er.support(lo, hi), burn, dtype=tdt)
    u = er.Vmt19937_64(42)
    e = oracle.Engine(42)
    for samples in (4096, 40):
        x = rows(g.generate(u, samples)).astype(np.float64)
        ref = oracle.truncmvn(e, mean, cov, lo, hi, samples, burn, npt).astype(np.float64)
        err = np.abs(x - ref) / (1 + np.abs(ref))
        assert err.max() <= tol and np.median(err) <= tol / 100, (err.max(), np.median(err))
        slack = 1e-5 if tdt == torch.float32 else 1e-12
        assert (x >= np.array(lo) - slack).all() and (x <= np.array(hi) + slack).all()
    if name == "tight":
        assert np.unique(x[:, 0]).size > 1
    K, samples = 3, 1001
    x = rows(g.generate(er.Vmt19937_64(7, streams=K), samples)).astype(np.float64)
    off = 0
    for k in range(K):
        n = samples // K + (1 if k < samples % K else 0)
        ref = oracle.truncmvn(oracle.Engine(7 + 4 * k), mean, cov, lo, hi, n, burn, npt).astype(np.float64)
        assert (np.abs(x[off:off + n] - ref) / (1 + np.abs(ref))).max() <= tol
        off += n


def test_truncmvn_from_lt_and_errors(er, oracle):
    """makeTruncMvNormalGenFromLt gives the covariance constructor's chains
    (test_mv.cpp:392-434); bad supports and dimensions are refused."""
    mean, cov, lo, hi, _ = TMVN_CASES["basic"]
    lt = np.linalg.cholesky(np.asarray(cov))
    a = rows(er.makeTruncMvNormalGenFromLt(mean, lt, er.support(lo, hi)).generate(er.Vmt19937_64(42), 2048))
    b = rows(er.makeTruncMvNormalGen(mean, cov, er.support(lo, hi)).generate(er.Vmt19937_64(42), 2048))
    assert np.abs(a - b).max() <= 1e-3 * (1 + np.abs(b).max())
    with pytest.raises(er.GrError):
        er.TruncMvNormalGen(mean, cov, er.support([0, 0, 5], [1, 1, 1]))
    with pytest.raises(er.GrError):
        er.TruncMvNormalGen(np.zeros(65), np.eye(65), er.support(-np.ones(65), np.ones(65)))


def test_multinomial_conditional_many_streams(er, oracle):
    """More streams than 7 CTAs per SM take the kernel form that tempers each
    word as it reads it (20 KB of shared memory per stream): every slice of
    a 1500-stream engine, and the engines' next draws, against the oracle."""
    w = np.random.default_rng(3).uniform(0.1, 2.0, 6)
    g = er.MultinomialGen(500, w)
    K = 1500
    u = er.Vmt19937_64(91, streams=K)
    samples = 8 * (2 * K + 7)
    a = rows(g.generate(u, samples))
    raw = er.raw_u64(u, 4 * K).cpu().numpy().view(np.uint64)
    gran, off = samples // 8, 0
    for k in range(K):
        n = 8 * (gran // K + (1 if k < gran % K else 0))
        e = oracle.Engine(91 + 4 * k)
        np.testing.assert_array_equal(a[off:off + n], oracle.multinomial_cond(e, w, 500, n), err_msg=f"stream {k}")
        np.testing.assert_array_equal(raw[4 * k:4 * k + 4], e.raw(1), err_msg=f"stream {k} after")
        off += n
