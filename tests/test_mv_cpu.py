"""CPU checks for the multivariate generators: the oracle's multinomial
against a second, independent route (the pinned DiscreteGen oracle and the
kernel's word-layout model), and the FP64 assembly restatements."""
import numpy as np
import pytest

import mn_model


@pytest.mark.parametrize("dim", [5, 20])
@pytest.mark.parametrize("trials", [1, 3, 4, 5, 7, 16, 17, 18, 19, 20, 36, 100, 1000])
def test_multinomial_layout_model_matches_oracle(oracle, dim, trials):
    """Two consecutive generate calls (the DiscreteGen cache carries over)."""
    rng = np.random.default_rng(dim * 1000 + trials)
    w = rng.uniform(0.0, 1.0, dim)
    w[1] = 0.0  # a category that can never be drawn
    samples = 7
    e = oracle.Engine(99)
    g = oracle.Gen()
    first = oracle.multinomial(e, g, w, trials, samples)
    second = oracle.multinomial(e, g, w, trials, samples)
    nxt = e.raw(1)
    table = oracle.discrete_table(w)
    ref = oracle.Engine(99)
    words = ref.raw(4096).view(np.uint32)
    m1, cf, cats, used1 = mn_model.counts(words, trials, dim, samples, 0, [0, 0, 0, 0], table)
    m2, _, _, used2 = mn_model.counts(words[used1:], trials, dim, samples, cf, cats, table)
    np.testing.assert_array_equal(first, m1)
    np.testing.assert_array_equal(second, m2)
    assert (first.sum(axis=1) == trials).all() and (first[:, 1] == 0).all()
    # the engine advanced by exactly the modelled packets
    used = used1 + used2
    assert used % 8 == 0
    np.testing.assert_array_equal(nxt.view(np.uint32), words[used:used + 8])


def test_multinomial_oracle_equals_discrete_histogram(oracle):
    """trials a multiple of 16: the counts are histograms of consecutive
    DiscreteGen packet draws (the pinned discrete oracle)."""
    rng = np.random.default_rng(5)
    w = rng.uniform(0.0, 1.0, 100)
    e1, g1 = oracle.Engine(7), oracle.Gen()
    m = oracle.multinomial(e1, g1, w, 64, 9)
    e2, g2 = oracle.Engine(7), oracle.Gen()
    d = oracle.generate(e2, g2, "DISCRETE", 64 * 9, weights=w).reshape(9, 64)
    for s in range(9):
        np.testing.assert_array_equal(m[s], np.bincount(d[s], minlength=100))


def test_get_lt_restatement():
    from pyoracle import get_lt
    rng = np.random.default_rng(1)
    a = rng.standard_normal((6, 6))
    cov = a @ a.T + 6 * np.eye(6)
    L = get_lt(cov)
    assert np.allclose(np.triu(L, 1), 0) and np.allclose(L @ L.T, cov)
    b = rng.standard_normal((6, 2))
    psd = b @ b.T  # rank 2: Cholesky fails, eigen form
    L2 = get_lt(psd)
    assert np.allclose(L2 @ L2.T, psd, atol=1e-12)


def test_bartlett_layout():
    from pyoracle import bartlett
    d, n = 4, 2
    normals = np.arange(n * d * (d - 1) // 2, dtype=np.float64) + 1
    chis = np.full((d, n), 4.0)
    A = bartlett(normals, chis, d, n)
    # draw 0: column 0 gets normals 1,2,3 (rows 1..3), column 1 gets 4,5, column 2 gets 6
    assert A[0, 1, 0] == 1 and A[0, 3, 0] == 3 and A[0, 2, 1] == 4 and A[0, 3, 2] == 6
    assert A[1, 1, 0] == 7 and np.all(np.diag(A[0]) == 2) and A[0, 0, 1] == 0


def test_multinomial_conditional_oracle_moments(oracle):
    """The conditional-binomial restatement: every sample sums to trials, and
    the category totals fit the multinomial (chi-squared); a single category
    gives 0, as the reference's last-row assignment overwrites row 0."""
    import numpy as np
    from scipy.stats import chi2
    w = np.random.default_rng(4).uniform(0.1, 2.0, 12)
    trials, samples = 1000, 8 * 2000
    m = oracle.multinomial_cond(oracle.Engine(9), w, trials, samples)
    assert (m.sum(axis=1) == trials).all() and m.min() >= 0
    p = w / w.sum()
    exp = p * trials * samples
    stat = ((m.sum(axis=0) - exp) ** 2 / exp).sum()
    assert chi2.sf(stat, len(w) - 1) > 1e-3, stat
    assert (oracle.multinomial_cond(oracle.Engine(9), [2.0], 300, 16) == 0).all()
    v = np.random.default_rng(2).uniform(size=13)
    s = oracle.eigen_sum_avx(v)
    assert abs(s - v.sum()) < 1e-14


def test_truncmvn_oracle_bounds_and_symmetry(oracle):
    """TruncMvNormalGen restatement: every chain inside the support, and the
    one-sided case's symmetry E[X0] = E[X2] (test_mv.cpp:305-333); the mean
    lies above the marginal truncated-normal mean there."""
    import numpy as np
    mean, lo, hi = [0, 0, 0], [0, 0, 0], [100, 100, 100]
    cov = [[1.0, 0.3, 0.0], [0.3, 1.0, 0.3], [0.0, 0.3, 1.0]]
    x = oracle.truncmvn(oracle.Engine(54321), mean, cov, lo, hi, 50000, burn_in=30, dtype=np.float64)
    assert (x >= 0).all() and (x <= 100).all()
    m = x.mean(axis=0)
    assert abs(m[0] - m[2]) < 0.02, m
    assert (m > np.sqrt(2 / np.pi) - 0.01).all(), m


def test_truncmvn_host_validation(gpulib):
    """Refused before any device work: inverted supports, dim above 64,
    negative burn-in."""
    import numpy as np
    er = gpulib
    with pytest.raises(er.GrError):
        er.TruncMvNormalGen([0, 0], np.eye(2), er.support([1, 0], [0, 1]))
    with pytest.raises(er.GrError):
        er.TruncMvNormalGen(np.zeros(65), np.eye(65), er.support(-np.ones(65), np.ones(65)))
    with pytest.raises(er.GrError):
        er.TruncMvNormalGen([0, 0], np.eye(2), er.support([0, 0], [1, 1]), burn_in=-1)
