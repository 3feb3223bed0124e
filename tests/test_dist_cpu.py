"""The oracle's univariate samplers checked in distribution, independently of
the restatement they come from.

Every bit-exact GPU test compares the CUDA path with oracle/, a restatement
of the reference's packet code.  A misreading of the reference would be
shared by both sides; these checks catch any that changes the law of the
samples.  One Vmt19937_64(1234) carried through the benchmark sweep, 2^21
samples per call, each call against its exact FP64 law:

* KS (continuous) or chi-squared (integer) p-value above 0.01;
* the sample mean and variance within 5 standard errors of the exact moments.

The GPU test (test_gpu_dist.py) repeats this on the CUDA output at the full
4096 x 4096 size of the benchmark's own engine configuration.
"""
import numpy as np
import pytest

pytest.importorskip("scipy")
import dist_checks as dc  # noqa: E402

N = 1 << 21


@pytest.fixture(scope="module")
def sweep_samples(oracle):
    e = oracle.Engine(1234)
    out = {}
    for (name, kind, t, a, b, tr, w) in dc.sweep():
        out[name] = oracle.generate(e, oracle.Gen(), kind, N, dc.NP_DTYPE[t], a, b, tr, w)
    return out


@pytest.mark.parametrize("item", dc.sweep(), ids=[it[0] for it in dc.sweep()])
def test_oracle_sweep_in_distribution(sweep_samples, item):
    name, w = item[0], item[6]
    r = dc.check(sweep_samples[name], name, w)
    assert r["p"] > 0.01, f"{name}: {r['test']} p = {r['p']:.4g} (stat {r['stat']:.4g})"
    if "z_mean" in r:
        assert abs(r["z_mean"]) < 5, f"{name}: mean {r['mean']} vs {r['mean_exact']} (z {r['z_mean']:.2f})"
        assert abs(r["z_var"]) < 5, f"{name}: variance {r['var']} vs {r['var_exact']} (z {r['z_var']:.2f})"


def test_checks_detect_a_planted_error(oracle):
    """The statistics have power: a gamma(5) sampler whose output is scaled
    by 1.004, or a poisson(4) sampler that moves 0.5% of its mass from 3 to
    4, fails at this sample size.  The mistake is planted in the oracle's
    output on the CPU."""
    e = oracle.Engine(77)
    x = oracle.generate(e, oracle.Gen(), "GAMMA", N, np.float32, 5.0, 1.0)
    assert dc.check(x, "gamma5/f32")["p"] > 0.01
    assert dc.check(x * np.float32(1.004), "gamma5/f32")["p"] < 1e-6
    k = oracle.generate(e, oracle.Gen(), "POISSON", N, np.int32, 4.0)
    assert dc.check(k, "poisson4/i32")["p"] > 0.01
    k2 = k.copy()
    idx = np.nonzero(k2 == 3)[0]
    k2[idx[: int(0.005 * N)]] = 4
    assert dc.check(k2, "poisson4/i32")["p"] < 1e-6


def test_emd_matches_reference_method():
    """dist_checks.emd restates accuracy.cpp's calc_emd_with_cdf: for the
    exact quantiles of U(0, 1) at (i + 0.5) / n the distance is the
    discretisation error alone, about 1 / (4 n)."""
    n = 32768
    x = (np.arange(n) + 0.5) / n
    d = dc.emd(x, "uniformReal/f32")
    assert abs(d - 0.25 / n) < 0.1 / n
