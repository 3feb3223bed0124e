"""Distribution-level checks of the univariate sweep against exact FP64 laws.

Shared by the CPU test (the oracle's samplers) and the GPU test (the CUDA
path at the benchmark's own configuration).  Each sweep call names its exact
distribution (scipy.stats, evaluated in FP64); the checks are:

* one-sample Kolmogorov-Smirnov against the exact CDF (continuous kinds);
* chi-squared against the exact PMF, tail cells merged until every expected
  count is at least 20 (integer kinds);
* standardised errors of the sample mean and variance against the exact
  moments (z-scores from the exact second and fourth central moments);
* the Earth Mover's Distance of 50 chunks of 32768 samples, computed as the
  reference's accuracy benchmark computes it (benchmark/accuracy.cpp:25-81,
  size 32768, step = 8 * size, 50 repeats), for the kinds the reference's
  README tabulates (README.md:146-158).

The sweep is EigenRand's benchmark sweep at 4096 x 4096 per call: the same
(name, kind, dtype, a, b, trials, weights) rows the benchmark draws.
"""
import math

import numpy as np

W16 = [0.5488135, 0.71518937, 0.60276338, 0.54488318, 0.4236548, 0.64589411, 0.43758721, 0.891773,
       0.96366276, 0.38344152, 0.79172504, 0.52889492, 0.56804456, 0.92559664, 0.07103606, 0.0871293]

_REAL = [
    ("uniformReal", "UNIFORM_REAL", 0.0, 0.0),
    ("balanced", "BALANCED", 0.0, 0.0),
    ("exponential", "EXPONENTIAL", 1.0, 0.0),
    ("normal", "NORMAL_STD", 0.0, 0.0),
    ("lognormal", "LOGNORMAL", 0.0, 1.0),
    ("cauchy", "CAUCHY", 0.0, 1.0),
    ("weibull", "WEIBULL", 1.5, 1.0),
    ("gamma0.5", "GAMMA", 0.5, 1.0),
    ("gamma1", "GAMMA", 1.0, 1.0),
    ("gamma5", "GAMMA", 5.0, 1.0),
    ("beta", "BETA", 0.5, 2.0),
]
_INT = [
    ("poisson4", "POISSON", 4.0, 0.0, 0, None),
    ("poisson100", "POISSON", 100.0, 0.0, 0, None),
    ("binomial20", "BINOMIAL", 0.3, 0.0, 20, None),
    ("discrete16", "DISCRETE", 0.0, 0.0, 0, W16),
]


def sweep():
    """(name, kind, dtype tag, a, b, trials, weights) of the 26 sweep calls."""
    items = []
    for name, kind, a, b in _REAL:
        items.append((name + "/f32", kind, "f32", a, b, 0, None))
        items.append((name + "/f64", kind, "f64", a, b, 0, None))
    for name, kind, a, b, t, w in _INT:
        items.append((name + "/i32", kind, "i32", a, b, t, w))
    return items


NP_DTYPE = {"f32": np.float32, "f64": np.float64, "i32": np.int32}


def law(name):
    """The exact distribution of a sweep call (a frozen scipy.stats law)."""
    from scipy import stats
    base = name.split("/")[0]
    return {
        "uniformReal": stats.uniform(0.0, 1.0),
        "balanced": stats.uniform(-1.0, 2.0),
        "exponential": stats.expon(),
        "normal": stats.norm(),
        "lognormal": stats.lognorm(1.0),
        "cauchy": stats.cauchy(),
        "weibull": stats.weibull_min(1.5),
        "gamma0.5": stats.gamma(0.5),
        "gamma1": stats.gamma(1.0),
        "gamma5": stats.gamma(5.0),
        "beta": stats.beta(0.5, 2.0),
        "poisson4": stats.poisson(4.0),
        "poisson100": stats.poisson(100.0),
        "binomial20": stats.binom(20, 0.3),
        "discrete16": None,
    }[base]


def discrete_pmf(weights):
    w = np.asarray(weights, np.float64)
    return w / w.sum()


def ks_test(x, dist):
    """One-sample KS statistic and p-value against an exact continuous CDF.
    The statistic is exact for the sample; the p-value uses the asymptotic
    Kolmogorov distribution (n is in the millions)."""
    from scipy import stats
    xs = np.sort(np.asarray(x, np.float64))
    n = xs.size
    cdf = dist.cdf(xs)
    i = np.arange(1, n + 1, dtype=np.float64)
    d = max(float(np.max(i / n - cdf)), float(np.max(cdf - (i - 1) / n)))
    p = float(stats.kstwobign.sf(d * math.sqrt(n)))
    return d, p


def chi2_test(x, pmf_values, support_lo=0, min_expected=20.0):
    """Chi-squared goodness of fit of integer samples against pmf_values
    (pmf_values[k] = P(X = support_lo + k)); the mass outside the listed
    support goes to the two tail cells; adjacent cells are merged until each
    expected count reaches min_expected."""
    from scipy import stats
    x = np.asarray(x, np.int64)
    n = x.size
    K = len(pmf_values)
    obs = np.bincount(np.clip(x - support_lo, 0, K - 1), minlength=K).astype(np.float64)
    exp_p = np.asarray(pmf_values, np.float64).copy()
    # the tails beyond the listed support fold into the end cells
    rest = 1.0 - exp_p.sum()
    if rest > 0:
        exp_p[-1] += rest
    exp_c = exp_p * n
    # merge from both ends towards the middle until every cell is large enough
    cells_o, cells_e = [], []
    acc_o = acc_e = 0.0
    for o, e in zip(obs, exp_c):
        acc_o += o
        acc_e += e
        if acc_e >= min_expected:
            cells_o.append(acc_o)
            cells_e.append(acc_e)
            acc_o = acc_e = 0.0
    if acc_e > 0:
        cells_o[-1] += acc_o
        cells_e[-1] += acc_e
    co, ce = np.array(cells_o), np.array(cells_e)
    chi2 = float(np.sum((co - ce) ** 2 / ce))
    dof = len(co) - 1
    return chi2, dof, float(stats.chi2.sf(chi2, dof))


def pmf_table(name, weights=None):
    """(pmf values, lowest support point) covering all but ~1e-15 of the mass."""
    if name.startswith("discrete16"):
        return discrete_pmf(weights), 0
    d = law(name)
    lo, hi = int(d.ppf(1e-15)), int(d.ppf(1 - 1e-15)) + 1
    k = np.arange(lo, hi + 1)
    return d.pmf(k), lo


def exact_moments(name, weights=None):
    """Exact mean, variance and fourth central moment (None for Cauchy)."""
    base = name.split("/")[0]
    if base == "cauchy":
        return None
    if base == "discrete16":
        p = discrete_pmf(weights)
        k = np.arange(len(p), dtype=np.float64)
        m = float(np.sum(p * k))
        return m, float(np.sum(p * (k - m) ** 2)), float(np.sum(p * (k - m) ** 4))
    d = law(name)
    m, v = float(d.mean()), float(d.var())
    # fourth central moment from the raw moments
    m1, m2, m3, m4 = (float(d.moment(j)) for j in (1, 2, 3, 4))
    mu4 = m4 - 4 * m1 * m3 + 6 * m1 * m1 * m2 - 3 * m1 ** 4
    return m, v, mu4


def moment_errors(x, name, weights=None):
    """Relative errors and z-scores of the sample mean and variance.  The
    sums run in FP64 (pairwise, numpy)."""
    ex = exact_moments(name, weights)
    if ex is None:
        return None
    m, v, mu4 = ex
    xd = np.asarray(x, np.float64)
    n = xd.size
    sm = float(xd.mean())
    sv = float(xd.var())
    z_mean = (sm - m) / math.sqrt(v / n)
    z_var = (sv - v) / math.sqrt(max(mu4 - v * v, 1e-300) / n)
    return {"mean": sm, "mean_exact": m, "mean_rel_err": (sm - m) / (abs(m) if m else 1.0), "z_mean": z_mean,
            "var": sv, "var_exact": v, "var_rel_err": (sv - v) / v, "z_var": z_var}


# ---- the reference's accuracy benchmark (Earth Mover's Distance) ----
# README.md:146-158: mean (stdev) of the EMD over 50 seeds, 32768 samples
# each, for the EigenRand column; the sweep calls that the table covers.
README_EMD = {
    "balanced": (0.0034, 0.0015),
    "exponential": (0.0072, 0.0022),
    "gamma1": (0.0065, 0.0023),
    "gamma5": (0.0170, 0.0051),
    "lognormal": (0.0067, 0.0022),
    "normal": (0.0073, 0.0020),
    "uniformReal": (0.0017, 0.0007),
}


def _emd_cdf_range(name):
    """The CDF and integration range of accuracy.cpp for a sweep call
    (normal_cdf -8..8, lognormal_cdf 0..4, exp_cdf 0..32, ur_cdf 0..1,
    balanced_cdf -1..1); gamma uses its pdf form, integrated the same way."""
    from scipy import stats
    base = name.split("/")[0]
    return {
        "uniformReal": (lambda x: np.clip(x, 0, 1), 0.0, 1.0, "cdf"),
        "balanced": (lambda x: (x + 1) / 2, -1.0, 1.0, "cdf"),
        "exponential": (lambda x: 1 - np.exp(-x), 0.0, 32.0, "cdf"),
        "normal": (stats.norm.cdf, -8.0, 8.0, "cdf"),
        "lognormal": (lambda x: stats.norm.cdf(np.log(np.maximum(x, 1e-300))), 0.0, 4.0, "cdf"),
        "gamma1": (lambda x: stats.gamma.pdf(x, 1.0), 0.0, 16.0, "pdf"),
        "gamma5": (lambda x: stats.gamma.pdf(x, 5.0), 0.0, 16.0, "pdf"),
    }[base]


def emd(sample, name, step=None):
    """accuracy.cpp's calc_emd_with_cdf / calc_emd_with_pdf: the grid
    x_i = lb + (rb - lb) i / step, the sample's empirical CDF counted as
    #{a <= x_i} / n, the pdf form accumulated as a left Riemann sum and
    normalised; sum |F(x_i) - F_n(x_i)| * (rb - lb) / step."""
    fn, lb, rb, form = _emd_cdf_range(name)
    a = np.sort(np.asarray(sample, np.float64))
    n = a.size
    step = step or 8 * n
    x = lb + (rb - lb) * np.arange(step, dtype=np.float64) / step
    if form == "cdf":
        F = fn(x)
    else:
        pdf = fn(x)
        F = np.concatenate(([0.0], np.cumsum(pdf)[:-1]))
        F = F / (F[-1] + pdf[-1])
    Fn = np.searchsorted(a, x, side="right") / n
    return float(np.sum(np.abs(F - Fn)) * (rb - lb) / step)


def emd_over_chunks(x, name, chunks=50, size=32768):
    """Mean and stdev of the EMD over `chunks` disjoint runs of `size`
    consecutive samples (the reference: 50 seeds of 32768 samples)."""
    x = np.asarray(x)
    vals = [emd(x[i * size:(i + 1) * size], name) for i in range(chunks)]
    return float(np.mean(vals)), float(np.std(vals))


def emd_floor(name):
    """The reference's EMD for a sweep call, if its README lists one: a run of
    50 chunks must have a mean within 4 standard errors above it."""
    base = name.split("/")[0]
    if base not in README_EMD:
        return None
    m, s = README_EMD[base]
    return m + 4 * s / math.sqrt(50)


def check(x, name, weights=None):
    """Every applicable statistic of one call's samples, as a dict."""
    out = {"n": int(np.asarray(x).size)}
    if name.endswith("/i32"):
        pmf, lo = pmf_table(name, weights)
        chi2, dof, p = chi2_test(x, pmf, lo)
        out.update({"test": "chi2", "stat": chi2, "dof": dof, "p": p})
    else:
        d, p = ks_test(x, law(name))
        out.update({"test": "ks", "stat": d, "p": p})
    me = moment_errors(x, name, weights)
    if me:
        out.update(me)
    return out
