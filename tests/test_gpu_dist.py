"""The benchmark's own configuration, on the GPU: bit-exact stream slices and
distribution checks of every call of the univariate sweep.

The sweep is drawn exactly as the benchmark draws it: one
Vmt19937_64(1234, streams=608) engine carried through the 26 calls, a fresh
generator object per call, 4096 x 4096 per call.  Stream k of the engine is
an independent Vmt19937_64(1234 + 4k) that fills slice k of every call.

* Bit-exact: slices 0, 1, 303 and 607 of every call against the oracle
  running the same carried sequence on Vmt19937_64(1234 + 4k).
* In distribution, on all 2^24 samples of a call (tolerances as in
  test_dist_cpu.py): KS / chi-squared p-value above 0.01 against the exact
  FP64 law, mean and variance within 5 standard errors, and for the kinds the
  reference's README tabulates, the reference's Earth Mover's Distance method
  (50 chunks of 32768) within 4 standard errors of the reference's figure.
* Against the reference's CPU samples: a two-sample KS (chi-squared
  homogeneity for integer kinds) of the GPU's 2^24 samples against 2^21
  samples of the oracle's single-engine Vmt19937_64(1234) sweep, p > 0.01.
* The single-engine form, Vmt19937_64(1234) carried through the sweep at
  2^22 per call, bit-exact against the oracle (every call runs as jump-ahead
  segments or the segmented rejection kernels at this size).

Set GR_DIST_REPORT=<path> to write the per-call statistics as JSON.
"""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytest.importorskip("scipy")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import dist_checks as dc  # noqa: E402

ROWS = COLS = 4096
N = ROWS * COLS
STREAMS = 608
SLICES = (0, 1, 303, 607)
TDT = {"f32": torch.float32, "f64": torch.float64, "i32": torch.int32}


def slice_of(n, gran, k):
    """Output range of stream k in a call of n samples (granule gran)."""
    per, rem = divmod(n // gran, STREAMS)
    g0 = k * per + min(k, rem)
    return g0 * gran, (per + (1 if k < rem else 0)) * gran


def granule(t):
    return 8 if t == "f32" else 4


def linear(t):
    """Eigen's linear (column-major) order of a (rows, cols) output."""
    return t.t().contiguous().reshape(-1).cpu().numpy()


@pytest.fixture(scope="module")
def er(gpulib):
    return gpulib


@pytest.fixture(scope="module")
def oracle_slices(oracle):
    """The oracle's carried sweep for the checked streams: {k: [call outputs]}."""
    out = {}
    for k in SLICES:
        e = oracle.Engine(1234 + 4 * k)
        outs = []
        for (name, kind, t, a, b, tr, w) in dc.sweep():
            outs.append(oracle.generate(e, oracle.Gen(), kind, slice_of(N, granule(t), k)[1], dc.NP_DTYPE[t],
                                        a, b, tr, w))
        out[k] = outs
    return out


@pytest.fixture(scope="module")
def oracle_single_engine(oracle):
    """2^21 samples per call of the oracle's Vmt19937_64(1234) carried sweep."""
    e = oracle.Engine(1234)
    return [oracle.generate(e, oracle.Gen(), kind, 1 << 21, dc.NP_DTYPE[t], a, b, tr, w)
            for (name, kind, t, a, b, tr, w) in dc.sweep()]


def two_sample_p(x, y, integer):
    from scipy import stats
    if not integer:
        return float(stats.ks_2samp(np.asarray(x, np.float64), np.asarray(y, np.float64), method="asymp").pvalue)
    lo = int(min(x.min(), y.min()))
    hi = int(max(x.max(), y.max()))
    c1 = np.bincount(x - lo, minlength=hi - lo + 1)
    c2 = np.bincount(y - lo, minlength=hi - lo + 1)
    keep = (c1 + c2) >= 40
    tab = np.array([np.append(c1[keep], c1[~keep].sum()), np.append(c2[keep], c2[~keep].sum())])
    tab = tab[:, tab.sum(0) > 0]
    return float(stats.chi2_contingency(tab)[1])


def test_bench_configuration_sweep(er, oracle_slices, oracle_single_engine):
    urng = er.Vmt19937_64(1234, streams=STREAMS)
    report = {}
    failures = []
    for i, (name, kind, t, a, b, tr, w) in enumerate(dc.sweep()):
        g = er._Gen(TDT[t], a, b, tr, w, kind=kind)
        x = linear(g.generate(ROWS, COLS, urng))
        torch.cuda.synchronize()
        # bit-exact stream slices
        for k in SLICES:
            lo, cnt = slice_of(N, granule(t), k)
            ref = oracle_slices[k][i]
            got = x[lo:lo + cnt]
            bits = np.uint64 if got.itemsize == 8 else np.uint32
            bad = np.count_nonzero(got.view(bits) != ref.view(bits))
            if bad:
                failures.append(f"{name}: stream {k}: {bad} of {cnt} samples differ")
        # distribution
        r = dc.check(x, name, w)
        if name.split("/")[0] in dc.README_EMD:
            r["emd_mean"], r["emd_std"] = dc.emd_over_chunks(x, name)
            r["emd_reference_bound"] = dc.emd_floor(name)
            if r["emd_mean"] > r["emd_reference_bound"]:
                failures.append(f"{name}: EMD {r['emd_mean']:.5f} above {r['emd_reference_bound']:.5f}")
        r["two_sample_p"] = two_sample_p(x, oracle_single_engine[i], t == "i32")
        report[name] = r
        if r["p"] <= 0.01:
            failures.append(f"{name}: {r['test']} p = {r['p']:.4g}")
        if r["two_sample_p"] <= 0.01:
            failures.append(f"{name}: two-sample p = {r['two_sample_p']:.4g}")
        if "z_mean" in r and (abs(r["z_mean"]) >= 5 or abs(r["z_var"]) >= 5):
            failures.append(f"{name}: moment z-scores {r['z_mean']:.2f}, {r['z_var']:.2f}")
        del x
    path = os.environ.get("GR_DIST_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(report, f, indent=1)
    for name, r in report.items():
        print(f"{name:18s} {r['test']:5s} p={r['p']:.4f} two-sample p={r['two_sample_p']:.4f} "
              f"z_mean={r.get('z_mean', float('nan')):+.2f} z_var={r.get('z_var', float('nan')):+.2f}")
    assert not failures, "\n".join(failures)


def test_single_engine_sweep_bit_exact(er, oracle):
    """Vmt19937_64(1234), one engine carried through the 26 calls, 2^22 per
    call (2048 x 2048), bit-exact with the oracle's single reference stream."""
    n = 1 << 22
    urng = er.Vmt19937_64(1234)
    e = oracle.Engine(1234)
    for (name, kind, t, a, b, tr, w) in dc.sweep():
        g = er._Gen(TDT[t], a, b, tr, w, kind=kind)
        got = linear(g.generate(2048, 2048, urng))
        ref = oracle.generate(e, oracle.Gen(), kind, n, dc.NP_DTYPE[t], a, b, tr, w)
        bits = np.uint64 if got.itemsize == 8 else np.uint32
        bad = np.count_nonzero(got.view(bits) != ref.view(bits))
        assert bad == 0, f"{name}: {bad} of {n} samples differ"
    # the engine continues exactly after the sweep
    raw = er.raw_u64(urng, 64).cpu().numpy().view(np.uint64)
    np.testing.assert_array_equal(raw, e.raw(16))
