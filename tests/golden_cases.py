"""Fixed small cases shared by the golden-fixture generator and the tests.

Each case draws n samples from a fresh engine seeded `seed` (the reference's
own test seeds and the configuration seeds: 42, 1234)."""
import numpy as np

W16 = [0.5488135, 0.71518937, 0.60276338, 0.54488318, 0.4236548, 0.64589411, 0.43758721, 0.891773,
       0.96366276, 0.38344152, 0.79172504, 0.52889492, 0.56804456, 0.92559664, 0.07103606, 0.0871293]
W5 = [1, 2, 3, 4, 5]

CASES = {}


def _add(name, kind, dtype, n, a=0.0, b=0.0, trials=0, weights=None, seed=1234, trunc=None):
    CASES[name] = dict(kind=kind, dtype=dtype, n=n, a=a, b=b, trials=trials, weights=weights, seed=seed,
                       trunc=trunc)


for dt, tag, n in ((np.float32, "f32", 256), (np.float64, "f64", 128)):
    _add(f"uniformReal_{tag}", "UNIFORM_REAL", dt, n)
    _add(f"uniformReal2_{tag}", "UNIFORM_REAL2", dt, n, -2.0, 3.0)
    _add(f"balanced_{tag}", "BALANCED", dt, n)
    _add(f"balanced2_{tag}", "BALANCED2", dt, n, -3.0, 5.0)
    _add(f"stdnormal_{tag}", "NORMAL_STD", dt, n)
    _add(f"normal23_{tag}", "NORMAL", dt, n, 2.0, 3.0)
    _add(f"lognormal_{tag}", "LOGNORMAL", dt, n, 0.0, 1.0)
    _add(f"exponential_{tag}", "EXPONENTIAL", dt, n, 1.0)
    _add(f"cauchy_{tag}", "CAUCHY", dt, n, 0.0, 1.0)
    _add(f"weibull_{tag}", "WEIBULL", dt, n, 1.5, 1.0)
    _add(f"extremeValue_{tag}", "EXTREME_VALUE", dt, n, 0.0, 1.0)
    _add(f"gamma1_{tag}", "GAMMA", dt, n, 1.0, 1.0)
    _add(f"gamma5_{tag}", "GAMMA", dt, n, 5.0, 1.0)
    _add(f"gamma05_{tag}", "GAMMA", dt, n, 0.5, 1.0)
    _add(f"beta_{tag}", "BETA", dt, n, 0.5, 2.0)
    _add(f"fisherF11_{tag}", "FISHER_F", dt, n, 1.0, 1.0)
    _add(f"fisherF55_{tag}", "FISHER_F", dt, n, 5.0, 5.0)
_add("raw_42", "RAW", np.uint64, 256, seed=42)
_add("binomial20", "BINOMIAL", np.int32, 256, 0.3, trials=20)
_add("poisson4", "POISSON", np.int32, 256, 4.0)
_add("discrete16", "DISCRETE", np.int32, 256, weights=W16)
_add("discrete5", "DISCRETE", np.int32, 256, weights=W5)
_add("randbits", "RANDBITS", np.int32, 256)
_add("bernoulli_f32", "BERNOULLI", np.float32, 256, 0.3)
_add("bernoulli_f64", "BERNOULLI", np.float64, 128, 0.3)
_add("bernoulli_i32", "BERNOULLI", np.int32, 256, 0.7)
_add("geometric", "GEOMETRIC", np.int32, 256, 0.25)
_add("uniformInt_0_9", "UNIFORM_INT", np.int32, 256, 0, 9)
_add("uniformInt_m5_5", "UNIFORM_INT", np.int32, 256, -5, 5)
_add("uniformInt_0_7", "UNIFORM_INT", np.int32, 256, 0, 7)
_add("uniformInt_big", "UNIFORM_INT", np.int32, 256, -1000, 100000)
_add("negbin_5_03", "NEGATIVE_BINOMIAL", np.int32, 256, 0.3, trials=5)
_add("negbin_1_05", "NEGATIVE_BINOMIAL", np.int32, 256, 0.5, trials=1)
_add("negbin_25_05", "NEGATIVE_BINOMIAL", np.int32, 256, 0.5, trials=25)
# TruncGen<Base>{base, support(lower, upper)} (Truncated.h), seed 42 as in test.cpp:1094-1404
for dt, tag, n in ((np.float32, "f32", 256), (np.float64, "f64", 128)):
    _add(f"truncNormal_{tag}", "NORMAL", dt, n, 0.0, 1.0, seed=42, trunc=(-1.0, 1.0))
    _add(f"truncExponential_{tag}", "EXPONENTIAL", dt, n, 1.0, seed=42, trunc=(0.5, 3.0))
    _add(f"truncCauchy_{tag}", "CAUCHY", dt, n, 0.0, 1.0, seed=42, trunc=(-2.0, 2.0))
    _add(f"truncWeibull_{tag}", "WEIBULL", dt, n, 2.0, 1.0, seed=42, trunc=(0.3, 1.5))
    _add(f"truncGamma_{tag}", "GAMMA", dt, n, 2.0, 1.0, seed=42, trunc=(0.5, 5.0))


def run_oracle(oracle, c):
    e = oracle.Engine(c["seed"])
    if c["kind"] == "RAW":
        return e.raw(c["n"] // 4)
    g = oracle.Gen()
    if c["trunc"]:
        return oracle.truncated(e, g, c["kind"], c["n"], c["trunc"][0], c["trunc"][1], c["dtype"], c["a"], c["b"])
    return oracle.generate(e, g, c["kind"], c["n"], c["dtype"], c["a"], c["b"], c["trials"], c["weights"])


def run_gpu(er, c):
    import torch
    u = er.Vmt19937_64(c["seed"])
    if c["kind"] == "RAW":
        return er.raw_u64(u, c["n"]).cpu().numpy().view(np.uint64)
    tdt = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32}[c["dtype"]]
    d, keep = er._desc(c["kind"], tdt, c["a"], c["b"], c["trials"], c["weights"])
    o = torch.empty(c["n"], dtype=tdt, device="cuda")
    if c["trunc"]:
        er._lib.check(er._L.gr_sample_truncated(u._h, er.ctypes.byref(d), c["trunc"][0], c["trunc"][1], er._ptr(o),
                                                c["n"], er._stream_ptr()))
        torch.cuda.synchronize()
        return o.cpu().numpy()
    er._lib.check(er._L.gr_sample(u._h, er.ctypes.byref(d), er._ptr(o), c["n"], er._stream_ptr()))
    torch.cuda.synchronize()
    return o.cpu().numpy()
