"""Sizes that are not a whole number of packets.

Eigen assigns a random expression with its linear vectorised loop: whole
packets first, then the generator's scalar operator() for the remaining
n % P elements, one engine draw each (pfirst of the packet engine's packet,
or one draw of a scalar engine).  For uniformReal, balanced (with and
without a range), bernoulli and randBits that scalar form is exact bit
arithmetic, so these tails are bit-exact with the oracle.  The shapes are
the reference's own tests' (test/test.cpp:114-160: 8x8, 3x3, 5x5, 5x3, 1x3
in a row on one engine), on Vmt19937_64 and on P8_mt19937_64, the
reference tests' engine.  Other kinds refuse a partial last packet: their
scalar forms go through the C library's log / exp / sqrt, which a GPU cannot
reproduce bit for bit.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

SHAPES = [(8, 8), (3, 3), (5, 5), (5, 3), (1, 3), (7, 1), (2, 9)]
NP = {torch.float32: np.float32, torch.float64: np.float64, torch.int32: np.int32}
CASES = [("BALANCED", torch.float32, -1.0, 1.0), ("BALANCED", torch.float64, -1.0, 1.0),
         ("BALANCED2", torch.float32, 0.5, 2.0), ("BALANCED2", torch.float64, 0.5, 2.0),
         ("UNIFORM_REAL", torch.float32, 0.0, 1.0), ("UNIFORM_REAL", torch.float64, 0.0, 1.0),
         ("UNIFORM_REAL2", torch.float32, 0.5, 2.0), ("UNIFORM_REAL2", torch.float64, 0.5, 2.0),
         ("BERNOULLI", torch.float32, 0.3, 0.0), ("BERNOULLI", torch.float64, 0.7, 0.0),
         ("BERNOULLI", torch.int32, 0.4, 0.0), ("RANDBITS", torch.int32, 0.0, 0.0)]


def bits(a):
    return a.view(np.uint64 if a.itemsize == 8 else np.uint32)


def draw(er, urng, kind, tdt, a, b, n):
    d, keep = er._desc(kind, tdt, a, b)
    o = torch.empty(n, dtype=tdt, device="cuda")
    fn = er._L.gr_sengine_sample if isinstance(urng, er._ScalarEngine) else er._L.gr_sample
    er._lib.check(fn(urng._h, ctypes.byref(d), er._ptr(o), n, er._stream_ptr()))
    torch.cuda.synchronize()
    return o.cpu().numpy()


@pytest.mark.parametrize("kind,tdt,a,b", CASES)
@pytest.mark.parametrize("engine", ["vmt", "p8"])
def test_reference_test_shapes_bit_exact(gpulib, oracle, engine, kind, tdt, a, b):
    er = gpulib
    if engine == "vmt":
        u, e = er.Vmt19937_64(42), oracle.Engine(42)
    else:
        u, e = er.P8_mt19937_64(42), oracle.ScalarEngine("p8", 42)
    g = oracle.Gen()
    for r, c in SHAPES:
        n = r * c
        got = draw(er, u, kind, tdt, a, b, n)
        if engine == "vmt":
            ref = oracle.generate(e, g, kind, n, NP[tdt], a, b)
        else:
            ref = e.generate(g, kind, n, NP[tdt], a, b)
        assert np.array_equal(bits(got), bits(ref)), f"{engine} {kind} {tdt} {r}x{c}"
    if engine == "vmt":  # the engine continues exactly after the scalar draws
        np.testing.assert_array_equal(er.raw_u64(u, 16).cpu().numpy().view(np.uint64), e.raw(4))


def test_tail_comes_from_the_last_stream(gpulib, oracle):
    """streams = 3: the whole packets split into three slices, the partial
    last packet extends the last slice, drawn by its engine."""
    er = gpulib
    u = er.Vmt19937_64(7, streams=3)
    n = 3 * 16 + 5
    got = draw(er, u, "UNIFORM_REAL", torch.float32, 0.0, 1.0, n)
    for k in range(3):
        per = 16 + (5 if k == 2 else 0)
        ref = oracle.generate(oracle.Engine(7 + 4 * k), oracle.Gen(), "UNIFORM_REAL", per, np.float32)
        assert np.array_equal(bits(got[16 * k:16 * k + per]), bits(ref)), f"stream {k}"


def test_long_call_with_tail(gpulib, oracle):
    """A long call (jump-ahead segments for the whole packets) then its tail."""
    er = gpulib
    u, e = er.Vmt19937_64(9), oracle.Engine(9)
    n = (1 << 21) + 3
    got = draw(er, u, "BALANCED", torch.float64, -1.0, 1.0, n)
    ref = oracle.generate(e, oracle.Gen(), "BALANCED", n, np.float64)
    assert np.array_equal(bits(got), bits(ref))


def test_kinds_without_an_exact_tail_refuse(gpulib):
    er = gpulib
    u = er.Vmt19937_64(1)
    d, keep = er._desc("NORMAL_STD", torch.float32)
    o = torch.empty(9, dtype=torch.float32, device="cuda")
    assert er._L.gr_sample(u._h, ctypes.byref(d), er._ptr(o), 9, er._stream_ptr()) == 1  # GR_ERR_INVALID
    assert "partial last packet" in er._L.gr_last_error().decode()
