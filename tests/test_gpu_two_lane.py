"""The 2-lane Vmt19937_64 (SSE / NEON profile, Pmt19937_64<Packet4i>,
EigenRand/PacketRandomEngine.h:585-588) against the CPU oracle, bit for bit.

Lane l is std::mt19937_64(seed + l) for l < 2; a packet holds two 64-bit
lanes; a Packet4f takes its four 32-bit words, a Packet2d its two lanes.
This is the stream EigenRand draws when it is built for the GPU machine's own
host (NEON).  Served: the raw stream and the kinds whose packetOp transforms
each word or lane on its own; everything else refuses with
GR_ERR_UNSUPPORTED.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

NP = {torch.float32: np.float32, torch.float64: np.float64}
KINDS = [("UNIFORM_REAL", 0.0, 1.0), ("UNIFORM_REAL2", -2.0, 3.0), ("EXPONENTIAL", 1.5, 0.0), ("CAUCHY", 0.5, 2.0),
         ("WEIBULL", 1.5, 2.0), ("EXTREME_VALUE", 1.0, 2.0), ("GAMMA", 1.0, 3.0)]
F32_ONLY = [("BALANCED", -1.0, 1.0), ("BALANCED2", 0.5, 2.0), ("BERNOULLI", 0.3, 0.0)]


def bits(a):
    return a.view(np.uint64 if a.itemsize == 8 else np.uint32)


def draw(er, u, kind, tdt, a, b, n):
    d, keep = er._desc(kind, tdt, a, b)
    o = torch.empty(n, dtype=tdt, device="cuda")
    er._lib.check(er._L.gr_sample(u._h, ctypes.byref(d), er._ptr(o), n, er._stream_ptr()))
    torch.cuda.synchronize()
    return o.cpu().numpy()


def test_raw_stream(gpulib, oracle):
    er = gpulib
    u = er.Vmt19937_64(42, lanes=2)
    e = oracle.Engine(42, lanes=2)
    for n in (2, 624, 1 << 20, 6, 1 << 22):  # the long calls run as jump-ahead segments
        got = er.raw_u64(u, n).cpu().numpy().view(np.uint64)
        assert np.array_equal(got, e.raw(n // 2)), f"n={n}"


@pytest.mark.parametrize("kind,a,b", KINDS + F32_ONLY)
@pytest.mark.parametrize("tdt", [torch.float32, torch.float64])
def test_kinds_consecutive_calls(gpulib, oracle, kind, a, b, tdt):
    er = gpulib
    if tdt == torch.float64 and (kind, a, b) in F32_ONLY:
        pytest.skip("float only on the 2-lane profile")
    u = er.Vmt19937_64(7, lanes=2)
    e = oracle.Engine(7, lanes=2)
    P = 4 if tdt == torch.float32 else 2
    for n in (P, 3 * P, 1 << 16, 5 * P, (1 << 21) + P):
        got = draw(er, u, kind, tdt, a, b, n)
        ref = oracle.generate(e, oracle.Gen(), kind, n, NP[tdt], a, b)
        assert np.array_equal(bits(got), bits(ref)), f"{kind} {tdt} n={n}"
    # the engine continues exactly after the calls
    assert np.array_equal(er.raw_u64(u, 8).cpu().numpy().view(np.uint64), e.raw(4))


def test_streams_split(gpulib, oracle):
    er = gpulib
    u = er.Vmt19937_64(11, streams=3, lanes=2)
    per = 4 * 1000
    got = draw(er, u, "UNIFORM_REAL", torch.float32, 0.0, 1.0, 3 * per)
    for k in range(3):
        ref = oracle.generate(oracle.Engine(11 + 4 * k, lanes=2), oracle.Gen(), "UNIFORM_REAL", per, np.float32)
        assert np.array_equal(bits(got[k * per:(k + 1) * per]), bits(ref)), f"stream {k}"


def test_other_kinds_refuse(gpulib):
    er = gpulib
    u = er.Vmt19937_64(1, lanes=2)
    d, keep = er._desc("NORMAL_STD", torch.float32)
    o = torch.empty(64, dtype=torch.float32, device="cuda")
    assert er._L.gr_sample(u._h, ctypes.byref(d), er._ptr(o), 64, er._stream_ptr()) == 3  # GR_ERR_UNSUPPORTED
    assert "2-lane" in er._L.gr_last_error().decode()
    with pytest.raises(er.GrError):
        er.MvNormalGen(np.zeros(2), np.eye(2)).generate(u, 16)
