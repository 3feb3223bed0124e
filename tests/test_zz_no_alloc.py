"""gr_raw_u64_noalloc, the allocation-free raw stream, against gr_raw_u64.

Some callers must not allocate device memory while they sample: a plugin
running inside a host framework that owns every device allocation, or a
thread with a real-time budget where cudaMalloc's unbounded latency is not
allowed.  They create the engine once at set-up and then call
gr_raw_u64_noalloc, which keeps its jump-ahead scratch in a fixed device
array instead of allocating.  This file checks, through the C ABI, that two
consecutive calls draw exactly what gr_raw_u64 draws from an identically
seeded engine, and what the CPU oracle draws from the reference stream.  The tolerance is the one every raw-stream test here uses:
bit-exact (the stream is integer data).

It is named so that pytest collects it last, and it needs nothing from the
other test files, so it runs the same alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _draw(er, fn, engine, n):
    out = torch.empty(n, dtype=torch.int64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    er._lib.check(fn(engine._h, ctypes.c_void_p(out.data_ptr()), n, stream))
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint64)


def test_noalloc_matches_allocating_raw_stream(gpulib, oracle):
    er = gpulib
    reference_engine = er.Vmt19937_64(20240)
    noalloc_engine = er.Vmt19937_64(20240)
    cpu_engine = oracle.Engine(20240)
    # the long calls take the jump-ahead path, which is the path that needs
    # scratch memory; their segment lengths differ (2^15 and 2^17 packets),
    # so consecutive calls switch between jump tables; the short ones run as
    # one segment
    for n in (1 << 22, 1 << 24, 1 << 22, (1 << 21) + 4 * 312, 1248, 4):
        want = _draw(er, er._L.gr_raw_u64, reference_engine, n)
        got = _draw(er, er._L.gr_raw_u64_noalloc, noalloc_engine, n)
        mismatches = np.count_nonzero(want != got)
        assert mismatches == 0, f"n={n}: {mismatches} draws differ from gr_raw_u64"
        # and directly against the CPU oracle's reference stream
        mismatches = np.count_nonzero(cpu_engine.raw(n // 4) != got)
        assert mismatches == 0, f"n={n}: {mismatches} draws differ from the oracle"


def test_noalloc_refuses_multi_stream_engines(gpulib):
    er = gpulib
    engine = er.Vmt19937_64(3, streams=4)
    dummy = torch.empty(16, dtype=torch.int64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    status = er._L.gr_raw_u64_noalloc(engine._h, ctypes.c_void_p(dummy.data_ptr()), 16, stream)
    assert status == 3  # GR_ERR_UNSUPPORTED
    assert "streams = 1" in er._L.gr_last_error().decode()


def test_noalloc_rejects_oversized_call(gpulib):
    er = gpulib
    engine = er.Vmt19937_64(1)
    dummy = torch.empty(4, dtype=torch.int64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    too_many = 4294967296 + 4  # GR_NOALLOC_MAX_DRAWS + one packet
    status = er._L.gr_raw_u64_noalloc(engine._h, ctypes.c_void_p(dummy.data_ptr()), too_many, stream)
    assert status == 1  # GR_ERR_INVALID, rejected before any launch
    assert "GR_NOALLOC_MAX_DRAWS" in er._L.gr_last_error().decode()
