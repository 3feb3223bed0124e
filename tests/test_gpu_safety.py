"""Iteration caps of the rejection and walk kernels.

The reference guards its unbounded loops with EIGENRAND_CHECK_INFINITY_LOOP
(EigenRand/RandUtils.h:342-346).  Here every data-dependent kernel bounds the
engine blocks it may generate in one call; at the bound it stops, records
GR_DEV_REJECT_LIMIT in the engine's status word and returns, so the GPU
context stays usable.  GR_MAX_BLOCKS (a test hook read on the host) lowers
the bound to one block, far below what the call needs, and the test checks
that gr_engine_sync reports GR_ERR_REJECT_LIMIT once, that the status word is
cleared afterwards, and that the same engine, reseeded, draws the reference
stream again.  No kernel waits on anything here: the cap is a loop bound.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

GR_OK, GR_ERR_REJECT_LIMIT = 0, 5


@pytest.mark.parametrize("kind,tdt,a,b,t,n,streams", [
    ("GAMMA", torch.float32, 0.5, 1.0, 0, 8 * 2048, 1),        # CompressMask rejection, one CTA per stream
    ("GAMMA", torch.float32, 0.5, 1.0, 0, 8 * 100000, 1),      # segmented rejection, last segment runs on
    ("GAMMA", torch.float64, 0.5, 1.0, 0, 4 * 4096, 8),        # rejection on several streams
    ("BETA", torch.float64, 0.5, 2.0, 0, 4 * 4096, 2),         # beta walk
    ("POISSON", torch.int32, 4.0, 0.0, 0, 4 * 4096, 1),        # Poisson walk
    ("POISSON", torch.int32, 4.0, 0.0, 0, 4 * 200000, 1),      # Poisson walk over segments
    ("POISSON", torch.int32, 100.0, 0.0, 0, 4 * 2048, 1),      # tan rejection, int32
])
def test_cap_reports_and_engine_recovers(gpulib, oracle, monkeypatch, kind, tdt, a, b, t, n, streams):
    er = gpulib
    u = er.Vmt19937_64(5, streams=streams)
    stream = er._stream_ptr()
    d, keep = er._desc(kind, tdt, a, b, t)
    o = torch.empty(n, dtype=tdt, device="cuda")
    monkeypatch.setenv("GR_MAX_BLOCKS", "1")
    # long single-engine calls run as planned segments and only the last one
    # may run past its plan: plan too few so that it runs into the cap
    monkeypatch.setenv("GR_REJECT_PLAN_SCALE", "0.3")
    monkeypatch.setenv("GR_WALK_PLAN_SCALE", "0.3")
    assert er._L.gr_sample(u._h, ctypes.byref(d), er._ptr(o), n, stream) == GR_OK  # the launch itself succeeds
    assert er._L.gr_engine_sync(u._h, stream) == GR_ERR_REJECT_LIMIT
    assert "iteration cap" in er._L.gr_last_error().decode()
    assert er._L.gr_engine_sync(u._h, stream) == GR_OK  # reported once, then cleared
    for v in ("GR_MAX_BLOCKS", "GR_REJECT_PLAN_SCALE", "GR_WALK_PLAN_SCALE"):
        monkeypatch.delenv(v)
    # the engine and the context remain usable: reseeded, it draws the reference stream
    u.seed(11)
    raw = er.raw_u64(u, 4 * 64 * streams).cpu().numpy().view(np.uint64)
    for k in range(streams):
        np.testing.assert_array_equal(raw[k * 256:(k + 1) * 256], oracle.Engine(11 + 4 * k).raw(64))
    # and a full call of the same kind completes and matches the oracle
    u.seed(13)
    assert er._L.gr_sample(u._h, ctypes.byref(d), er._ptr(o), n, stream) == GR_OK
    assert er._L.gr_engine_sync(u._h, stream) == GR_OK
    got = o.cpu().numpy()
    npdt = {torch.float32: np.float32, torch.float64: np.float64, torch.int32: np.int32}[tdt]
    per = n // streams
    for k in (0, streams - 1):
        ref = oracle.generate(oracle.Engine(13 + 4 * k), oracle.Gen(), kind, per, npdt, a, b, t)
        bits = np.uint64 if got.itemsize == 8 else np.uint32
        assert np.array_equal(got[k * per:(k + 1) * per].view(bits), ref.view(bits)), f"stream {k}"
