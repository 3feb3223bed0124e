"""Batched vectorize-over-params sets (gr_sample_batched) against the oracle.

Set i is a fresh Vmt19937_64(seed + 4 i) with a fresh generator; the oracle
replays exactly that per set (bit-exact)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _sets(kind, nsets, seed):
    rng = np.random.default_rng(seed)
    counts = rng.integers(1, 300, nsets).astype(np.int32)
    if kind == "GAMMA":
        a = (10.0 ** rng.uniform(-1, 2, nsets)).astype(np.float32)
        a[:4] = [1.0, 5.0, 0.5, 19.0]  # the closed-form and edge branches
        b = rng.uniform(0.5, 2.0, nsets).astype(np.float32)
        return counts, a, b, None
    a = rng.uniform(0, 1, nsets).astype(np.float32)
    t = rng.integers(1, 1000, nsets).astype(np.int32)
    a[:6] = [0.5, 0.01, 0.99, 0.3, 0.8, 0.0]
    t[:6] = [1, 50, 100, 24, 3, 7]
    return counts, a, None, t


@pytest.mark.parametrize("kind", ["GAMMA", "BINOMIAL_V"])
def test_batched_sets_match_oracle(gpulib, oracle, kind):
    er = gpulib
    counts, a, b, t = _sets(kind, 80, 3)
    out, off = er.sample_batched(kind, torch.from_numpy(counts), torch.from_numpy(a),
                                 None if b is None else torch.from_numpy(b),
                                 None if t is None else torch.from_numpy(t), seed=777)
    torch.cuda.synchronize()
    out = out.cpu().numpy()
    off = off.cpu().numpy()
    for i in range(len(counts)):
        ref = oracle.vop_set(777 + 4 * i, kind, int(counts[i]), float(a[i]), 1.0 if b is None else float(b[i]),
                             0 if t is None else int(t[i]))
        got = out[off[i]:off[i] + counts[i]]
        bad = np.nonzero(got.view(np.uint32) != ref.view(np.uint32))[0]
        assert bad.size == 0, f"set {i} ({a[i]}, {None if b is None else b[i]}, {None if t is None else t[i]}): {bad[:5]}"


@pytest.mark.parametrize("kind", ["GAMMA", "BINOMIAL_V"])
def test_batched_equals_per_call_and_graph_replay(gpulib, kind):
    er = gpulib
    counts, a, b, t = _sets(kind, 40, 9)
    tc, ta = torch.from_numpy(counts), torch.from_numpy(a)
    tb = None if b is None else torch.from_numpy(b)
    tt = None if t is None else torch.from_numpy(t)
    out, off = er.sample_batched(kind, tc, ta, tb, tt, seed=1234)
    torch.cuda.synchronize()
    whole = out.cpu().numpy()
    # per-call: one set per call, same seeds
    for i in range(len(counts)):
        o1, _ = er.sample_batched(kind, tc[i:i + 1], ta[i:i + 1], None if tb is None else tb[i:i + 1],
                                  None if tt is None else tt[i:i + 1], seed=1234 + 4 * i)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(o1.cpu().numpy()[:counts[i]], whole[off[i].item():off[i].item() + counts[i]])
    # captured in a CUDA graph and replayed (inputs staged on the device first)
    dc, da = tc.cuda(), ta.cuda()
    db = None if tb is None else tb.cuda()
    dt = None if tt is None else tt.cuda()
    out2 = torch.empty_like(out)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        er.sample_batched(kind, dc, da, db, dt, seed=1234, out=out2, offsets=off, stream=s)  # tuned already
        s.synchronize()
        g = torch.cuda.CUDAGraph()
        out3 = torch.zeros_like(out)
        with torch.cuda.graph(g, stream=s):
            er.sample_batched(kind, dc, da, db, dt, seed=1234, out=out3, offsets=off, stream=s)
    g.replay()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out3.cpu().numpy(), whole)
