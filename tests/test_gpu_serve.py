"""GPU checks of the serving loop: every result served in a concurrent mix is
bit-identical to the same client's plain call sequence run alone."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


@pytest.fixture(scope="module")
def er(gpulib):
    return gpulib


def make_trace(nreq, nclients, seed, lo=3, hi=5):
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(nreq):
        kind = ["NORMAL", "GAMMA", "BINOMIAL", "MVNORMAL"][rng.integers(4)]
        count = int(10 ** rng.uniform(lo, hi))
        c = int(rng.integers(nclients))
        if kind == "NORMAL":
            r = dict(kind=kind, dtype=[torch.float32, torch.float64][rng.integers(2)], a=0.0, b=1.0, trials=0)
        elif kind == "GAMMA":
            r = dict(kind=kind, dtype=[torch.float32, torch.float64][rng.integers(2)], a=float(10 ** rng.uniform(-1, 1)),
                     b=1.0, trials=0)
        elif kind == "BINOMIAL":
            r = dict(kind=kind, dtype=torch.int32, a=float(rng.uniform()), b=0.0, trials=int(rng.integers(1, 1001)))
        else:
            r = dict(kind=kind, dtype=torch.float32, a=0.0, b=0.0, trials=0)
        r.update(client=c, count=count)
        reqs.append(r)
    return reqs


def run_served(er, reqs, nclients, seeds, budget, slots, mv):
    from eigenrand_gb300.serving import Server
    srv = Server(nclients, seeds, budget, slots=slots)
    srv.set_mvnormal(*mv)
    tickets = [srv.submit(r["client"], r["kind"], r["dtype"], r["count"], r["a"], r["b"], r["trials"]) for r in reqs]
    results, done = {}, 0
    max_running, max_held = 0, 0
    while done < len(reqs):
        for c in srv.progress():
            assert c["status"] == 0, c
            results[c["ticket"]] = srv.read(c["ticket"], c["count"])
            srv.release(c["ticket"])
            done += 1
        q, r, b = srv.pending()
        max_running = max(max_running, r)
        max_held = max(max_held, b)
    return [results[t] for t in tickets], max_running, max_held


def run_alone(er, reqs, nclients, seeds, mv):
    """Each client's requests in order, plain calls on its own engine."""
    out = [None] * len(reqs)
    for c in range(nclients):
        u = er.Vmt19937_64(seeds[c])
        g = er.MvNormalGen(mv[0], mv[1])
        for i, r in enumerate(reqs):
            if r["client"] != c:
                continue
            if r["kind"] == "MVNORMAL":
                d = len(mv[0])
                s = -(-r["count"] // d)
                while (s * d) % 8:
                    s += 1
                x = g.generate(u, s)
                torch.cuda.synchronize()
                out[i] = x.t().contiguous().reshape(-1).cpu().numpy()
            else:
                P = 8 if r["dtype"] == torch.float32 else 4
                n = -(-r["count"] // P) * P
                x = er._sample(r["kind"], n, 1, u, r["dtype"], r["a"], r["b"], r["trials"])
                torch.cuda.synchronize()
                out[i] = x.reshape(-1).cpu().numpy()
    return out


def mv_params(d=64, seed=3):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((d, d))
    return rng.standard_normal(d), a @ a.T + d * np.eye(d)


def test_served_equals_alone(er):
    nclients = 6
    seeds = [1000 + c for c in range(nclients)]
    reqs = make_trace(90, nclients, 1)
    mv = mv_params()
    served, max_running, max_held = run_served(er, reqs, nclients, seeds, budget=1 << 30, slots=8, mv=mv)
    alone = run_alone(er, reqs, nclients, seeds, mv)
    for i, (a, b) in enumerate(zip(served, alone)):
        assert a.dtype == b.dtype and a.shape == b.shape, (i, reqs[i])
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (i, reqs[i])
    assert max_running > 1  # requests overlapped on the GPU


def test_budget_limits_memory_and_still_completes(er):
    nclients = 4
    seeds = [7 + c for c in range(nclients)]
    reqs = make_trace(40, nclients, 2, lo=4, hi=6)
    mv = mv_params()
    budget = 6 << 20  # 6 MiB: large requests have to wait for memory

    def budgeted(r):  # the server's accounting: output, plus 1.5x for data-dependent samplers' scratch
        b = r["count"] * (8 if r["dtype"] == torch.float64 else 4) + 1024
        return b * 5 // 2 if r["kind"] in ("GAMMA", "BINOMIAL") else b

    reqs = [r for r in reqs if budgeted(r) <= budget]
    served, _, max_held = run_served(er, reqs, nclients, seeds, budget=budget, slots=16, mv=mv)
    assert max_held <= budget
    alone = run_alone(er, reqs, nclients, seeds, mv)
    for a, b in zip(served, alone):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_oversized_request_is_refused(er):
    from eigenrand_gb300.serving import Server
    srv = Server(2, [1, 2], 1 << 20, slots=2)
    with pytest.raises(er.GrError, match="NOMEM"):
        srv.submit(0, "NORMAL", torch.float32, 1 << 20)


# ------------------------------------------------------------ cancellation and faults
# Failures are made on the host (a cancel, a client that goes away, a failing
# allocation from the test hook); no GPU fault is involved.
CANCELLED, NOMEM = 8, 4


def _drain(srv, tickets, limit_s=120.0):
    """progress() until every ticket is reported; {ticket: (status, data or None)}; every ticket released"""
    import time
    got = {}
    t_end = time.time() + limit_s
    while len(got) < len(tickets):
        for c in srv.progress():
            data = srv.read(c["ticket"], c["count"]) if c["status"] == 0 else None
            got[c["ticket"]] = (c["status"], data)
            srv.release(c["ticket"])
        assert time.time() < t_end, "server did not finish"
    return got


def _plain(er, seed, reqs):
    """the same requests as plain calls, in order, on Vmt19937_64(seed)"""
    u = er.Vmt19937_64(seed)
    out = []
    for kind, dt, count, a, b, trials in reqs:
        P = 8 if dt == torch.float32 else 4
        x = er._sample(kind, -(-count // P) * P, 1, u, dt, a, b, trials)
        torch.cuda.synchronize()
        out.append(x.reshape(-1).cpu().numpy())
    return out


def _same(a, b):
    return a.dtype == b.dtype and a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_cancel_queued_request_never_runs(er):
    from eigenrand_gb300.serving import Server
    srv = Server(1, [11], 1 << 30, slots=4)
    reqs = [("NORMAL", torch.float32, 4096, 0.0, 1.0, 0), ("GAMMA", torch.float32, 8192, 0.5, 1.0, 0),
            ("NORMAL", torch.float64, 2048, 1.0, 2.0, 0)]
    t = [srv.submit(0, *r) for r in reqs]
    srv.cancel(t[1])  # still queued: nothing has been admitted
    got = _drain(srv, t)
    assert got[t[1]] == (CANCELLED, None)
    ref = _plain(er, 11, [reqs[0], reqs[2]])  # the engine never drew for the cancelled one
    assert _same(got[t[0]][1], ref[0]) and _same(got[t[2]][1], ref[1])
    assert srv.pending() == (0, 0, 0)


def test_cancel_running_request_consumes_its_draws(er):
    from eigenrand_gb300.serving import Server
    srv = Server(1, [12], 1 << 30, slots=4)
    reqs = [("NORMAL", torch.float32, 1 << 22, 0.0, 1.0, 0), ("NORMAL", torch.float32, 4096, 0.0, 1.0, 0)]
    t = [srv.submit(0, *r) for r in reqs]
    assert srv.progress() == []  # the first request is admitted, not yet harvested
    assert srv.pending()[1] == 1
    srv.cancel(t[0])
    got = _drain(srv, t)
    assert got[t[0]] == (CANCELLED, None)
    ref = _plain(er, 12, reqs)  # it ran: its draws are consumed
    assert _same(got[t[1]][1], ref[1])
    assert srv.pending() == (0, 0, 0)
    with pytest.raises(er.GrError, match="INVALID"):
        srv.cancel(t[0])  # reported and released
    with pytest.raises(er.GrError, match="INVALID"):
        srv.cancel(12345)


def test_client_disconnect_mid_stream(er):
    """Client 1 goes away after its first request started: its running request
    finishes and is dropped, its queued ones never run, the memory comes back,
    and the other clients' results are unchanged."""
    from eigenrand_gb300.serving import Server
    seeds = [21, 22, 23]
    srv = Server(3, seeds, 1 << 30, slots=8)
    per = {0: [("NORMAL", torch.float32, 1 << 16, 0.0, 1.0, 0), ("GAMMA", torch.float64, 1 << 14, 2.5, 1.0, 0)],
           1: [("NORMAL", torch.float32, 1 << 21, 0.0, 1.0, 0), ("BINOMIAL", torch.int32, 1 << 14, 0.3, 0.0, 20),
               ("NORMAL", torch.float64, 1 << 12, 0.0, 1.0, 0)],
           2: [("BINOMIAL", torch.int32, 1 << 15, 0.7, 0.0, 50), ("NORMAL", torch.float32, 1 << 13, 3.0, 0.5, 0)]}
    tk = {c: [] for c in per}
    for i in range(3):  # interleaved submission
        for c in per:
            if i < len(per[c]):
                tk[c].append(srv.submit(c, *per[c][i]))
    srv.progress()  # every client's first request starts
    srv.cancel_client(1)
    got = _drain(srv, [t for c in tk for t in tk[c]])
    assert all(got[t] == (CANCELLED, None) for t in tk[1])
    for c in (0, 2):
        ref = _plain(er, seeds[c], per[c])
        assert all(_same(got[t][1], r) for t, r in zip(tk[c], ref))
    assert srv.pending() == (0, 0, 0)


def test_allocation_failure_leaves_engine_untouched(er):
    from eigenrand_gb300.serving import Server
    srv = Server(1, [13], 1 << 30, slots=2)
    srv.fail_allocs(1)
    reqs = [("NORMAL", torch.float32, 4096, 0.0, 1.0, 0), ("GAMMA", torch.float32, 4096, 0.7, 1.0, 0)]
    t = [srv.submit(0, *r) for r in reqs]
    got = _drain(srv, t)
    assert got[t[0]] == (NOMEM, None)
    ref = _plain(er, 13, [reqs[1]])
    assert _same(got[t[1]][1], ref[0])
    assert srv.pending() == (0, 0, 0)
