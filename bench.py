"""Benchmark: EigenRand's univariate sweep on one GB300.

Workload (one step): every distribution of the univariate sweep drawn into a
4096x4096 array, float32 and float64 (int32 for the integer kinds), from one
Vmt19937_64 engine seeded 1234 that is carried across the whole sweep, as the
reference benchmark does (benchmark/benchmark.cpp:15-20: one engine, all
distributions in sequence).  Each distribution writes its own output buffer,
so a step writes ~2.4 GB, far more than the 129 MB L2.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--mode compat|streams]

--mode streams (default): 608 independent Vmt19937_64(1234 + 4k) engines, every
                call's output split into contiguous slices (bit-exact per slice
                with the reference run as one engine per thread).
--mode compat : the engine is a single Vmt19937_64 (bit-exact with the single
                reference stream; long closed-form calls use jump-ahead
                segments, the data-dependent samplers run on one CTA).
Prints one JSON line.  N > 1 runs independent replicas (the sampler has no
data-parallel exchange), one per rank.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

ROWS = COLS = 4096
N = ROWS * COLS

# (name, kind, dtype tag, a, b, trials, weights) — the univariate sweep
W16 = [0.5488135, 0.71518937, 0.60276338, 0.54488318, 0.4236548, 0.64589411, 0.43758721, 0.891773,
       0.96366276, 0.38344152, 0.79172504, 0.52889492, 0.56804456, 0.92559664, 0.07103606, 0.0871293]
SWEEP_REAL = [
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
SWEEP_INT = [
    ("poisson4", "POISSON", 4.0, 0.0, 0, None),
    ("poisson100", "POISSON", 100.0, 0.0, 0, None),
    ("binomial20", "BINOMIAL", 0.3, 0.0, 20, None),
    ("discrete16", "DISCRETE", 0.0, 0.0, 0, W16),
]


def sweep_items():
    items = []
    for name, kind, a, b in SWEEP_REAL:
        items.append((name + "/f32", kind, "f32", a, b, 0, None))
        items.append((name + "/f64", kind, "f64", a, b, 0, None))
    for name, kind, a, b, t, w in SWEEP_INT:
        items.append((name + "/i32", kind, "i32", a, b, t, w))
    return items


def elem_bytes(tag):
    return {"f32": 4, "f64": 8, "i32": 4}[tag]


def kernel_of(name, compat=False):
    """Sampling kernel of a sweep entry (streams mode: one launch per call;
    compat: the single-engine kernels)."""
    base, tag = name.split("/")
    if compat:
        if base == "beta":
            return f"k_beta<{'float' if tag == 'f32' else 'double'}, GS, integral> (one CTA, visit table)"
        if base == "poisson4":
            return "k_poisson (one CTA)"
        if base in ("gamma0.5", "poisson100"):
            return "k_rs_count/scan/write/gather/finish (segmented rejection)"
        return "k_prefix + k_jump + " + ("k_staged" if base in ("gamma5", "binomial20") else "k_direct") + \
            " (jump-ahead segments)"
    if base == "beta":
        return f"k_beta<{'float' if tag == 'f32' else 'double'}, GS, integral>"
    if base in ("gamma0.5", "poisson100"):
        return "k_reject"
    if base in ("gamma5", "binomial20"):
        return "k_staged"
    if base == "poisson4":
        return "k_poisson"
    return "k_direct"


# DRAM bytes per sample of a sweep entry's kernel, from one ncu capture each
# (dram__bytes_read.sum + dram__bytes_write.sum over the samples of the
# launch; the capture command is in the named profiles/ summary), and what
# binds the kernel when it is not HBM
MEASURED = {
    "uniformReal/f32": {"dram_bytes_per_sample": 3.276, "profile": "profiles/k_direct_uniform_f32_8192sq.md"},
    "beta/f64": {"dram_bytes_per_sample": 5.19, "fp64_pipe_active": 0.270, "issue_active": 0.633,
                 "note": "issue-bound on the integer double log / exp of the masks and values (the walk "
                         "runs on its own warp): issue active 63%, ALU 52%, FP64 pipe 27% (not HBM)",
                 "profile": "profiles/k_beta_f64_2048sq.md"},
}


def roofline_entry(name, pd, hbm_peak, peaks, measured=True):
    """Roofline of one sweep entry's kernel: algorithmic bytes (the output,
    4 or 8 B per sample, 2^24 samples per launch) / its graph-replay time.
    measured=False: the ncu figures (captured on the 608-stream engine) do
    not apply."""
    m = MEASURED.get(name, {}) if measured else {}
    bps = m.get("dram_bytes_per_sample")
    e = {"kernel": f"{kernel_of(name, compat=not measured)} ({name})", "bound": "hbm", "achieved": pd["gbs"], "peak": hbm_peak,
         "unit": "GB/s", "frac": round(pd["gbs"] / hbm_peak, 4),
         "traffic": round(bps * N) if bps else None,
         "peak_source": "measured" if peaks else "fallback"}
    for key in ("fp64_pipe_active", "issue_active", "note"):
        if m.get(key) is not None:
            e[key] = m[key]
    if m.get("profile"):
        e["profile"] = m["profile"]
    return e


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, idx=0):
        self.idx = idx
        self.samples = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx.append(float(s[1]))
                for nm, v in zip(names, s[3:7]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


# --------------------------------------------------------------------------- ours
class Sweep:
    """The 26 calls of the sweep on one engine: one generator object per
    distribution (the reference benchmark's "/gen" form, reused across steps;
    4096^2 is a whole number of packets, so no cache carries between calls and
    the values equal the free functions'), one output buffer per call."""

    def __init__(self, er, urng, items):
        import torch
        self.er, self.urng, self.items = er, urng, items
        tdt = {"f32": torch.float32, "f64": torch.float64, "i32": torch.int32}
        self.outs = [torch.empty(N, dtype=tdt[t], device="cuda") for (_, _, t, *_r) in items]
        self.gens = []
        for (name, kind, t, a, b, tr, w) in items:
            d, keep = er._desc(kind, tdt[t], a, b, tr, w)
            h = ctypes.c_void_p()
            er._lib.check(er._L.gr_gen_create(ctypes.byref(h), ctypes.byref(d)))
            self.gens.append(h)

    def close(self):
        for h in self.gens:
            self.er._L.gr_gen_destroy(h)
        self.gens = []
        self.outs = []

    def one(self, i, s=None):
        import torch
        sp = ctypes.c_void_p((s or torch.cuda.current_stream()).cuda_stream)
        self.er._lib.check(self.er._L.gr_generate(self.gens[i], self.urng._h,
                                                  ctypes.c_void_p(self.outs[i].data_ptr()), N, sp))

    def step(self):
        for i in range(len(self.items)):
            self.one(i)

    def per_call_ms(self, R):
        """Device time of each call: R calls captured in a CUDA graph, replayed
        between CUDA events (no host launch gaps in the interval); median of 3."""
        import torch
        stream = torch.cuda.current_stream()
        per = {}
        for i, it in enumerate(self.items):
            g = torch.cuda.CUDAGraph()
            cs = torch.cuda.Stream()
            cs.wait_stream(stream)
            with torch.cuda.stream(cs):
                self.one(i, cs)  # warm on the capture stream
                cs.synchronize()
                with torch.cuda.graph(g, stream=cs):
                    for _ in range(R):
                        self.one(i, cs)
            stream.wait_stream(cs)
            torch.cuda.synchronize()
            for rep in range(3):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                g.replay()
                e1.record(stream)
                e1.synchronize()
                per.setdefault(it[0], []).append(e0.elapsed_time(e1) / R)
            del g
        torch.cuda.synchronize()
        return {k: statistics.median(v) for k, v in per.items()}

    def timed_steps(self, steps):
        """ms for `steps` whole sweeps between CUDA events on the launching stream."""
        import torch
        stream = torch.cuda.current_stream()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(steps):
            self.step()
        t1.record(stream)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1)


def per_dist_table(items, per, hbm_peak):
    out = {}
    for name, kind, t, *_r in items:
        m = per[name]
        gb = N * elem_bytes(t) / 1e9
        out[name] = {"ms": round(m, 4), "gsamples_s": round(N / (m / 1e3) / 1e9, 3),
                     "gbs": round(gb / (m / 1e3), 1), "hbm_frac": round(gb / (m / 1e3) / hbm_peak, 3)}
    return out


def run_ours(args, rank, world):
    import torch
    import eigenrand_gb300 as er

    dev = rank % max(1, torch.cuda.device_count())
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    streams = 608 if args.mode == "streams" else 1
    seed = 1234 + rank * 4 * 1000003  # replicas draw disjoint engines
    urng = er.Vmt19937_64(seed, streams=streams)
    items = sweep_items()
    sw = Sweep(er, urng, items)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        sw.step()
    torch.cuda.synchronize()
    per = sw.per_call_ms(8 if streams > 1 else 1)

    clocks = ClockSampler(dev)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ms = sw.timed_steps(args.steps)
    barrier()
    clk = clocks.stop()
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    samples_per_step = N * len(items)
    value = samples_per_step * args.steps * world / (ms / 1e3) / 1e9

    # e2e: the same sweep through the public API into host memory (pinned),
    # D2H copy of every result inside the timed region.  The copies run on a
    # second stream, each after its call's event, so call i + 1 samples while
    # call i's result travels to the host; before a call rewrites a buffer it
    # waits for the previous step's copy out of it.
    outs = sw.outs
    host = [torch.empty(N, dtype=o.dtype, pin_memory=True) for o in outs]
    cstream = torch.cuda.Stream()
    done = [torch.cuda.Event() for _ in outs]
    copied = [torch.cuda.Event() for _ in outs]

    def e2e_step():
        for i in range(len(items)):
            stream.wait_event(copied[i])
            sw.one(i)
            done[i].record(stream)
            cstream.wait_event(done[i])
            with torch.cuda.stream(cstream):
                host[i].copy_(outs[i], non_blocking=True)
            copied[i].record(cstream)

    for ev in copied:
        ev.record(cstream)
    e2e_step()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    stream.wait_stream(cstream)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1)
    d2h = sum(o.numel() * o.element_size() for o in outs)
    del host

    peaks = load_peaks()
    hbm_peak = peaks["hbm_gbs"] if peaks else 6800.0
    per_dist = per_dist_table(items, per, hbm_peak)
    # roofline of the dominant kernel (the slowest call of the step) and of
    # the HBM-write-bound uniform float kernel
    best_name = max(per, key=per.get)
    launches_per_call = 1 if streams > 1 else 3
    if streams > 1:
        workload = (f"univariate sweep 4096x4096 per call, 26 calls (11 kinds f32 + f64, 4 int32 kinds); "
                    f"engine: {streams} independent Vmt19937_64(1234 + 4k) streams (one per engine, the "
                    f"reference's one-engine-per-thread usage), each filling a contiguous slice of every call; "
                    f"the single-engine Vmt19937_64(1234) sweep is timed under 'compat'")
    else:
        workload = ("univariate sweep 4096x4096 per call, 26 calls; engine: one Vmt19937_64(1234) carried "
                    "across the sweep (the reference stream, bit-exact)")
    res = {
        "metric": "Gsamples/s (univariate sweep, 4096x4096 per distribution)",
        "value": round(value, 3),
        "unit": "Gsamples/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64+i32",
        "data": "synthetic (engine seeded 1234)",
        "config": {"workload": workload,
                   "engine_mode": args.mode, "engine_streams": streams,
                   "distributions": [it[0] for it in items],
                   "l2": "distinct output buffer per distribution; 2.4 GB written per step > 129 MB L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "per_dist": per_dist,
        "roofline": roofline_entry(best_name, per_dist[best_name], hbm_peak, peaks),
        "roofline_hbm_kernel": roofline_entry("uniformReal/f32", per_dist["uniformReal/f32"], hbm_peak, peaks),
        "e2e": {"value": round(samples_per_step * args.steps * world / (e2e_ms / 1e3) / 1e9, 3),
                "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches_per_call * len(items) * args.steps,
        "clocks": clk,
    }
    sw.close()
    del sw, outs
    torch.cuda.empty_cache()
    if streams > 1 and not args.no_compat:
        res["compat"] = bench_compat(er, items, hbm_peak, peaks, steps=max(3, min(args.steps, 10)))
    if not args.no_extras:
        res["workloads"] = {"batched_vop": bench_batched(er), "multivariate": bench_multivariate(er),
                            "truncated_and_per_element": bench_next_rows(er),
                            "serving": bench_serving(er, seconds=args.serve_seconds)}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline(seconds=args.cpu_seconds)
    return res


def bench_compat(er, items, hbm_peak, peaks, steps=5, warmup=3):
    """The sweep on ONE Vmt19937_64(1234) carried across all 26 calls: the
    single reference stream, bit-exact with the reference run as written.
    Long calls run as jump-ahead segments (closed forms) or segmented
    rejection; the data-dependent walks run on one CTA."""
    import torch
    urng = er.Vmt19937_64(1234)
    sw = Sweep(er, urng, items)
    for _ in range(warmup):
        sw.step()
    torch.cuda.synchronize()
    per = sw.per_call_ms(1)
    ms = sw.timed_steps(steps)
    value = N * len(items) * steps / (ms / 1e3) / 1e9
    per_dist = per_dist_table(items, per, hbm_peak)
    best = max(per, key=per.get)
    sw.close()
    torch.cuda.empty_cache()
    return {"workload": "univariate sweep 4096x4096 per call, 26 calls, one Vmt19937_64(1234) carried across "
                        "the sweep (the reference benchmark's engine use, benchmark/benchmark.cpp:15-20)",
            "value": round(value, 3), "unit": "Gsamples/s", "steps": steps, "warmup": warmup,
            "ms_per_step": round(ms / steps, 4), "per_dist": per_dist,
            "roofline": roofline_entry(best, per_dist[best], hbm_peak, peaks, measured=False),
            "roofline_hbm_kernel": roofline_entry("uniformReal/f32", per_dist["uniformReal/f32"], hbm_peak, peaks,
                                                  measured=False)}


# --------------------------------------------------------------------------- other workloads
def _median_ms(fn, reps=3, warm=1):
    """Median device time of fn() in ms (CUDA events on the current stream)."""
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    ts = []
    st = torch.cuda.current_stream()
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fn()
        e1.record(st)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def bench_batched(er, nsets=1_000_000, percall_sets=2048):
    """Batched vectorize-over-params: 10^6 sets in one launch (captured in a
    CUDA graph, CTA width from the library's autotuner) against the plain
    per-call path (one gr_sample_batched call per set, the same values)."""
    import numpy as np
    import torch
    rng = np.random.default_rng(7)
    counts = rng.integers(1, 4097, nsets).astype(np.int32)
    res = {}
    for kind in ("GAMMA", "BINOMIAL_V"):
        if kind == "GAMMA":
            a = (10.0 ** rng.uniform(-1, 2, nsets)).astype(np.float32)
            b = np.ones(nsets, np.float32)
            t = None
        else:
            a = rng.uniform(0, 1, nsets).astype(np.float32)
            b = None
            t = rng.integers(1, 1001, nsets).astype(np.int32)
        tc = torch.from_numpy(counts).cuda()
        ta = torch.from_numpy(a).cuda()
        tb = torch.from_numpy(b).cuda() if b is not None else None
        tt = torch.from_numpy(t).cuda() if t is not None else None
        out, off = er.sample_batched(kind, tc, ta, tb, tt, seed=7)  # first call autotunes
        torch.cuda.synchronize()
        total = int(counts.astype(np.int64).sum())
        s = torch.cuda.Stream()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            er.sample_batched(kind, tc, ta, tb, tt, seed=7, out=out, offsets=off, stream=s)
            s.synchronize()
            with torch.cuda.graph(g, stream=s):
                er.sample_batched(kind, tc, ta, tb, tt, seed=7, out=out, offsets=off, stream=s)
        torch.cuda.synchronize()
        ms = _median_ms(g.replay)
        # plain per-call path on the first sets
        M = percall_sets
        outs1 = torch.empty(4096 + 8, dtype=out.dtype, device="cuda")
        off1 = torch.zeros(1, dtype=torch.int64, device="cuda")
        one = [(tc[i:i + 1], ta[i:i + 1], None if tb is None else tb[i:i + 1], None if tt is None else tt[i:i + 1])
               for i in range(M)]

        def percall():
            for i in range(M):
                c, aa, bb, trr = one[i]
                er.sample_batched(kind, c, aa, bb, trr, seed=7 + 4 * i, out=outs1, offsets=off1)
        ms1 = _median_ms(percall, reps=2)
        m_samples = int(counts[:M].astype(np.int64).sum())
        res[kind.lower()] = {
            "sets": nsets, "samples": total, "batched_ms": round(ms, 3),
            "batched_gsamples_s": round(total / (ms / 1e3) / 1e9, 3),
            "batched_gbs_out": round(total * 4 / (ms / 1e3) / 1e9, 1),
            "percall_sets_timed": M, "percall_ms": round(ms1, 3),
            "percall_gsamples_s": round(m_samples / (ms1 / 1e3) / 1e9, 4),
            "speedup_batched_vs_percall": round((total / ms) / (m_samples / ms1), 1),
        }
        del out, g
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return res


def bench_multivariate(er, streams=608):
    """MvNormal d in {16, 64, 128, 256} (N = 10^6), Wishart d=32 df=40 (10^5 draws),
    Dirichlet K=64 (10^6), Multinomial K=100 trials=1000 (10^6); float32."""
    import numpy as np
    import torch
    urng = er.Vmt19937_64(99, streams=streams)
    res = {}
    N = 1_000_000
    for d in (16, 64, 128, 256):
        rng = np.random.default_rng(99)
        A = rng.standard_normal((d, d))
        cov = A @ A.T + d * np.eye(d)
        mean = rng.standard_normal(d)
        g = er.MvNormalGen(mean, cov)
        out = torch.empty((N, d), dtype=torch.float32, device="cuda").t()
        ms = _median_ms(lambda: g.generate(urng, N, out=out))
        z = er.StdNormalGen()
        ms_z = _median_ms(lambda: z.generate(d, N, urng, out=out))
        gemm = max(ms - ms_z, 1e-6)
        res[f"mvnormal_d{d}"] = {
            "samples": N, "ms": round(ms, 3), "msamples_s": round(N / ms / 1e3, 1),
            "gbs_out": round(4 * d * N / (ms / 1e3) / 1e9, 1),
            "normals_ms": round(ms_z, 3), "lz_ms": round(gemm, 3),
            "lz_tflops_full": round(2 * d * d * N / (gemm / 1e3) / 1e12, 2),
            "lz_bytes_gbs": round(8 * d * N / (gemm / 1e3) / 1e9, 1)}
        del out
    d, df, n = 32, 40, 100_000
    rng = np.random.default_rng(99)
    A = rng.standard_normal((d, d))
    w = er.WishartGen(df, A @ A.T + d * np.eye(d))
    out = torch.empty((d * n, d), dtype=torch.float32, device="cuda").t()
    ms = _median_ms(lambda: w.generate(urng, n, out=out))
    res["wishart_d32"] = {"draws": n, "ms": round(ms, 3), "kdraws_s": round(n / ms, 1),
                          "gbs_out": round(4 * d * d * n / (ms / 1e3) / 1e9, 1)}
    del out
    K, n = 64, 1_000_000
    alpha = np.random.default_rng(99).uniform(0.1, 2.0, K)
    dg = er.DirichletGen(alpha)
    out = torch.empty((n, K), dtype=torch.float32, device="cuda").t()
    ms = _median_ms(lambda: dg.generate(urng, n, out=out))
    res["dirichlet_k64"] = {"draws": n, "ms": round(ms, 3), "mdraws_s": round(n / ms / 1e3, 2),
                            "gbs_out": round(4 * K * n / (ms / 1e3) / 1e9, 1)}
    del out
    K, trials, n = 100, 1000, 1_000_000
    p = np.random.default_rng(99).dirichlet(np.ones(K))
    mg = er.MultinomialGen(trials, p)
    out = torch.empty((n, K), dtype=torch.int32, device="cuda").t()
    ms = _median_ms(lambda: mg.generate(urng, n, out=out))
    res["multinomial_k100_t1000"] = {"draws": n, "ms": round(ms, 3), "mdraws_s": round(n / ms / 1e3, 2),
                                     "alias_draws_g_s": round(n * trials / (ms / 1e3) / 1e9, 1),
                                     "gbs_out": round(4 * K * n / (ms / 1e3) / 1e9, 1)}
    del out
    # trials >= max(30 (K - 1), 100): the conditional-binomial path
    K, trials, n = 10, 1000, 1_000_000
    p = np.random.default_rng(99).dirichlet(np.ones(K))
    mg = er.MultinomialGen(trials, p)
    out = torch.empty((n, K), dtype=torch.int32, device="cuda").t()
    ms = _median_ms(lambda: mg.generate(urng, n, out=out))
    res["multinomial_k10_t1000_conditional"] = {"draws": n, "ms": round(ms, 3), "mdraws_s": round(n / ms / 1e3, 2),
                                                "binomial_rows_g_s": round(n * (K - 1) / (ms / 1e3) / 1e9, 2),
                                                "gbs_out": round(4 * K * n / (ms / 1e3) / 1e9, 1)}
    del out
    # TruncMvNormalGen, the 9-dimensional case of the reference's tests, default
    # burn-in (5 * dim sweeps, one scalar draw per component and chain)
    c = np.zeros((9, 9))
    c[0, 1], c[2, 7], c[3, 1] = 0.5, 0.5, 0.7
    c[np.diag_indices(9)] = [1, 1.2, 1.4, 1.6, 1.8, 1.6, 1.4, 1.2, 1]
    tg = er.TruncMvNormalGen([-1, 0, 1, 2, 3, 2, 1, 0, -1], c @ c.T,
                             er.support([-4, -3, -2, -1, 0, -1, -2, -3, -4], [4, 5, 6, 7, 8, 7, 6, 5, 4]))
    n = 100_000
    out = torch.empty((n, 9), dtype=torch.float32, device="cuda").t()
    ms = _median_ms(lambda: tg.generate(urng, n, out=out))
    res["truncmvnormal_d9_n1e5"] = {"samples": n, "ms": round(ms, 3), "gibbs_steps_g_s":
                                    round(n * 9 * 45 / (ms / 1e3) / 1e9, 2)}
    del out
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return res


def bench_next_rows(er, streams=608):
    """Truncated family and per-element forms at 4096x4096: inverse-CDF
    TruncGen / TruncNormalGen and *VGen on the streams engine; TruncGen's
    CompressMask rejection (gamma base) on one Vmt19937_64, the only engine
    form it takes."""
    import torch
    N = 4096 * 4096
    urng = er.Vmt19937_64(1234, streams=streams)
    res = {}

    def entry(ms, nbytes):
        return {"ms": round(ms, 3), "gsamples_s": round(N / (ms / 1e3) / 1e9, 2),
                "gbs": round(nbytes / (ms / 1e3) / 1e9, 1)}
    for tdt, tag in ((torch.float32, "f32"), (torch.float64, "f64")):
        es = 4 if tdt == torch.float32 else 8
        out = torch.empty((4096, 4096), dtype=tdt, device="cuda")
        tn = er.TruncNormalGen(0.0, 1.0, er.support(-1.0, 2.0), dtype=tdt)
        res[f"truncNormal/{tag}"] = entry(_median_ms(lambda: tn.generate(4096, 4096, urng, out=out)), N * es)
        te = er.TruncGen(er.ExponentialGen(1.0, dtype=tdt), er.support(0.5, 3.0))
        res[f"truncExponential/{tag}"] = entry(_median_ms(lambda: te.generate(4096, 4096, urng, out=out)), N * es)
        mean = torch.rand(N, dtype=tdt, device="cuda")
        sd = torch.rand(N, dtype=tdt, device="cuda") + 0.5
        res[f"normalV/{tag}"] = entry(_median_ms(lambda: er.normal(urng, mean, sd, out=out.view(-1))), 3 * N * es)
        res[f"studentTV/{tag}"] = entry(_median_ms(lambda: er.studentT(urng, sd, out=out.view(-1))), 2 * N * es)
        one = er.Vmt19937_64(1234)
        tg = er.TruncGen(er.GammaGen(2.0, 1.0, dtype=tdt), er.support(0.5, 5.0))
        tg.generate(4096, 4096, one, out=out)  # first call: pilot chunk learns the acceptance
        res[f"truncGammaReject/{tag}"] = entry(_median_ms(lambda: tg.generate(4096, 4096, one, out=out)), N * es)
        res[f"gamma2_single_stream/{tag}"] = entry(
            _median_ms(lambda: er.gamma(4096, 4096, one, 2.0, 1.0, dtype=tdt, out=out)), N * es)
        del out, mean, sd
    # binomialV: the reference's vectorize-over-params pattern (trials 20 / 50 /
    # 100 by column, p 0.5 / 0.01 / 0.75 by row), 12 bytes per sample
    idx = torch.arange(4096, device="cuda")
    trials = torch.tensor([20, 50, 100], dtype=torch.int32, device="cuda")[idx % 3][None, :].expand(4096, 4096)
    pr = torch.tensor([0.5, 0.01, 0.75], device="cuda")[idx % 3][:, None].expand(4096, 4096)
    trials, pr = trials.t().contiguous().t(), pr.t().contiguous().t()
    outi = torch.empty_like(trials)
    res["binomialV/i32"] = entry(_median_ms(lambda: er.binomial(urng, trials, pr, out=outi)), 12 * N)
    del trials, pr, outi
    # gamma(0.5) with P8_mt19937_64 (the reference tests' engine) as the Urng:
    # pre-drawn words, all trials evaluated at once, CompressMask filter
    p8 = er.P8_mt19937_64(1234)
    for tdt, tag in ((torch.float32, "f32"), (torch.float64, "f64")):
        es = 4 if tdt == torch.float32 else 8
        out = torch.empty((4096, 4096), dtype=tdt, device="cuda")
        res[f"gamma0.5_P8_mt19937_64/{tag}"] = entry(
            _median_ms(lambda: er.gamma(4096, 4096, p8, 0.5, 1.0, dtype=tdt, out=out)), N * es)
        del out
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return res


def make_serving_trace(seconds, rate=2000.0, nclients=256, seed=5):
    """Poisson arrivals (exponential gaps, mean 1/rate); kind uniform over
    {normal, gamma(alpha = 10^U(-1,1)), binomial(n ~ U{1..1000}, p ~ U(0,1)),
    MvNormal d=64}; output scalars log-uniform in [10^3, 10^8]; float32 /
    float64 half and half (MvNormal float32, binomial int32)."""
    import numpy as np
    import torch
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        kind = ("NORMAL", "GAMMA", "BINOMIAL", "MVNORMAL")[rng.integers(4)]
        count = int(10 ** rng.uniform(3, 8))
        f64 = bool(rng.integers(2))
        r = dict(t=t, client=int(rng.integers(nclients)), kind=kind, count=count, a=0.0, b=0.0, trials=0,
                 dtype=torch.float64 if f64 else torch.float32)
        if kind == "NORMAL":
            r.update(b=1.0)
        elif kind == "GAMMA":
            r.update(a=float(10 ** rng.uniform(-1, 1)), b=1.0)
        elif kind == "BINOMIAL":
            r.update(trials=int(rng.integers(1, 1001)), a=float(rng.uniform()), dtype=torch.int32)
        else:
            r.update(dtype=torch.float32)
        out.append(r)
    return out


def _pct(v, q):
    import numpy as np
    return float(np.percentile(np.asarray(v), q)) if v else None


def bench_serving(er, seconds=6.0, rates=(2000.0, 500.0), nclients=256, budget=40 << 30, slots=64, serial_cap=1.5):
    """Trace-driven serving runs (per arrival rate) against the serial
    plain-call path on the same trace."""
    import numpy as np
    import torch
    from eigenrand_gb300.serving import Server, now
    rng = np.random.default_rng(99)
    A = rng.standard_normal((64, 64))
    cov, mean = A @ A.T + 64 * np.eye(64), rng.standard_normal(64)
    seeds = [1000 + c for c in range(nclients)]
    out = {"config": {"clients": nclients, "trace_s": seconds, "budget_gb": budget / 2**30, "slots": slots,
                      "counts": "log-uniform [1e3, 1e8]",
                      "kinds": "normal, gamma(10^U(-1,1)), binomial(U{1..1000}, U(0,1)), MvNormal d=64; "
                               "f32/f64 half and half (MvNormal f32, binomial int32)",
                      "engines": "one Vmt19937_64(1000 + c) per client (single stream, bit-exact)"}}
    for rate in rates:
        trace = make_serving_trace(seconds, rate=rate, nclients=nclients)
        warm = make_serving_trace(0.5, rate=rate, nclients=nclients, seed=6)
        srv = Server(nclients, seeds, budget, slots=slots)
        srv.set_mvnormal(mean, cov)

        def replay(reqs):
            t0 = now()
            i, done, lat, nbytes, last = 0, 0, [], 0, t0
            while done < len(reqs):
                tn = now() - t0
                while i < len(reqs) and reqs[i]["t"] <= tn:
                    r = reqs[i]
                    srv.submit(r["client"], r["kind"], r["dtype"], r["count"], r["a"], r["b"], r["trials"],
                               arrival=t0 + r["t"])
                    i += 1
                comp = srv.progress()
                for c in comp:
                    srv.release(c["ticket"])
                    if c["status"] != 0:
                        raise RuntimeError(f"request failed: {c}")
                    lat.append(c["completed"] - c["arrival"])
                    nbytes += c["bytes"]
                    last = max(last, c["completed"])
                    done += 1
                if not comp:
                    time.sleep(20e-6)
            return lat, nbytes, last - t0

        replay(warm)
        lat, nbytes, span = replay(trace)
        served = {"requests": len(trace), "p50_ms": round(_pct(lat, 50) * 1e3, 2),
                  "p99_ms": round(_pct(lat, 99) * 1e3, 2), "mean_ms": round(float(np.mean(lat)) * 1e3, 2),
                  "span_s": round(span, 3), "gbs_out": round(nbytes / span / 1e9, 2),
                  "req_s": round(len(trace) / span, 1)}
        del srv
        torch.cuda.synchronize()
        # serial plain calls: one stream, arrival order, one call at a time on
        # the same per-client engines (fresh, same seeds); stops after
        # serial_cap x the trace duration and reports how far it got
        engines = [er.Vmt19937_64(s) for s in seeds]
        mv = [None] * nclients
        lat_s, nbytes_s, ndone = [], 0, 0
        st = torch.cuda.current_stream()
        t0 = now()
        for r in trace:
            while now() - t0 < r["t"]:
                time.sleep(20e-6)
            c = r["client"]
            if r["kind"] == "MVNORMAL":
                if mv[c] is None:
                    mv[c] = er.MvNormalGen(mean, cov)
                s = -(-r["count"] // 64)
                o = torch.empty((s, 64), dtype=torch.float32, device="cuda").t()
                mv[c].generate(engines[c], s, out=o)
            else:
                P = 8 if r["dtype"] == torch.float32 else 4
                n = -(-r["count"] // P) * P
                o = torch.empty((1, n), dtype=r["dtype"], device="cuda").t()
                er._sample(r["kind"], n, 1, engines[c], r["dtype"], r["a"], r["b"], r["trials"], out=o)
            st.synchronize()
            tdone = now()
            lat_s.append(tdone - (t0 + r["t"]))
            nbytes_s += o.numel() * o.element_size()
            ndone += 1
            del o
            if tdone - t0 > serial_cap * seconds:
                break
        span_s = now() - t0
        serial = {"requests_done": ndone, "of": len(trace), "p50_ms": round(_pct(lat_s, 50) * 1e3, 2),
                  "p99_ms": round(_pct(lat_s, 99) * 1e3, 2), "span_s": round(span_s, 3),
                  "gbs_out": round(nbytes_s / span_s / 1e9, 2), "req_s": round(ndone / span_s, 1),
                  "stopped_early": ndone < len(trace)}
        del engines, mv
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        out[f"rate_{int(rate)}"] = {"served": served, "serial_plain": serial}
    return out


# --------------------------------------------------------------------------- reference arm
def host_cpu():
    """ISA and model of the host cores that run the CPU baseline."""
    import platform
    info = {"isa": platform.machine(), "model": None}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            k, _, v = line.partition(":")
            if k.strip() == "Model name" and v.strip():
                info["model"] = v.strip()
    except (OSError, subprocess.SubprocessError):
        pass
    info["code"] = ("scalar C restatement of the reference's packet algorithms (oracle/), -O2, no SIMD "
                    "intrinsics: the reference's AVX2 / NEON packet code needs Eigen, which is absent")
    return info


def cpu_run(per_dist_samples, threads=1):
    """The reference's CPU path over a bounded sample of the sweep.  The
    reference needs Eigen, which is absent, so this runs its restatement
    (oracle/, the same packet algorithms, plain C).  threads > 1 is the
    one-engine-per-thread harness: thread k owns Vmt19937_64(1234 + 4k) and
    fills its slice.  Returns (samples, wall seconds)."""
    import numpy as np
    import pyoracle
    from concurrent.futures import ThreadPoolExecutor
    pyoracle.build()
    pyoracle.set_fp_math(True)  # FP64 log / exp, the reference's speed class on a CPU
    items = sweep_items()
    dt = {"f32": np.float32, "f64": np.float64, "i32": np.int32}
    per_thread = max(8, (per_dist_samples // threads) // 8 * 8)
    engines = [pyoracle.Engine(1234 + 4 * k) for k in range(threads)]

    def work(k):
        e = engines[k]
        for (name, kind, t, a, b, tr, w) in items:
            pyoracle.generate(e, pyoracle.Gen(), kind, per_thread, dt[t], a, b, tr, w)

    t0 = time.perf_counter()
    if threads == 1:
        work(0)
    else:
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(work, range(threads)))
    secs = time.perf_counter() - t0
    return per_thread * threads * len(items), secs


def cpu_baseline(seconds=15.0):
    threads = max(1, os.cpu_count() or 1)
    # calibrate on 2^14 samples per distribution per thread, then scale to ~seconds
    n0 = (1 << 14) * threads
    s0, t0 = cpu_run(n0, threads)
    n = int(n0 * max(1.0, seconds / max(t0, 1e-3)))
    s, t = cpu_run(n, threads)
    return {"value": round(s / t / 1e9, 5), "unit": "Gsamples/s", "cores": threads, "kind": "port",
            "cpu": host_cpu(),
            "sample": f"{s // len(sweep_items())} samples per distribution x {len(sweep_items())} distributions "
                      f"({t:.1f} s), {threads} threads each with its own Vmt19937_64(1234+4k); the reference needs "
                      "Eigen (absent), so its plain-C restatement in oracle/ runs, with the C library's FP64 "
                      "log / exp standing in for Eigen's plog / pexp"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    # each step: a bounded sample of the sweep on all host cores
    threads = max(1, os.cpu_count() or 1)
    n = (1 << 16) * threads
    cpu_run(1 << 12, threads)
    tot, secs = 0, 0.0
    for _ in range(args.warmup):
        cpu_run(n, threads)
    for _ in range(args.steps):
        s, t = cpu_run(n, threads)
        tot += s
        secs += t
    v = tot / secs / 1e9
    return {"metric": "Gsamples/s (univariate sweep, 4096x4096 per distribution)", "value": round(v, 5),
            "unit": "Gsamples/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(secs * 1e3 / args.steps, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64+i32", "data": "synthetic (engine seeded 1234)",
            "config": {"workload": "univariate sweep (same distributions), bounded sample: 2^16 samples per "
                                   "distribution per thread per step", "threads": threads},
            "impl": "reference",
            "cpu_baseline": {"value": round(v, 5), "unit": "Gsamples/s", "cores": threads, "kind": "port",
                             "cpu": host_cpu(),
                             "sample": f"2^16 samples per distribution per thread per step, {threads} threads, "
                                       "one Vmt19937_64(1234+4k) per thread; the reference needs Eigen (absent), "
                                       "so its restatement in oracle/ runs"},
            "e2e": {"value": round(v, 5), "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_case(args):
    """One named workload, repeated (small cases for profiler captures)."""
    import numpy as np
    import torch
    import eigenrand_gb300 as er
    name = args.case
    urng = er.Vmt19937_64(1234, streams=608)
    if name == "uniform_f32":
        out = torch.empty((4096, 4096), dtype=torch.float32, device="cuda")
        fn = lambda: er.uniformReal(4096, 4096, urng, out=out)
    elif name == "uniform_f32_big":  # 256 MiB output, twice the L2: DRAM traffic of the sweep's kernel
        out = torch.empty((8192, 8192), dtype=torch.float32, device="cuda")
        fn = lambda: er.uniformReal(8192, 8192, urng, out=out)
    elif name.startswith("mvnormal_d"):
        d = int(name[len("mvnormal_d"):])
        rng = np.random.default_rng(99)
        A = rng.standard_normal((d, d))
        g = er.MvNormalGen(rng.standard_normal(d), A @ A.T + d * np.eye(d))
        n = (1 << 28) // (4 * d)  # 256 MiB of output, twice the L2
        out = torch.empty((n, d), dtype=torch.float32, device="cuda").t()
        fn = lambda: g.generate(urng, n, out=out)
    elif name == "multinomial":
        g = er.MultinomialGen(1000, np.random.default_rng(99).dirichlet(np.ones(100)))
        n = 1 << 16
        out = torch.empty((n, 100), dtype=torch.int32, device="cuda").t()
        fn = lambda: g.generate(urng, n, out=out)
    elif name == "wishart_d32":
        rng = np.random.default_rng(99)
        A = rng.standard_normal((32, 32))
        g = er.WishartGen(40, A @ A.T + 32 * np.eye(32))
        n = 1 << 14
        out = torch.empty((32 * n, 32), dtype=torch.float32, device="cuda").t()
        fn = lambda: g.generate(urng, n, out=out)
    elif name in ("beta_f32", "beta_f64", "beta_f64_4096"):
        dt = torch.float32 if name == "beta_f32" else torch.float64
        g = er.BetaGen(0.5, 2.0, dtype=dt)
        side = 4096 if name.endswith("4096") else 2048  # 4096: the sweep's launch
        out = torch.empty((side, side), dtype=dt, device="cuda")
        fn = lambda: g.generate(side, side, urng, out=out)
    elif name in ("weibull_f64", "exponential_f64", "gamma05_f64", "normal_f64", "cauchy_f64"):  # 2048x2048 f64
        kind = {"weibull_f64": ("WEIBULL", 1.5, 1.0), "exponential_f64": ("EXPONENTIAL", 1.0, 0.0),
                "gamma05_f64": ("GAMMA", 0.5, 1.0), "normal_f64": ("NORMAL_STD", 0.0, 0.0),
                "cauchy_f64": ("CAUCHY", 0.0, 1.0)}[name]
        d, keep = er._desc(kind[0], torch.float64, kind[1], kind[2])
        out = torch.empty((2048, 2048), dtype=torch.float64, device="cuda")
        fn = lambda: er._lib.check(er._L.gr_sample(urng._h, er.ctypes.byref(d), er._ptr(out), out.numel(),
                                                   er._stream_ptr()))
    elif name == "binomial20":
        g = er.BinomialGen(20, 0.3)
        out = torch.empty((2048, 2048), dtype=torch.int32, device="cuda")
        fn = lambda: g.generate(2048, 2048, urng, out=out)
    elif name == "poisson4":
        g = er.PoissonGen(4.0)
        out = torch.empty((2048, 2048), dtype=torch.int32, device="cuda")
        fn = lambda: g.generate(2048, 2048, urng, out=out)
    elif name == "binomial_v":  # per-element binomial, trials 20 / 50 / 100 by column, p 0.5 / 0.01 / 0.75 by row
        idx = torch.arange(2048, device="cuda")
        tr = torch.tensor([20, 50, 100], dtype=torch.int32, device="cuda")[idx % 3][None, :].expand(2048, 2048)
        pr = torch.tensor([0.5, 0.01, 0.75], device="cuda")[idx % 3][:, None].expand(2048, 2048)
        tr, pr = tr.t().contiguous().t(), pr.t().contiguous().t()
        out = torch.empty_like(tr)
        fn = lambda: er.binomial(urng, tr, pr, out=out)
    elif name == "truncmvn_d9":  # TruncMvNormalGen, the reference tests' d = 9 case, 10^5 chains
        c = np.zeros((9, 9))
        c[0, 1], c[2, 7], c[3, 1] = 0.5, 0.5, 0.7
        c[np.diag_indices(9)] = [1, 1.2, 1.4, 1.6, 1.8, 1.6, 1.4, 1.2, 1]
        g = er.TruncMvNormalGen([-1, 0, 1, 2, 3, 2, 1, 0, -1], c @ c.T,
                                er.support([-4, -3, -2, -1, 0, -1, -2, -3, -4], [4, 5, 6, 7, 8, 7, 6, 5, 4]))
        out = torch.empty((100000, 9), dtype=torch.float32, device="cuda").t()
        fn = lambda: g.generate(urng, 100000, out=out)
    elif name == "multinomial_cond":  # conditional-binomial path, K = 10, trials = 1000
        g = er.MultinomialGen(1000, np.random.default_rng(99).dirichlet(np.ones(10)))
        n = 1 << 18
        out = torch.empty((n, 10), dtype=torch.int32, device="cuda").t()
        fn = lambda: g.generate(urng, n, out=out)
    elif name == "gamma_compat":
        u1 = er.Vmt19937_64(1234)
        g = er.GammaGen(0.5, 1.0)
        out = torch.empty((4096, 4096), dtype=torch.float32, device="cuda")
        fn = lambda: g.generate(4096, 4096, u1, out=out)
    else:
        raise SystemExit(f"unknown case {name}")
    ms = _median_ms(fn, reps=args.steps, warm=args.warmup)
    print(json.dumps({"case": name, "ms": round(ms, 4)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="streams", choices=["compat", "streams"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=6.0, help="length of each serving trace")
    ap.add_argument("--case", default=None,
                    help="run one named small workload instead (uniform_f32, uniform_f32_big, mvnormal_dD, multinomial, wishart_d32, "
                         "beta_f32, beta_f64, poisson4, gamma_compat), for profiler captures")
    ap.add_argument("--no-compat", action="store_true", help="skip the single-engine sweep (the 'compat' key)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched, multivariate and serving workloads (extra keys of the JSON line)")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    if world != args.gpus and "RANK" not in os.environ:
        world = 1
    res = run_reference(args, rank, world) if args.impl == "reference" else run_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
