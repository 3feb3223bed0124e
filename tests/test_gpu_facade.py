"""The Eigen::Rand C++ facade (include/gpurand/EigenRand.hpp), called from a
C++ program the way EigenRand code is written, against the CPU oracle.

tests/cpp/facade_check.cpp is compiled with g++ against the facade and
libgpurand.so, run on the GPU, and its results are read back: bit-exact for
the univariate free functions and generator objects (consecutive calls on
one engine, caches carried by generator objects, P8_mt19937_64 as the Urng)
and the multinomial; the multivariate normal within the FP64-error bound of
test_gpu_mv.py (1e-5 of |L||Z| + |mean|).  A non-finite weight surfaces as a
C++ exception.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def read_records(path):
    recs = {}
    with open(path, "rb") as f:
        data = f.read()
    o = 0
    while o < len(data):
        (ln,) = struct.unpack_from("<I", data, o)
        o += 4
        name = data[o:o + ln].decode()
        o += ln
        dt, n = struct.unpack_from("<IQ", data, o)
        o += 12
        npdt = {0: np.float32, 1: np.float64, 2: np.int32}[dt]
        size = np.dtype(npdt).itemsize * n
        recs[name] = np.frombuffer(data[o:o + size], dtype=npdt).copy()
        o += size
    return recs


@pytest.fixture(scope="module")
def facade_results(gpulib, tmp_path_factory):
    lib_dir = os.path.dirname(gpulib._lib.LIB_PATH)
    d = tmp_path_factory.mktemp("facade")
    exe = str(d / "facade_check")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "cpp", "facade_check.cpp"),
           "-L" + lib_dir, "-lgpurand", "-L" + os.path.join(CUDA, "lib64"), "-lcudart",
           "-Wl,-rpath," + lib_dir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = str(d / "results.bin")
    r = subprocess.run([exe, out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return read_records(out)


def bits(a):
    return a.view(np.uint64 if a.itemsize == 8 else np.uint32)


def test_free_functions_on_one_engine(facade_results, oracle):
    r = facade_results
    e = oracle.Engine(42)
    cases = [("normal_f32", "NORMAL_STD", 1 << 20, np.float32, 0.0, 0.0, 0, None),
             ("uniformReal_f32", "UNIFORM_REAL", 64 * 32, np.float32, 0.0, 0.0, 0, None),
             ("normal2_f64", "NORMAL", 128 * 64, np.float64, 0.5, 2.0, 0, None),
             ("gamma05_f64", "GAMMA", 128 * 64, np.float64, 0.5, 1.0, 0, None),
             ("poisson4_i32", "POISSON", 256 * 64, np.int32, 4.0, 0.0, 0, None),
             ("binomial20_i32", "BINOMIAL", 256 * 64, np.int32, 0.3, 0.0, 20, None),
             ("discrete6_i32", "DISCRETE", 64 * 64, np.int32, 0.0, 0.0, 0, [1, 2, 3, 4, 5, 6]),
             ("beta_f32", "BETA", 64 * 64, np.float32, 0.5, 2.0, 0, None)]
    for name, kind, n, dt, a, b, t, w in cases:
        ref = oracle.generate(e, oracle.Gen(), kind, n, dt, a, b, t, w)
        got = r[name]
        assert got.size == n, name
        assert np.array_equal(bits(got), bits(ref)), f"{name}: {np.count_nonzero(bits(got) != bits(ref))} differ"


def test_generator_objects_keep_caches(facade_results, oracle):
    r = facade_results
    e = oracle.Engine(7)
    g = oracle.Gen()
    for name, n in (("normalgen_a", 12), ("normalgen_b", 20)):
        ref = oracle.generate(e, g, "NORMAL", n, np.float64, 1.0, 3.0)
        assert np.array_equal(bits(r[name]), bits(ref)), name
    g = oracle.Gen()
    for name in ("gammagen_a", "gammagen_b"):
        ref = oracle.generate(e, g, "GAMMA", 40, np.float32, 0.5, 1.0)
        assert np.array_equal(bits(r[name]), bits(ref)), name


def test_p8_engine_as_urng(facade_results, oracle):
    r = facade_results
    se = oracle.ScalarEngine("p8", 42)
    g = oracle.Gen()
    ref = se.generate(g, "BALANCED", 64, np.float32)
    assert np.array_equal(bits(r["p8_balanced_f32"]), bits(ref))
    ref = se.generate(g, "UNIFORM_REAL", 64, np.float32)
    assert np.array_equal(bits(r["p8_uniformReal_f32"]), bits(ref))


def test_multivariate(facade_results, oracle):
    r = facade_results
    mean = np.array([0.0, 1.0, -1.0, 2.0])
    cov = np.array([4.0, 1.0, 0.5, 0.0, 1.0, 3.0, 0.2, 0.1, 0.5, 0.2, 2.0, 0.3, 0.0, 0.1, 0.3, 1.0]).reshape(4, 4)
    e = oracle.Engine(99)
    d, n = 4, 1024
    z = oracle.generate(e, oracle.Gen(), "NORMAL_STD", d * n, np.float32).astype(np.float64).reshape(n, d).T
    L64 = oracle.get_lt(cov.T)  # the facade passes the matrix column-major
    x64 = oracle.mvnormal_f64(L64, z, mean)
    x = r["mvnormal_f32"].astype(np.float64).reshape(n, d).T
    scale = np.abs(L64) @ np.abs(z) + np.abs(mean)[:, None]
    assert np.max(np.abs(x - x64) / scale) <= 1e-5
    ref = oracle.multinomial(e, oracle.Gen(), [0.1, 0.2, 0.3, 0.4], 20, 64)
    got = r["multinomial_i32"].reshape(64, 4)
    assert np.array_equal(got, ref)


def test_errors_are_exceptions(facade_results):
    assert facade_results["nan_weight_threw"][0] == 1
