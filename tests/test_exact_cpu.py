"""Division-free forms of the reference's floating-point quotients (gr_exact.h),
checked exhaustively on the CPU against the IEEE division they replace."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exact_integer_forms(tmp_path):
    exe = tmp_path / "exact_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "eigenrand_gb300", "csrc"), "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "exact_check.cpp")], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0 of 2^31" in r.stdout
    assert "one_minus_ur_d mismatches 0 of" in r.stdout
    assert "untemper mismatches 0" in r.stdout
    assert "untwist mismatches 0" in r.stdout


def _has_avx2():
    import platform
    if platform.machine() not in ("x86_64", "AMD64"):
        return False
    try:
        return "avx2" in open("/proc/cpuinfo").read()
    except OSError:
        return False


@pytest.mark.skipif(not _has_avx2(), reason="pins GCC's x86-64 AVX2 build of the reference")
def test_scalar_engine_rawbits_order_pinned(tmp_path, oracle):
    """GCC evaluates the set intrinsics' draw arguments right to left, and
    rawbits_34's words, built with the real intrinsics from std::mt19937_64,
    give the oracle's scalar-engine float uniforms bit for bit."""
    import numpy as np
    exe = tmp_path / "rawbits_order"
    subprocess.run(["g++", "-O2", "-mavx2", "-std=c++17", "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "rawbits_order.cpp")], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    lines = dict(ln.split(" ", 1) for ln in r.stdout.strip().splitlines())
    assert lines["set_epi64x"] == "1 2 3 4"
    assert lines["setr_epi64x"] == "3 2 1 0"
    assert lines["mm_set_epi64x"] == "1 2"
    words = np.array([int(v) for v in lines["rawbits_34"].split()], dtype=np.uint32)
    ref = ((words & 0x7FFFFF) | (127 << 23)).view(np.float32) - np.float32(1)
    got = oracle.ScalarEngine("mt19937_64", 42).generate(oracle.Gen(), "UNIFORM_REAL", 32, np.float32)
    np.testing.assert_array_equal(got, ref)
