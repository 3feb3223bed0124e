"""Division-free forms of the reference's floating-point quotients (gr_exact.h),
checked exhaustively on the CPU against the IEEE division they replace."""
import os
import subprocess

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
