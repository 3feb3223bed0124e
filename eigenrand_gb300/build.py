"""Build libgpurand.so (the C-ABI sampling library) in-tree for sm_103a.

    python eigenrand_gb300/build.py          # incremental
    python eigenrand_gb300/build.py --force  # rebuild everything

Translation units are compiled in parallel with nvcc and linked into
eigenrand_gb300/_build/libgpurand.so.  The kernels are compiled with
--fmad=false: every multiply and add rounds on its own unless the source asks
for a fused multiply-add, which keeps the sample values reproducible on the
host.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgpurand.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off"]
SOURCES = ["gr_kernels.cu", "gr_samplers.cu", "gr_vop.cu", "gr_mv.cu", "gr_api.cu", "gr_mvapi.cu", "gr_serve.cu",
           "gr_noalloc.cu", "gr_trunc.cu", "gr_umma.cu", "gr_mncond.cu", "gr_tmvn.cu", "gr_binomv.cu",
           "gr_poly.cpp"]
HEADERS = ["gr_exact.h", "gr_internal.h", "gr_kernels.cuh", "gr_math.cuh", "gr_math_tables.h", "gr_mt.cuh", "gr_mv.cuh", "gr_admit.h", "gr_poly.h"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "gpurand.h")]
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + hdrs):
            cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", path, "-o", obj]
            if src.endswith(".cpp"):
                cmd = [nvcc, "-x", "cu"] + ARCH + NVCC_FLAGS + ["-c", path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "static", "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
