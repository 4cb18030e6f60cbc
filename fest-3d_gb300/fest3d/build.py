"""Build recipe of the in-tree CUDA library (sm_103a only).

``build()`` compiles every ``csrc/*.cu`` with nvcc in parallel and links
``_build/libfest_gpu.so``.  No cmake; one -gencode; a minute at most.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OUT = os.path.join(ROOT, "_build")
LIB = os.path.join(OUT, "libfest_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def _nvcc():
    for c in ("nvcc", "/usr/local/cuda/bin/nvcc"):
        try:
            subprocess.run([c, "--version"], check=True, capture_output=True)
            return c
        except Exception:
            pass
    raise RuntimeError("nvcc not found")


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(x) > t for x in [src] + deps)


def build(verbose=False, extra_flags=()):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    deps = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [
        os.path.join(os.path.dirname(ROOT), "include", "fest_gpu.h")]
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _stale(o, s, deps):
            jobs.append([nvcc, "-c", s, "-o", o] + ARCH + FLAGS + list(extra_flags))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run([nvcc, "-shared", "-o", LIB] + objs + ARCH)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
