"""
Build of the CUDA library libatomistica_gb300.so (sm_103a only) with nvcc.

Each .cu translation unit is compiled in parallel, then linked into a shared
library that exposes the C-ABI of include/atomistica_gb300.h.  Output lands
next to this file (git-ignored).
"""

import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libatomistica_gb300.so")
SOURCES = ["core.cu", "bop.cu", "eam.cu", "api.cu", "diag.cu", "batch.cu",
           "autodiff.cu", "workload.cu"]
HEADERS = ["internal.h", "potential.h", "bop_math.h", "ff.h", "ff_tables.h", "bop_mixed.cuh",
           "elements.h",
           "bop_scr.cuh",
           "batch.h"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without FP contraction so that the cell inverse, the
# binning set-up and the spline tables are bit-identical on x86 and Arm hosts.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-diag-suppress", "1444",
              "-I" + os.path.join(ROOT, "include")]


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
    """Compile (if needed) and return the path of libatomistica_gb300.so.

    Extra nvcc flags (e.g. -D tuning macros) may be given in the environment
    variable GB_NVCC_FLAGS; changing them needs force=True."""
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + \
        [os.path.join(ROOT, "include", "atomistica_gb300.h")]
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + os.environ.get("GB_NVCC_FLAGS", "").split() +
                        ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for err in ex.map(run, jobs):
            if verbose and err.strip():
                print(err, file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
