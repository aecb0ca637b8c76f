"""Build of libdyfox_gb300.so: every CUDA unit of ``csrc/`` compiled for
sm_103a with nvcc (one process per unit, in parallel) and linked in-tree.

    python -m dyfox_gb300.build [--force]
"""

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdyfox_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr",
              # a declaration hiding an outer variable is an error (device
              # and host code)
              "-Xcudafe", "--diag_error=1348"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required")


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile and link; returns the library path.  Incremental unless
    ``force``."""
    os.makedirs(OBJ, exist_ok=True)
    units = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    heads = _headers()
    cc = nvcc()
    jobs = []
    for u in units:
        o = os.path.join(OBJ, os.path.basename(u)[:-3] + ".o")
        if force or _stale(o, [u] + heads):
            jobs.append((u, o))

    def compile_one(job):
        u, o = job
        cmd = [cc, *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", u, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return u, r

    failed = []
    if jobs:
        workers = min(len(jobs), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(workers) as ex:
            for u, r in ex.map(compile_one, jobs):
                if verbose or r.returncode:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode:
                    failed.append(os.path.basename(u))
    if failed:
        raise RuntimeError(f"nvcc failed on {failed}")
    objs = [os.path.join(OBJ, os.path.basename(u)[:-3] + ".o") for u in units]
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        subprocess.check_call([cc, *ARCH, "-shared", "-o", tmp, *objs,
                               "-lcudart"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
