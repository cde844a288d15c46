"""Build libpytreegrav_gb300.so in-tree for sm_103a (GB300).

Each CUDA translation unit compiles in parallel with nvcc, then one shared library is linked. The
library depends only on the CUDA runtime, so it loads in any process (torch is not needed by the
library itself). Output: pytreegrav_gb300/_build/libpytreegrav_gb300.so (git-ignored).

    python -m pytreegrav_gb300.build [--force] [--verbose]
"""

import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libpytreegrav_gb300.so"
LIB = os.path.join(OUT_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc_path():
    cand = [shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pytreegrav_gb300")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = nvcc_path()
    srcs = sources()
    hdrs = headers()
    if not force and not _stale(LIB, srcs + hdrs + [__file__]):
        return LIB
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs + [__file__]):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-I", os.path.join(ROOT, "include"), "-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout.strip() or r.stderr.strip()):
            print(r.stdout + r.stderr, file=sys.stderr)
        return r

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    if verbose:
        print(" ".join(link), file=sys.stderr)
    subprocess.check_call(link)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
