"""Builds libtkknn.so in-tree: every CUDA source for sm_103a with nvcc, the
host tree builder with g++, compiled in parallel and linked into one shared
library next to this file.  Re-running only recompiles what changed."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(HERE, "libtkknn.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libtkknn.so")


def _headers():
    out = [os.path.join(ROOT, "include", "tk_knn.h")]
    for f in os.listdir(CSRC):
        if f.endswith((".h", ".cuh", ".inc")):
            out.append(os.path.join(CSRC, f))
    return out


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _headers()
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    cmds = []
    objs = []
    for f in srcs:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if not _stale(obj, [src] + hdrs):
            continue
        if f.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
                   "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
        else:
            # -O3 vectorises the CPU search's distance loops; without -ffast-math
            # every lane rounds each operation as the scalar code does
            cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
                   "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
        cmds.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    if cmds:
        with ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
            for err in ex.map(run, cmds):
                if verbose and err.strip():
                    print(err, file=sys.stderr)
    if _stale(LIB, objs):
        tmp = LIB + ".tmp"
        run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
