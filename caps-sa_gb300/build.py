"""Build libcapssa_gb300.so from csrc/ with nvcc for sm_103a (GB300).

Each translation unit compiles in parallel; the objects link into one
shared library with the CUDA runtime linked statically, so the library
carries no dependency beyond the NVIDIA kernel driver.  Output: _build/ next to
this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcapssa_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
         "--expt-relaxed-constexpr", "-Xptxas", "-O3"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(SRC) if f.endswith(".cu"))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".cuh")]
    deps.append(os.path.join(HERE, "..", "include", "capssa.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    jobs = []
    for f in sources():
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f[:-3] + ".o")
        if force or _stale(obj, src):
            cmd = [cc, *ARCH, *FLAGS, *(extra or []), "-c", src, "-o", obj]
            jobs.append((f, cmd))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): f
                    for f, cmd in jobs}
            for fut in cf.as_completed(futs):
                r = fut.result()
                if verbose or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed on %s" % futs[fut])
    objs = [os.path.join(OUT, f[:-3] + ".o") for f in sources()]
    if jobs or not os.path.exists(LIB):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-cudart=static", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
