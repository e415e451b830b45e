"""Compile the hicops_gb300 C ABI library (libhicops_gb300.so) for sm_103a.

Each translation unit is compiled in parallel; the result lives in
hicops_gb300/_build/ (git-ignored). Run: python -m hicops_gb300.build
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libhicops_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU = ["hc_index.cu", "hc_query.cu", "hc_mlp.cu", "hc_noalloc.cu", "hc_output.cu", "hc_ms2.cu"]
CPP = ["hc_api.cpp", "hc_host.cpp", "hc_batch.cpp", "hc_stream.cpp", "hc_store.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cmds(verbose_ptxas: bool = False):
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    cmds = []
    for f in CU:
        o = os.path.join(OUT, f + ".o")
        c = [nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
             *inc, "-c", os.path.join(CSRC, f), "-o", o]
        if verbose_ptxas:
            c.insert(3, "-Xptxas=-v")
        cmds.append((o, c, os.path.join(CSRC, f)))
    for f in CPP:
        o = os.path.join(OUT, f + ".o")
        c = [nvcc(), "-O2", "-std=c++17", "-x", "c++", "-Xcompiler", "-fPIC,-ffp-contract=off",
             *inc, "-c", os.path.join(CSRC, f), "-o", o]
        cmds.append((o, c, os.path.join(CSRC, f)))
    return cmds


def _stale(o: str, src: str) -> bool:
    if not os.path.exists(o):
        return True
    deps = [src, os.path.join(ROOT, "include", "hicops_gb300.h")]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return any(os.path.getmtime(d) > os.path.getmtime(o) for d in deps if os.path.exists(d))


def build(force: bool = False, verbose_ptxas: bool = False, quiet: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    jobs = [(o, c) for o, c, src in _cmds(verbose_ptxas) if force or verbose_ptxas or _stale(o, src)]
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = {ex.submit(subprocess.run, c, capture_output=True, text=True): o for o, c in jobs}
            for fu in cf.as_completed(futs):
                r = fu.result()
                if r.returncode != 0:
                    raise RuntimeError(f"compile failed: {' '.join(r.args)}\n{r.stderr}")
                if verbose_ptxas or (r.stderr.strip() and not quiet):
                    sys.stderr.write(r.stderr)
    objs = [o for o, _, _ in _cmds()]
    if jobs or not os.path.exists(LIB):
        r = subprocess.run([nvcc(), ARCH, "-shared", "-o", LIB, *objs, "-lpthread"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
