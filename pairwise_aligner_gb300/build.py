"""In-tree build of libpa_gb300.so for sm_103a (nvcc, no cmake)."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libpa_gb300.so")
SOURCES = ["pa_capi.cu", "pa_kern_v0.cu", "pa_kern_v1.cu", "pa_kern_v2.cu", "pa_kern_v3.cu", "pa_kern_v4.cu", "pa_kern_v5.cu", "pa_kern_v6.cu", "pa_kern_v7.cu", "pa_kern_v8.cu", "pa_kern_short_local.cu", "pa_kern_short_global.cu", "pa_kern_short_free.cu", "pa_kern_cta.cu", "pa_kern_cluster.cu", "pa_band_labels.cu", "pa_band.cu", "pa_band_dp.cu", "pa_static.cu", "pa_input.cu", "pa_traceback.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(REPO, "include", "pairwise_aligner_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile csrc/*.cu (in parallel) and link pairwise_aligner_gb300/libpa_gb300.so; skipped when up to date."""
    if not force and not _stale(LIB):
        return LIB
    objdir = os.path.join(HERE, "_build")
    os.makedirs(objdir, exist_ok=True)
    flags = [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-diag-suppress", "177"]
    if verbose:
        flags.append("-Xptxas=-v")
    procs, objs = [], []
    for src in SOURCES:
        obj = os.path.join(objdir, src.replace(".cu", f".{os.getpid()}.o"))
        objs.append(obj)
        cmd = [nvcc(), *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append(subprocess.Popen(cmd))
    try:
        failed = [p.args for p in procs if p.wait() != 0]
        if failed:
            raise RuntimeError(f"nvcc failed: {failed}")
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call([nvcc(), *ARCH, "-shared", "-o", tmp, *objs])
        os.replace(tmp, LIB)
    finally:
        for o in objs:
            if os.path.exists(o):
                os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
