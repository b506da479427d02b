"""Build recipe of the native parts: libmepgl_gb300.so and the ``mepgl`` CLI.

Compiles the CUDA sources for sm_103a only (one ``-gencode``), translation
units in parallel, into ``mepgl_gb300/_lib/`` (in-tree, git-ignored).  No
cmake; ``nvcc`` and ``g++`` are invoked directly.
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
# MEPGL_LIB_DIR / MEPGL_NVCC_FLAGS: build a variant elsewhere with extra flags
LIB_DIR = os.environ.get("MEPGL_LIB_DIR", os.path.join(PKG, "_lib"))
LIB = os.path.join(LIB_DIR, "libmepgl_gb300.so")
CLI = os.path.join(LIB_DIR, "mepgl")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Werror=return-type",
              "--diag-error=940", "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CU_SOURCES = ["kernels.cu", "api.cu", "refine.cu"]
HEADERS = ["common.cuh", "site_ops.cuh", "site_pair.cuh", "kernels.cuh", "strip.cuh", "pair_float.cuh", "context.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


TUNING = os.path.join(PKG, "tuning.json")


def tuned_flags() -> list:
    """-D definitions chosen by mepgl_gb300.autotune (tuning.json), unless
    MEPGL_NO_TUNING is set; MEPGL_NVCC_FLAGS given later on the command line wins."""
    if os.environ.get("MEPGL_NO_TUNING") or not os.path.exists(TUNING):
        return []
    with open(TUNING) as f:
        sel = json.load(f).get("selected", {})
    return ["-D%s=%d" % (k, int(v)) for k, v in sorted(sel.items())]


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "mepgl.h")]
    if os.path.exists(TUNING):
        hdrs.append(TUNING)
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(LIB_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or ptxas_info or _stale(o, [s] + hdrs):
            extra = tuned_flags() + os.environ.get("MEPGL_NVCC_FLAGS", "").split()
            cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", s, "-o", o]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose or ptxas_info:
                sys.stdout.write(out)
    if jobs or _stale(LIB, objs):
        tmp = LIB + f".{os.getpid()}.tmp"
        _run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-ldl"])
        os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "cli.cpp")
    npy_src = os.path.join(CSRC, "npy.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, npy_src, LIB, os.path.join(CSRC, "npy.h")])):
        tmp = CLI + f".{os.getpid()}.tmp"
        _run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-pthread", "-o", tmp, cli_src, npy_src,
              "-I", os.path.join(ROOT, "include"), "-L", LIB_DIR, "-lmepgl_gb300", "-Wl,-rpath,$ORIGIN"])
        os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
