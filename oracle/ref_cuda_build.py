"""Build and time the reference's own CUDA NLCG on this GPU (a timing baseline only).

The reference compiles its kernels for sm_61 with N, dx, the component count
and the precision fixed at compile time (mepgl/src/CMakeLists.txt:5-13,
mepgl/src/config.cuh), and its main() needs Boost.program_options.  This
recipe:

* ``stage()`` (where the reference tree is, $MEPGL_REFERENCE or a checkout
  named ``reference`` beside this repository): copies the unmodified
  nlcg.cu, parallel_sum.cu and their headers into
  ``baseline/_ref/cuda/src`` (git-ignored; nothing of the reference enters
  the repository);
* ``compile(n, dx, comps, prec)``: writes the generated config.cuh and
  real.cuh of that variant and compiles the staged sources for sm_103a
  together with ``oracle/ref_cuda_driver.cu`` (a plain input reader and
  timer in place of the reference's main);
* ``run(prob, state, prec, steps, warmup)``: writes the input file, runs the
  variant and returns its JSON line (ms per NLCG step, site-image/s and the
  energies after the steps).

The reference's own nlcgSteps host loop runs unchanged: twelve kernel
launches, four two-level sums with per-call cudaMalloc/cudaFree and host
synchronisations per step (mepgl/src/nlcg.cu:1462-1586).
"""
from __future__ import annotations

import json
import os
import shutil
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BASE = os.path.join(ROOT, "baseline", "_ref", "cuda")
SRC = os.path.join(BASE, "src")
FILES = ("nlcg.cu", "nlcg.cuh", "parallel_sum.cu", "parallel_sum.cuh", "cuda_errors.cuh")


def reference_src() -> str:
    root = os.environ.get("MEPGL_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
    return os.path.join(root, "mepgl", "src")


def staged() -> bool:
    return all(os.path.isfile(os.path.join(SRC, f)) for f in FILES)


def stage() -> bool:
    """Copy the reference's NLCG sources into baseline/_ref/cuda/src; False if absent."""
    src = reference_src()
    if not all(os.path.isfile(os.path.join(src, f)) for f in FILES):
        return staged()
    os.makedirs(SRC, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(src, f), os.path.join(SRC, f))
    return True


def variant_dir(n: int, dx: float, comps: int, prec: str) -> str:
    return os.path.join(BASE, f"N{n}_dx{dx!r}_C{comps}_{prec}")


def _config_cuh(n: int, dx: float, comps: int, prec: str) -> str:
    """config.cuh as the reference's header generator writes it
    (mepgl/mepgl_lib/launcher_utils.py:84-110): 512 threads per block in FP64,
    1024 in FP32."""
    lines = ["#ifndef CONFIG_CUH", "#define CONFIG_CUH", '#include <string>', '#include "real.cuh"',
             "const int devNumber = 0;"]
    if comps == 2:
        lines.append("#define MULTICOMPONENT")
    lines += [f"constexpr int N = {n};", f"constexpr int blockSizeX = {512 if prec == 'f64' else 1024};",
              "constexpr int gridSizeX = (int)((N*N)/blockSizeX + 1);", f"constexpr real dx = {dx!r};",
              "constexpr int default_relaxation_step_number = 10;", "#endif"]
    return "\n".join(lines) + "\n"


def compile(n: int, dx: float, comps: int, prec: str) -> str:
    """Compile one variant (sm_103a) and return the path of its binary.

    FP32 variants get -maxrregcount=64: nvcc 13 gives the reference's
    heaviest kernel 68 registers for sm_103a, and its 1024-thread blocks
    (above) then need more than the 65,536 registers of an SM, so the launch
    fails -- silently, since the reference checks no launch (the sm_61 build
    it was written for fits in 64).  The sources are unchanged."""
    from oracle.ref_build import _real_cuh
    if not staged():
        raise FileNotFoundError("reference CUDA sources not staged (oracle.ref_cuda_build.stage())")
    d = variant_dir(n, dx, comps, prec)
    exe = os.path.join(d, "ref_nlcg")
    drv = os.path.join(HERE, "ref_cuda_driver.cu")
    srcs = [os.path.join(SRC, "nlcg.cu"), os.path.join(SRC, "parallel_sum.cu"), drv]
    os.makedirs(d, exist_ok=True)
    for name, text in (("config.cuh", _config_cuh(n, dx, comps, prec)), ("real.cuh", _real_cuh(prec))):
        path = os.path.join(d, name)
        if not os.path.isfile(path) or open(path).read() != text:
            with open(path, "w") as f:
                f.write(text)
    deps = srcs + [os.path.join(d, "config.cuh"), os.path.join(d, "real.cuh"), os.path.abspath(__file__)]
    if os.path.isfile(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(s) for s in deps):
        return exe
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w", "-I", d, "-I", SRC, "-o", exe + ".tmp"]
    if prec != "f64":
        cmd += ["-maxrregcount=64"]
    r = subprocess.run(cmd + srcs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference CUDA build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(exe + ".tmp", exe)
    return exe


def write_input(path: str, prob, state, prec: str) -> None:
    """The driver's binary input: header, masks, parameters, couplings, fields."""
    from mepgl_gb300.problem import PARAM_NAMES
    dt = np.float64 if prec == "f64" else np.float32
    n, F = prob.nx, state.n_images
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", F, n))
        f.write(np.ascontiguousarray(prob.comp_domain, np.int32).tobytes())
        f.write(np.ascontiguousarray(prob.sc_domain, np.int32).tobytes())
        for name in PARAM_NAMES:
            f.write(np.ascontiguousarray(getattr(prob, name), dt).tobytes())
        f.write(np.array([prob.q_1, prob.q_2, prob.eta, prob.gamma, prob.delta], dt).tobytes())
        p2 = state.psi_2 if state.psi_2 is not None else np.zeros_like(state.psi_1)
        for arr in (state.a, state.psi_1, p2):
            f.write(np.ascontiguousarray(arr, dt).tobytes())


def run(prob, state, prec: str, steps: int, warmup: int, workdir: str | None = None, timeout: float = 600) -> dict:
    """Compile (if needed) and run the reference build on one workload."""
    if prob.nx != prob.ny:
        raise ValueError("the reference lattice is square")
    exe = compile(prob.nx, prob.dx, prob.ncomp, prec)
    workdir = workdir or os.path.dirname(exe)
    path = os.path.join(workdir, "input.bin")
    write_input(path, prob, state, prec)
    r = subprocess.run([exe, path, str(steps), str(warmup)], capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference CUDA run failed ({r.returncode}): {r.stderr[-2000:]}")
    out = json.loads(r.stdout.strip().splitlines()[-1])
    if out.get("launch_error"):
        raise RuntimeError(f"reference CUDA kernels failed to launch: {out['launch_error']}")
    return out


if __name__ == "__main__":
    print("staged" if stage() else "reference sources not found")
