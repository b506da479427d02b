#!/usr/bin/env python3
"""Build recipe for ``oracle/_ref``: the reference's own kernels, host-compiled.

Test infrastructure only.  The reference engine (maiani/mepgl) is CUDA C++
whose lattice size ``N`` and spacing ``dx`` are compile-time constants
(mepgl/src/config.cuh:23,32, generated by mepgl/mepgl_lib/launcher_utils.py:
14-125).  Its ``__global__`` kernels are plain C++ bodies, so they compile for
the host once the CUDA language extensions are stubbed (``ref_shim.h``) and the
``__host__`` wrapper functions -- the only code holding ``<<<...>>>`` launches
or cuSPARSE calls -- are left out.  ``ref_driver.cpp`` then emulates each
launch serially and restates the host-side call sequence.

For every variant (N, dx, components, precision, thin film) this script
compiles, in a temporary directory that is removed afterwards:

* ``real.cuh`` / ``config.cuh`` -- the two headers the reference generates per
  run, written here from the variant;
* ``nlcg_kernels.inc`` / ``interp_kernels.inc`` -- the kernels of
  mepgl/src/nlcg.cu and mepgl/src/interpolation.cu with ``#include`` lines and
  ``__host__`` functions removed, read from the reference tree at build time;

and writes ``oracle/_ref/<tag>/libref.so`` -- ``ref_driver.cpp`` compiled
against them -- and nothing else: no reference text is kept in or shipped
with the repository.

The FP64 variants do not define ``DOUBLE_PRECISION``; the reference compiles
its cubic spline only without that macro (interpolation.cu:359,483), and this
keeps the spline kernels available in double for the oracle.  Nothing else in
the kernels depends on the macro.

Usage: ``python oracle/ref_build.py N DX C PREC [--film]``; the Python helper
``oracle.refkernels.load_ref`` calls it on demand.  Requires the reference
tree at ``$MEPGL_REFERENCE``; without it, a checkout named ``reference``
beside this repository's directory (``<repo>/../reference``) is used.
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("MEPGL_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
REF_SRC = os.path.join(REF_ROOT, "mepgl", "src")
OUT_ROOT = os.path.join(HERE, "_ref")


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REF_SRC, "nlcg.cu"))


def variant_tag(n: int, dx: float, comps: int, prec: str, film: bool) -> str:
    return f"N{n}_dx{dx!r}_C{comps}_{prec}_{'film' if film else 'bulk'}"


def _strip_host_functions(text: str) -> str:
    """Remove every function introduced by ``__host__`` (signature and body).

    Braces are matched with comments and string literals skipped.
    """
    out = []
    i = 0
    n = len(text)
    pat = re.compile(r"^[ \t]*__host__\b", re.M)
    while True:
        m = pat.search(text, i)
        if not m:
            out.append(text[i:])
            break
        out.append(text[i:m.start()])
        j = text.index("{", m.end())
        depth = 0
        k = j
        while k < n:
            c = text[k]
            if text.startswith("//", k):
                k = text.index("\n", k)
                continue
            if text.startswith("/*", k):
                k = text.index("*/", k) + 2
                continue
            if c == '"':
                k += 1
                while text[k] != '"':
                    k += 2 if text[k] == "\\" else 1
                k += 1
                continue
            if c == "'":
                k += 1
                while text[k] != "'":
                    k += 2 if text[k] == "\\" else 1
                k += 1
                continue
            if c == "{":
                depth += 1
            elif c == "}":
                depth -= 1
                if depth == 0:
                    k += 1
                    break
            k += 1
        i = k
    return "".join(out)


def _strip_includes(text: str) -> str:
    return re.sub(r"^[ \t]*#include[^\n]*\n", "", text, flags=re.M)


def _real_cuh(prec: str) -> str:
    t, t2, t4 = ("double", "double2", "double4") if prec == "f64" else ("float", "float2", "float4")
    return (
        "#ifndef REAL_CUH\n#define REAL_CUH\n"
        f"typedef {t} real;\ntypedef {t2} real2;\ntypedef {t4} real4;\n"
        "#endif\n"
    )


def _config_cuh(n: int, dx: float, comps: int, film: bool) -> str:
    lines = [
        "#ifndef CONFIG_CUH", "#define CONFIG_CUH", '#include "real.cuh"',
        "const int devNumber = 0;",
    ]
    if comps == 2:
        lines.append("#define MULTICOMPONENT")
    if film:
        lines.append("#define NO_SELF_FIELD")
    lines += [
        f"constexpr int N = {n};",
        "constexpr int blockSizeX = 1024;",
        "constexpr int gridSizeX = (int)((N*N)/blockSizeX + 1);",
        f"constexpr real dx = {dx!r};",
        "constexpr int default_relaxation_step_number = 10;",
        "#endif",
    ]
    return "\n".join(lines) + "\n"


def build(n: int, dx: float, comps: int, prec: str, film: bool, force: bool = False) -> str:
    """Build (if needed) and return the path of the variant's ``libref.so``."""
    tag = variant_tag(n, dx, comps, prec, film)
    d = os.path.join(OUT_ROOT, tag)
    lib = os.path.join(d, "libref.so")
    if os.path.isfile(lib) and not force:
        return lib
    if not reference_available():
        raise FileNotFoundError(f"reference sources not found under {REF_SRC}")
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(REF_SRC, "nlcg.cu")) as f:
        nlcg = f.read()
    with open(os.path.join(REF_SRC, "interpolation.cu")) as f:
        interp = f.read()
    files = {
        "real.cuh": _real_cuh(prec),
        "config.cuh": _config_cuh(n, dx, comps, film),
        "nlcg_kernels.inc": _strip_includes(_strip_host_functions(nlcg)),
        "interp_kernels.inc": _strip_includes(_strip_host_functions(interp)),
    }
    # the filtered kernel text lives only in a temporary directory for the
    # compile; the variant directory keeps the library alone
    with tempfile.TemporaryDirectory(prefix="mepgl_ref_") as tmp:
        for name, body in files.items():
            with open(os.path.join(tmp, name), "w") as f:
                f.write(body)
        cmd = [
            os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
            "-w", "-I", tmp, "-I", HERE, "-include", os.path.join(HERE, "ref_shim.h"),
            os.path.join(HERE, "ref_driver.cpp"), "-o", lib + ".tmp",
        ]
        subprocess.run(cmd, check=True)
    os.replace(lib + ".tmp", lib)
    return lib


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("N", type=int)
    ap.add_argument("dx", type=float)
    ap.add_argument("C", type=int, choices=(1, 2))
    ap.add_argument("prec", choices=("f32", "f64"))
    ap.add_argument("--film", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    print(build(a.N, a.dx, a.C, a.prec, a.film, a.force))
    return 0


if __name__ == "__main__":
    sys.exit(main())
