"""Autotuner for the tile shape and residency of the two NLCG passes.

The stencil tile is 32 sites wide with a one-site halo; its height (rows per
tile, hence the halo-to-interior ratio) and the minimum resident blocks per
SM requested from ptxas (hence the register budget) are compile-time
template parameters, and the FP32 passes exist in two designs: warp strips
(one warp per tile walking down its rows, neighbours by shuffles) and
shared-memory tiles (eight warps per tile, with variants of the halo copy).  The tuner builds one library
per candidate (in parallel, into a scratch directory), times the FP32 NLCG
step of a workload with each (CUDA events on the context's stream, after
warm-up), and writes the fastest candidate's definitions to
``mepgl_gb300/tuning.json``, which ``mepgl_gb300.build`` applies to every
later build.

    python -m mepgl_gb300.autotune [--workload string|sweep] [--out mepgl_gb300/tuning.json]

Workloads: ``string`` = the 256x256, 64-image two-component string;
``sweep`` = the 64 strings of the parameter sweep (uneven sizes, one
component).  ``--keep-selection`` records a workload's results beside the
others without changing the definitions the build applies.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys
import tempfile

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
TUNING = os.path.join(PKG, "tuning.json")

# Strip candidates: rows per tile, single-warp blocks per SM for the
# gradient and the direction pass (register budget 65536 / (32 x blocks)),
# row loop unrolled by the window period, unit-weight path for interior
# sites, packed FP32x2 stencils for two components, all steps of a call in
# one fused persistent launch, and its blocks per SM or explicit register cap.
STRIP = [(40, 16, 16, 0, 0, 1, 1, 12, 0), (32, 16, 16, 0, 0, 1, 1, 12, 0), (32, 16, 16, 0, 0, 1, 1, 16, 152), (32, 16, 16, 0, 0, 1, 1, 16, 144),
         (32, 16, 16, 0, 0, 1, 1, 16, 128), (32, 16, 16, 0, 0, 1, 0, 16, 0)]
# Tile candidates: rows per FP32 tile, min blocks per SM for the gradient
# pass, for the direction pass, gradient-pass halo copy (0 through
# registers, 1 cp.async), direction pass (0 fused, 1 split into a pointwise
# update + polynomial pass), fused direction pass halo copy (0 x by cp.async
# and g, d through registers, 1 all three by cp.async).
TILE = [(16, 4, 4, 0, 0, 0)]
CANDIDATES = [dict(MEPGL_STRIP=1, MEPGL_ROWS_F32=r, MEPGL_MINB_STRIP_GRAD=mg, MEPGL_MINB_STRIP_DIR=md,
                   MEPGL_STRIP_UNROLL=u, MEPGL_STRIP_INTERIOR=i, MEPGL_STRIP_PAIR=pk, MEPGL_STRIP_FUSED=fu,
                   MEPGL_MINB_STRIP_FUSED=mf, MEPGL_MAXREG_FUSED=mr) for r, mg, md, u, i, pk, fu, mf, mr in STRIP] + [
    dict(MEPGL_STRIP=0, MEPGL_ROWS_F32=r, MEPGL_MINB_GRAD=g, MEPGL_MINB_DIR=d, MEPGL_GRAD_ASYNC=a,
         MEPGL_SPLIT_DIR=sp, MEPGL_DIR_ASYNC=da) for r, g, d, a, sp, da in TILE]


def defines(c):
    return dict(c)


def _build(c, base):
    d = os.path.join(base, "_".join("%s%d" % (k.replace("MEPGL_", "").lower(), v) for k, v in sorted(c.items())))
    env = dict(os.environ, MEPGL_LIB_DIR=d,
               MEPGL_NVCC_FLAGS=" ".join("-D%s=%d" % kv for kv in defines(c).items()), MEPGL_NO_TUNING="1")
    r = subprocess.run([sys.executable, "-c", "from mepgl_gb300 import build; build.build(force=True)"], cwd=ROOT,
                       env=env, capture_output=True, text=True)
    return c, d, r.returncode, r.stderr[-2000:]


def measure(workload: str, steps: int = 20, warmup: int = 4):
    """ms per FP32 NLCG step of the workload with the library MEPGL_LIB points to."""
    import torch
    from . import native, workloads
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    if workload == "string":
        prob, st = workloads.config2()
        ctx = native.StringContext(prob, st.n_images, "fp32", stream=stream.cuda_stream,
                                   line_polynomial=native.POLY_EXACT)
        ctx.set_state(st)
    else:
        from .sweep import build_batch
        ctx, *_ = build_batch(64, stream=stream.cuda_stream)
    ctx.nlcg_steps(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.nlcg_steps(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", choices=("string", "sweep"), default="string")
    ap.add_argument("--out", default=TUNING)
    ap.add_argument("--measure", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--jobs", type=int, default=min(8, os.cpu_count() or 1))
    ap.add_argument("--keep-selection", action="store_true",
                    help="record this workload's results without changing the build's selection")
    a = ap.parse_args(argv)
    if a.measure:
        print(json.dumps({"ms_per_step": measure(a.workload)}))
        return
    base = tempfile.mkdtemp(prefix="mepgl_tune_")
    with cf.ThreadPoolExecutor(a.jobs) as ex:
        built = list(ex.map(lambda c: _build(c, base), CANDIDATES))
    results = []
    for c, d, rc, err in built:
        if rc != 0:
            results.append(dict(defines=defines(c), error=err.strip().splitlines()[-1:] or ["build failed"]))
            continue
        env = dict(os.environ, MEPGL_LIB=os.path.join(d, "libmepgl_gb300.so"))
        r = subprocess.run([sys.executable, "-m", "mepgl_gb300.autotune", "--measure", "--workload", a.workload],
                           cwd=ROOT, env=env, capture_output=True, text=True)
        if r.returncode != 0:
            results.append(dict(defines=defines(c), error=r.stderr.strip().splitlines()[-1:]))
            continue
        results.append(dict(defines=defines(c), ms_per_step=json.loads(r.stdout.strip().splitlines()[-1])["ms_per_step"]))
        print(json.dumps(results[-1]), flush=True)
    ok = [r for r in results if "ms_per_step" in r]
    if not ok:
        raise SystemExit("no candidate built and ran")
    best = min(ok, key=lambda r: r["ms_per_step"])
    try:
        import torch
        device = torch.cuda.get_device_name(0)
    except Exception:
        device = "unknown"
    doc = {}
    if os.path.exists(a.out):
        with open(a.out) as f:
            doc = json.load(f)
    doc.setdefault("by_workload", {})[a.workload] = dict(device=device, results=results, best=best["defines"])
    if not a.keep_selection or "selected" not in doc:
        doc["selected"] = best["defines"]
        doc["selected_by"] = a.workload
    with open(a.out, "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps({"selected": best["defines"], "ms_per_step": best["ms_per_step"]}))


if __name__ == "__main__":
    main()
