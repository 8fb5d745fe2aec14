"""Operator-apply bandwidth sweep over the polynomial degree.

    python -m schrodingersem_gb300.apply_sweep [--nodes 2e7] [--p 2-16] [--prec fp32,fp64]

For each degree p an n x n jittered mesh of [-12,12]^2 with
n = round(sqrt(nodes)/p) (about ``nodes`` global nodes) runs the
standalone Schroedinger Res apply (element kernel plus assembly into the
masked format) with L2 flushed before every apply.  Algorithmic bytes per
apply: n_loc * s * 9 (psi in 2 planes, out 2, g11 g12 g22 mass, V; s = 8
or 4); assembly traffic is not counted.  One JSON line per (p, precision)
with the time, GB/s and the fraction of the measured copy bandwidth.
"""
from __future__ import annotations

import argparse
import json
import math
import os

import numpy as np

HBM_FALLBACK_GBS = 6800.0


def hbm_peak():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    try:
        with open(os.path.join(root, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        for k in ("hbm_gbs", "hbm_GBs", "hbm"):
            if k in d:
                v = d[k]
                return float(v["value"] if isinstance(v, dict) else v), "measured"
    except Exception:
        pass
    return HBM_FALLBACK_GBS, "fallback"


def degrees(spec: str):
    out = []
    for part in spec.split(","):
        if "-" in part:
            a, b = part.split("-")
            out += list(range(int(a), int(b) + 1))
        else:
            out.append(int(part))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nodes", type=float, default=2e7)
    ap.add_argument("--p", default="2-16")
    ap.add_argument("--prec", default="fp32,fp64")
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--pipeline", type=int, default=1, help="1: bulk-copy pipelined kernel, 0: one-pass kernel")
    a = ap.parse_args()
    import torch

    import schrodingersem_gb300 as S
    from schrodingersem_gb300.meshgen import structured_quads
    S.build()
    peak, src = hbm_peak()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for p in degrees(a.p):
        n = max(2, int(round(math.sqrt(a.nodes) / p)))
        co, el = structured_quads(n, box=(-12.0, 12.0, -12.0, 12.0), jitter=0.1, seed=1)
        ctx = S.Context(p, coords=co, elements=el)
        from schrodingersem_gb300 import capi
        ctx.set_option(capi.OPT_APPLY_PIPELINE, a.pipeline)
        for prec in a.prec.split(","):
            dt, s = (torch.float64, 8) if prec == "fp64" else (torch.float32, 4)
            g = torch.Generator(device="cuda").manual_seed(p)
            q = [torch.randn(ctx.shape, dtype=dt, device="cuda", generator=g) for _ in range(3)]
            yr, yi = torch.empty_like(q[0]), torch.empty_like(q[0])
            f = ctx.schro_res if prec == "fp64" else ctx.schro_res_f32
            for _ in range(3):
                f(q[2], 0.01, q[0], q[1], yr, yi)
            st = torch.cuda.current_stream()
            times = []
            for _ in range(a.reps):
                flush.fill_(1.0)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                f(q[2], 0.01, q[0], q[1], yr, yi)
                e1.record(st)
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
            ms = float(np.median(times))
            nbytes = ctx.n * s * 9
            gbs = nbytes / ms / 1e6
            print(json.dumps({"p": p, "n": n, "elements": ctx.E, "global_nodes": ctx.info.n_nodes,
                              "n_loc": ctx.n, "prec": prec, "pipeline": a.pipeline, "ms": round(ms, 4), "bytes": nbytes,
                              "gbs": round(gbs, 1), "frac_hbm": round(gbs / peak, 4), "peak_source": src}),
                  flush=True)
            del q, yr, yi
        ctx.close()
        del ctx
        torch.cuda.empty_cache()


if __name__ == "__main__":
    main()
