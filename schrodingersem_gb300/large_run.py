"""Large combined workload: adaptive SDIRK4 5-stage on a 21-million-node
mesh with FP32 inner iterations, FP64 refinement and the element
preconditioner.

    python -m schrodingersem_gb300.large_run [--n 384] [--p 12] [--steps 3]

Mesh: n x n jittered quads (+-0.1 h, seed 1) on [-12,12]^2, degree p
(n = 384, p = 12: 4609^2 = 21.2M global nodes, 24.9M element-local nodes per
component).  Potential: double well V = 0.5 (x^2 - 9)^2 + y^2 / 2 plus a
seeded sum of six Gaussians of amplitude U(-0.5, 0.5) (widths U(0.3,1.5)).
Initial state: Gaussian packet (sigma 1, centre (-3,0), momentum (1,0)) in
the left well.  The equation i psi_t = -lap/2 psi + V psi runs in the
reference's convention (V' = 2V, dt' = dt/2, psi' = conj psi).  The step
size adapts to keep the embedded error estimate below 1e-8; the run stops
after --steps accepted steps.  Prints one JSON line: device seconds per
accepted step, accepted/rejected counts, iterations per stage.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=384)
    ap.add_argument("--p", type=int, default=12)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--dt0", type=float, default=4e-4, help="first trial step (workload units)")
    ap.add_argument("--err-tol", type=float, default=1e-8)
    a = ap.parse_args()
    import torch

    import schrodingersem_gb300 as S
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.meshgen import gaussian_packet, structured_quads
    S.build()
    t0 = time.time()
    co, el = structured_quads(a.n, box=(-12.0, 12.0, -12.0, 12.0), jitter=0.1, seed=1)
    ctx = S.Context(a.p, coords=co, elements=el)
    setup_s = time.time() - t0
    X, Y = ctx.node_coords()
    rng = np.random.default_rng(5)
    V = 0.5 * (X * X - 9.0) ** 2 + 0.5 * Y * Y
    for _ in range(6):
        A, w = rng.uniform(-0.5, 0.5), rng.uniform(0.3, 1.5)
        cx, cy = rng.uniform(-12, 12), rng.uniform(-12, 12)
        V += A * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * w * w))
    re, im = gaussian_packet(X, Y, (-3.0, 0.0), 1.0, (1.0, 0.0))
    dre, dim, dV = ctx.to_device(re), ctx.to_device(-im), ctx.to_device(2.0 * V)
    del X, Y, V, re, im
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
    ctx.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
    ctx.set_option(capi.OPT_STAGE_GUESS, capi.GUESS_EXTRAPOLATE)
    ctx.set_option(capi.OPT_PROFILE, 1)
    s0 = ctx.stats()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    ok, dts, nrej = ctx.schrodinger_adaptive(dre, dim, dV, 1e9, a.dt0 / 2, 20 * ctx.dof(), 1e-10, a.err_tol,
                                             n_steps=a.steps)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    s1 = ctx.stats()
    stages = 5 * (len(dts) + nrej)
    print(json.dumps({
        "metric": "adaptive SDIRK4-5 seconds per accepted step", "value": ms / 1e3 / max(1, len(dts)),
        "unit": "s/step", "accepted": len(dts), "rejected": nrej, "success": ok,
        "dt_workload_units": [2 * d for d in dts.tolist()], "last_error_estimate": s1.last_error_estimate,
        "inner_iterations_per_stage": (s1.solver_iterations_fp32 - s0.solver_iterations_fp32) / max(1, stages),
        "solver_kernel_ms": s1.solver_kernel_ms - s0.solver_kernel_ms, "setup_s": setup_s,
        "config": {"workload": f"{a.n}x{a.n} jittered quads on [-12,12]^2, p={a.p} ({(a.n * a.p + 1) ** 2:,} "
                               f"nodes), double well + 0.5-amplitude Gaussian disorder, adaptive SDIRK4-5 at "
                               f"embedded error {a.err_tol:g}, MINRES 1e-10, FP32 inner + FP64 refinement, "
                               f"element preconditioner", "local_nodes_per_component": ctx.n},
    }))


if __name__ == "__main__":
    main()
