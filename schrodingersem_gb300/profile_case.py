"""Small, self-contained workloads for profiling one kernel under ncu.

    python -m schrodingersem_gb300.profile_case --case minres --n 192 --p 8 --maxit 30
    python -m schrodingersem_gb300.profile_case --case apply --n 192 --p 8 --prec fp32

``minres``: one Schroedinger stage solve (persistent MINRES, capped at
``maxit`` iterations) on an n x n jittered mesh; ``apply``: a few standalone
Res applies.  Sizes default to a working set larger than L2 (129 MB) but a
few hundred MB on the device.
"""
from __future__ import annotations

import argparse

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="minres", choices=["minres", "apply", "batch"])
    ap.add_argument("--instances", type=int, default=64, help="batch: ensemble size")
    ap.add_argument("--n", type=int, default=192)
    ap.add_argument("--p", type=int, default=8)
    ap.add_argument("--maxit", type=int, default=30)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--prec", default="fp64", choices=["fp64", "fp32", "mixed"])
    ap.add_argument("--tol", type=float, default=1e-10, help="0 runs exactly maxit iterations")
    ap.add_argument("--time", action="store_true", help="print device time per iteration")
    ap.add_argument("--pipeline", type=int, default=1, help="apply: 1 bulk-copy pipelined kernel, 0 one-pass")
    ap.add_argument("--precond", type=int, default=0, help="mixed minres: 0 none, 1 diagonal, 2 element FDM")
    a = ap.parse_args()
    import torch

    import schrodingersem_gb300 as S
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.meshgen import gaussian_packet, structured_quads
    S.build()
    if a.case == "batch":  # a few BDF2 steps of the seeded ensemble workload
        from schrodingersem_gb300.batch import Batch
        from schrodingersem_gb300.batch_bench import instance_fields, make_instances
        from schrodingersem_gb300.meshgen import element_node_coords
        insts = make_instances(a.instances)
        B = Batch([(i["p"], i["coords"], i["elements"]) for i in insts])
        z = {}
        for pp in sorted({i["p"] for i in insts}):
            c = S.Context(pp, coords=insts[0]["coords"], elements=insts[0]["elements"])
            z[pp] = c.quadrature()[0]
            c.close()
        re, im, V = [], [], []
        for inst in insts:
            X, Y = element_node_coords(inst["coords"], inst["elements"], z[inst["p"]])
            v, r, i = instance_fields(inst, X, Y)
            re.append(torch.as_tensor(r, device="cuda"))
            im.append(torch.as_tensor(i, device="cuda"))
            V.append(torch.as_tensor(v, device="cuda"))
        ok = B.bdf2(re, im, V, (a.reps - 0.5) * 2.5e-3, 2.5e-3, 200000, 1e-10)
        st = B.stats()
        print(f"batch: instances={a.instances} steps={a.reps} converged={sum(ok)} ms_per_step={st.kernel_ms / a.reps:.3f}"
              f" inner_iterations={st.krylov_iterations}")
        return
    co, el = structured_quads(a.n, box=(-8.0, 8.0, -8.0, 8.0), jitter=0.1, seed=1)
    ctx = S.Context(a.p, coords=co, elements=el)
    X, Y = ctx.node_coords()
    re, im = gaussian_packet(X, Y, (-2.0, 0.0), 1.0, (3.0, 0.0))
    V = X * X + Y * Y
    if a.case == "apply":
        ctx.set_option(capi.OPT_APPLY_PIPELINE, a.pipeline)
        dt = torch.float64 if a.prec == "fp64" else torch.float32
        q = [ctx.to_device(t, dt) for t in (re, im, V)]
        f = ctx.schro_res if a.prec == "fp64" else ctx.schro_res_f32
        for _ in range(a.reps):
            f(q[2], 0.01, q[0], q[1])
        torch.cuda.synchronize()
        return
    if a.prec == "mixed":
        ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
        ctx.set_option(capi.OPT_INNER_TOL, max(a.tol, 1e-30))
        ctx.set_option(capi.OPT_MAX_REFINE, 1)
        ctx.set_option(capi.OPT_PRECOND, a.precond)
    ctx.set_option(capi.OPT_PROFILE, 1)
    dV = ctx.to_device(V)
    br, bi = ctx.schro_f(dV, ctx.to_device(re), ctx.to_device(im))
    for rep in range(a.reps if a.time else 1):
        xr, xi = ctx.zeros(), ctx.zeros()
        s0 = ctx.stats()
        ok, it, res = ctx.minres_schro(dV, 0.0054, xr, xi, br, bi, a.maxit, a.tol, x_is_zero=True)
        torch.cuda.synchronize()
        s1 = ctx.stats()
    ms = s1.solver_kernel_ms - s0.solver_kernel_ms
    print(f"minres: n={a.n} p={a.p} prec={a.prec} success={ok} iterations={it} residual={res:.3e} "
          f"kernel_ms={ms:.3f} us_per_iteration={1e3 * ms / max(it, 1):.2f}")


if __name__ == "__main__":
    main()
