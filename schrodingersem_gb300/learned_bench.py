"""Learned warm start workload: SDIRK4 5-stage on random Gaussian-sum
potentials; the network is trained on stage solves of training seeds and
evaluated on held-out seeds against the extrapolated and the zero guess.

    python -m schrodingersem_gb300.learned_bench [--n 128] [--train 8] [--eval 4] [--steps 8]

Mesh: n x n jittered quads (seed 1) on [-10,10]^2, p = 8.  Seed s draws a
potential (six Gaussians, amplitude U(-20,20), width U(0.3,1.5), centres
uniform in the box) and a Gaussian packet (sigma U(0.5,1.5), momentum
uniform in [-4,4]^2, centre uniform in [-5,5]^2); the equation
i psi_t = -lap/2 psi + V psi runs in the reference's convention
(V' = 2V, dt' = dt/2, psi' = conj psi), dt = 5e-3, MINRES 1e-10, FP32
inner iterations with FP64 refinement and the element preconditioner.
Training rows are recorded from the training seeds' stage solves (up to
--rows rows) and fitted with the library's BF16 network; every held-out
seed then runs --steps steps with the zero, the extrapolated and the
learned guess.  Prints one JSON line with iterations per stage and device
seconds per step of each guess.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def seed_fields(X, Y, seed):
    from schrodingersem_gb300.meshgen import gaussian_packet
    rng = np.random.default_rng(1000 + seed)
    V = np.zeros_like(X)
    for _ in range(6):
        A, w = rng.uniform(-20, 20), rng.uniform(0.3, 1.5)
        cx, cy = rng.uniform(-10, 10), rng.uniform(-10, 10)
        V += A * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * w * w))
    sg, k, c = rng.uniform(0.5, 1.5), rng.uniform(-4, 4, 2), rng.uniform(-5, 5, 2)
    re, im = gaussian_packet(X, Y, (float(c[0]), float(c[1])), float(sg), (float(k[0]), float(k[1])))
    return 2.0 * V, re, -im


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--p", type=int, default=8)
    ap.add_argument("--train", type=int, default=8)
    ap.add_argument("--eval", type=int, default=4)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--train-steps", type=int, default=8)
    ap.add_argument("--rows", type=int, default=600000)
    ap.add_argument("--hidden", type=int, default=384)
    ap.add_argument("--epochs", type=int, default=4)
    a = ap.parse_args()
    import torch

    import schrodingersem_gb300 as S
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.learned import Learner
    from schrodingersem_gb300.meshgen import structured_quads
    S.build()
    co, el = structured_quads(a.n, box=(-10.0, 10.0, -10.0, 10.0), jitter=0.1, seed=1)
    ctx = S.Context(a.p, coords=co, elements=el)
    X, Y = ctx.node_coords()
    dt, tol = 2.5e-3, 1e-10
    maxit = 20 * ctx.dof()
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
    ctx.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
    ctx.set_option(capi.OPT_REFINE_TOL_SCALE, 0.1)
    ctx.set_option(capi.OPT_PROFILE, 1)

    def run(seed, guess, steps):
        ctx.set_option(capi.OPT_STAGE_GUESS, guess)
        V, re, im = seed_fields(X, Y, seed)
        dre, dim, dV = ctx.to_device(re), ctx.to_device(im), ctx.to_device(V)
        s0 = ctx.stats()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(torch.cuda.current_stream())
        ok = ctx.schrodinger("dirk4s5", dre, dim, dV, (steps - 0.5) * dt, dt, maxit, tol)
        e1.record(torch.cuda.current_stream())
        torch.cuda.synchronize()
        s1 = ctx.stats()
        return ok, e0.elapsed_time(e1), s1.solver_iterations_fp32 - s0.solver_iterations_fp32, s0, s1

    # training data: stage solves of the training seeds (extrapolated guesses)
    t0 = time.time()
    ctx.record(a.rows)
    for sd in range(a.train):
        ok, *_ = run(sd, capi.GUESS_EXTRAPOLATE, a.train_steps)
        assert ok
    Xd, Td = ctx.dataset()
    ctx.record(0)
    record_s = time.time() - t0
    t0 = time.time()
    net = Learner.for_mesh(ctx.N, hidden=a.hidden, seed=3)
    loss = net.fit(Xd, Td, epochs=a.epochs, batch=1024, lr=1e-3, seed=11)
    torch.cuda.synchronize()
    fit_s = time.time() - t0
    tvar = float(Td.float().pow(2).mean())
    ctx.set_learner(net)
    del Xd, Td
    out = {}
    for name, guess in (("zero", capi.GUESS_ZERO), ("extrapolated", capi.GUESS_EXTRAPOLATE),
                        ("learned", capi.GUESS_LEARNED)):
        ms_tot, it_tot, ratio_sum, n_learned = 0.0, 0, 0.0, 0
        for sd in range(a.train, a.train + a.eval):
            ok, ms, its, s0, s1 = run(sd, guess, a.steps)
            assert ok
            ms_tot += ms
            it_tot += its
            ratio_sum += s1.learned_ratio_sum - s0.learned_ratio_sum
            n_learned += s1.learned_guesses - s0.learned_guesses
        stages = 5 * a.steps * a.eval
        out[name] = {"s_per_step": ms_tot / 1e3 / (a.steps * a.eval), "iterations_per_stage": it_tot / stages}
        if n_learned:
            out[name]["mean_guess_residual_ratio"] = ratio_sum / n_learned
    params = net.d_in * net.hidden + net.hidden + net.hidden * net.hidden + net.hidden + net.hidden * net.d_out + net.d_out
    print(json.dumps({
        "metric": "SDIRK4-5 stage guess: held-out seeds", "forms": out,
        "training": {"seeds": a.train, "steps": a.train_steps, "rows": int(min(a.rows, 5 * (a.train_steps - 2) * a.train * ctx.E)),
                     "record_s": record_s, "fit_s": fit_s, "final_mse_rel": loss / tvar if tvar else None,
                     "params": params, "epochs": a.epochs},
        "config": {"workload": f"{a.n}x{a.n} jittered quads on [-10,10]^2, p={a.p}, Gaussian-sum potentials and packets "
                               f"per seed, SDIRK4-5 dt=5e-3, MINRES 1e-10, FP32 inner + FP64 refinement, element "
                               f"preconditioner; {a.eval} held-out seeds x {a.steps} steps",
                   "local_nodes_per_component": ctx.n},
    }))


if __name__ == "__main__":
    main()
