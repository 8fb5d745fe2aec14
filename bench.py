#!/usr/bin/env python3
"""Benchmark: seconds per Schroedinger time step on one GB300.

Workload (the configuration the headline metric is quoted on): SDIRK4
3-stage on 64x64 bilinear quads over [-8,8]^2, interior vertices jittered by
+-0.1h (seed 1), p = 8 (513^2 = 263,169 global nodes, 331,776 element-local
nodes per component), V = (x^2+y^2)/2, normalised Gaussian packet (sigma 1,
centre (-2,0), momentum (3,0)), dt = 1e-2, MINRES tolerance 1e-10.  The
reference solves i psi_t = -(-lap + V) psi; the workload's
i psi_t = -lap/2 psi + V psi maps onto it exactly with V' = 2V, dt' = dt/2 and
psi' = conj(psi).

A step is one time step (3 implicit stages).  ``value`` is the device-time
of a step with the state resident in HBM (L2 flushed before every step);
``e2e`` is the same step through the C ABI with host (pinned) buffers, the
host<->device copies inside the timed region.  ``--impl reference`` times
the CPU oracle (a restatement of the reference's OpenMP path; the reference
itself cannot be built here) on the host cores on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "s/time-step at 1e-8 rel err vs FP64: learned+FP32 vs plain GPU; apply GB/s"
WORKLOAD = ("Schroedinger SDIRK4-3 time step, 64x64 jittered quads on [-8,8]^2 (seed 1), p=8 "
            "(263,169 nodes), V=(x^2+y^2)/2, Gaussian packet sigma=1 r0=(-2,0) k=(3,0), dt=1e-2, "
            "MINRES tol 1e-10")
DT, TOL, P, NEL = 1e-2, 1e-10, 8, 64
ORACLE_TOL = 1e-13  # MINRES tolerance of the FP64 accuracy reference run
# DRAM bytes (read + write) per launch of the element-preconditioned FP32
# solver kernel on this workload: mean of three launches of the timed steps
# captured with ncu (dram__bytes_read.sum + dram__bytes_write.sum).  The
# solver's working set stays in L2, so this is far below the algorithmic bytes.
SOLVER_DRAM_BYTES_PER_LAUNCH = 90.8e6


def workload_inputs():
    """mesh + reference-convention inputs (V' = 2V, dt' = dt/2, psi' = conj psi)"""
    from schrodingersem_gb300.meshgen import element_node_coords, gaussian_packet, structured_quads
    co, el = structured_quads(NEL, box=(-8.0, 8.0, -8.0, 8.0), jitter=0.1, seed=1)
    return co, el


def fields(ctx_or_mesh):
    X, Y = ctx_or_mesh.node_coords()
    from schrodingersem_gb300.meshgen import gaussian_packet
    re, im = gaussian_packet(X, Y, (-2.0, 0.0), 1.0, (3.0, 0.0))
    return X, Y, re, im


def mass_norm(J, w, re, im):
    ww = w[None, :, None] * w[None, None, :]
    return math.sqrt(float(np.sum(ww * J * (re * re + im * im))))


def flush_l2(buf):
    buf.zero_()


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region"""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [t.strip() for t in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- reference
def run_reference(args):
    """CPU oracle (restatement of the reference's OpenMP path) on host cores."""
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    co, el = workload_inputs()
    om = O.Mesh(P, coords=co, elements=el)
    X, Y, re, im = fields(om)
    nrm = mass_norm(om.J, om.w, re, im)
    re, im = re / nrm, im / nrm
    Vr = 2.0 * 0.5 * (X * X + Y * Y)
    dtr = DT / 2.0
    # a full CPU step of this workload takes tens of seconds, so the run is
    # bounded: at most one warm-up step, then timed steps until the budget
    # is spent (at least one)
    budget_s = float(os.environ.get("SEM_REF_BUDGET_S", "150"))
    warm = min(args.warmup, 1)
    total = warm + args.steps
    times = []
    t_last = [0.0]
    import ctypes as C

    def _cb(user, step, a, b, iters, n):
        now = time.perf_counter()
        times.append(now - t_last[0])
        t_last[0] = now
        if step >= total:
            return 1
        if step > warm and sum(times[warm:]) > budget_s:
            return 1
        return 0

    cbf = O._CB(_cb)
    pr, pi = np.ascontiguousarray(re), np.ascontiguousarray(-im)
    V = np.ascontiguousarray(Vr)
    opts = O.OrOpts(20 * om.dof(), TOL, dtr, 0)
    t_last[0] = time.perf_counter()
    O.lib().or_schrodinger_dirk4s3(om._ptr, O._p(pr), O._p(pi), O._p(V), 1e9, C.byref(opts), cbf, None)
    timed = times[warm:] if len(times) > warm else times[-1:]
    sps = float(np.mean(timed))
    line = {"impl": "reference", "metric": METRIC, "value": sps, "unit": "s/step", "n_gpus": args.gpus,
            "steps": len(timed), "warmup": warm,
            "ms_per_step": sps * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": "reference OpenMP path (CPU oracle port)"},
            "cpu_baseline": {"value": sps, "unit": "s/step", "cores": threads, "kind": "port",
                             "sample": f"{len(timed)} timed SDIRK4-3 steps after {warm} warm-up, "
                                       f"OpenMP {threads} threads"},
            "e2e": {"value": sps, "unit": "s/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- ours
def cpu_baseline_sample(iters_per_step, cap=60):
    """Bounded CPU sample: the oracle's first-stage MINRES of the workload,
    capped at `cap` iterations (plus its right-hand side), after one untimed
    repetition; scaled to a step by the step's measured MINRES iteration
    total (the GPU runs the same algorithm, so the counts agree)."""
    import ctypes as C

    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    co, el = workload_inputs()
    om = O.Mesh(P, coords=co, elements=el)
    X, Y, re, im = fields(om)
    nrm = mass_norm(om.J, om.w, re, im)
    V = np.ascontiguousarray(X * X + Y * Y)
    opts = O.OrOpts(int(cap), TOL, DT / 2, 0)
    secs = []
    for _ in range(2):
        pr, pi = np.ascontiguousarray(re / nrm), np.ascontiguousarray(-im / nrm)
        t0 = time.perf_counter()
        O.lib().or_schrodinger_dirk4s3(om._ptr, O._p(pr), O._p(pi), O._p(V), 1e9, C.byref(opts),
                                       O._CB(0), None)
        secs.append(time.perf_counter() - t0)
    per_iter = secs[-1] / cap
    return {"value": per_iter * iters_per_step, "unit": "s/step", "cores": threads, "kind": "port",
            "sample": f"CPU oracle, OpenMP {threads} threads: first-stage MINRES of the workload capped at "
                      f"{cap} iterations ({secs[-1]:.2f} s, after one untimed repetition), scaled by the "
                      f"step's measured {iters_per_step:.0f} MINRES iterations"}


def _batch_cpu_worker(args):
    """one ensemble instance on the CPU oracle (one thread): seconds per BDF2 step"""
    inst, steps, dt, tol = args
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    from schrodingersem_gb300.batch_bench import instance_fields
    O.build()
    O.set_threads(1)
    om = O.Mesh(inst["p"], coords=inst["coords"], elements=inst["elements"])
    X, Y = om.node_coords()
    V, re, im = instance_fields(inst, X, Y)
    t0 = time.perf_counter()
    _, _, ok = om.schrodinger("bdf2", re, im, V, (steps - 0.5) * dt, dt, 20 * om.dof(), tol)
    return (time.perf_counter() - t0) / steps, bool(ok), int(inst["n"]) ** 2 * (inst["p"] + 1) ** 2


def batch_cpu_baseline(n_instances, sample=16, steps=2):
    """the ensemble on the host cores: a size-stratified sample of instances,
    one process (one thread) per instance, every core busy; the machine's
    instance-steps/s scaled to the ensemble's mean instance size"""
    import multiprocessing as mp

    from schrodingersem_gb300.batch_bench import make_instances
    insts = make_instances(n_instances)
    size = [i["n"] ** 2 * (i["p"] + 1) ** 2 for i in insts]
    order = sorted(range(len(insts)), key=lambda i: size[i])
    pick = [order[int(round(q))] for q in np.linspace(0, len(order) - 1, min(sample, len(order)))]
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(min(cores, len(pick))) as pool:
        res = pool.map(_batch_cpu_worker, [(insts[i], steps, 2.5e-3, 1e-10) for i in pick])
    wall = time.perf_counter() - t0
    s_node_step = sum(r[0] for r in res) / sum(r[2] for r in res)
    per_inst_step = s_node_step * float(np.mean(size))
    return {"value": cores / per_inst_step, "unit": "instance-steps/s", "cores": cores, "kind": "port",
            "sample": f"{len(pick)} instances stratified by size, {steps} BDF2 steps each on the CPU oracle (FP64 "
                      f"MINRES, one thread per process, {wall:.1f} s wall); rate = cores / (mean instance size x "
                      f"measured seconds per node-step)", "all_converged": all(r[1] for r in res)}


APPLY_NEL = 559  # 559^2 elements at p = 8: 4473^2 = 20.0 M global nodes
FP64_PEAK_TFLOPS = 1.19  # FMA-chain probe of the FP64 pipe on this GB300


def apply_gbs(S, torch, reps=20):
    """standalone Res apply (element kernel + assembly into the masked
    format) on 559x559 jittered quads over [-12,12]^2 at p = 8 (20.0 M global
    nodes, 25.3 M element-local nodes per plane, above L2), L2 flushed before
    each apply.  Algorithmic bytes n_loc * s * 9 (psi 2 planes, out 2,
    g11 g12 g22 mass, V) and flops n_loc * (16 N + 23) per apply."""
    from schrodingersem_gb300.meshgen import structured_quads
    co, el = structured_quads(APPLY_NEL, box=(-12.0, 12.0, -12.0, 12.0), jitter=0.1, seed=1)
    ctx = S.Context(P, coords=co, elements=el)
    n = ctx.n
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out = {"workload": f"{APPLY_NEL}x{APPLY_NEL} jittered quads on [-12,12]^2, p={P} "
                       f"({(APPLY_NEL * P + 1) ** 2:,} global nodes, {n:,} element-local nodes per plane)",
           "l2": "flushed before every apply (256 MiB write)", "reps": reps}
    for prec, dt, s in (("fp64", torch.float64, 8), ("fp32", torch.float32, 4)):
        g = torch.Generator(device="cuda").manual_seed(0)
        q = [torch.randn(ctx.shape, dtype=dt, device="cuda", generator=g) for _ in range(3)]
        yr, yi = torch.empty_like(q[0]), torch.empty_like(q[0])
        f = ctx.schro_res if prec == "fp64" else ctx.schro_res_f32
        for _ in range(3):
            f(q[2], 0.01, q[0], q[1], yr, yi)
        st = torch.cuda.current_stream()
        tot = 0.0
        for _ in range(reps):
            flush_l2(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            f(q[2], 0.01, q[0], q[1], yr, yi)
            e1.record(st)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        ms = tot / reps
        bytes_ = n * s * 9
        flops = n * (16 * ctx.N + 23)
        out[prec] = {"ms": ms, "gbs": bytes_ / ms / 1e6, "bytes": bytes_,
                     "tflops": flops / ms / 1e9, "flops": flops}
        del q, yr, yi
    out["fp32"]["bound"] = "hbm"
    out["fp64"]["bound"] = "fp64"
    out["fp64"]["frac_fp64"] = out["fp64"]["tflops"] / FP64_PEAK_TFLOPS
    out["fp64"]["fp64_peak_tflops"] = FP64_PEAK_TFLOPS
    ctx.close()
    del flush
    torch.cuda.empty_cache()
    return out


FORMS = {
    # name: (solve precision, inner tolerance, preconditioner, description)
    "fp64": ("fp64", None, 0, "plain FP64 GPU MINRES (reference algorithm, zero stage guess)"),
    "mixed": ("mixed", 1e-4, 0, "FP32-inner MINRES in FP64 iterative refinement (true FP64 residual "
                                "judged by the reference's criterion), zero stage guess"),
    "mixed_diag": ("mixed", 1e-4, 1, "FP32-inner MINRES with diagonal preconditioner in FP64 iterative "
                                     "refinement, zero stage guess"),
    "mixed_extrap": ("mixed", 1e-4, 0, "FP32-inner MINRES in FP64 iterative refinement, stage guess "
                                       "extrapolated linearly from the last two steps (test relative to |b|)"),
    "mixed_diag_extrap": ("mixed", 1e-4, 1, "FP32-inner MINRES with diagonal preconditioner in FP64 iterative "
                                            "refinement, extrapolated stage guess (test relative to |b|)"),
    "mixed_fdm": ("mixed", 3e-4, 2, "FP32-inner MINRES with the element fast-diagonalisation |A|^-1 "
                                    "preconditioner in FP64 iterative refinement, zero stage guess"),
    "mixed_fdm_extrap": ("mixed", 3e-4, 2, "FP32-inner MINRES with the element fast-diagonalisation "
                                           "preconditioner in FP64 iterative refinement, extrapolated stage "
                                           "guess (test relative to |b|)"),
    "mixed_fdm_learned": ("mixed", 3e-4, 2, "FP32-inner MINRES with the element fast-diagonalisation "
                                            "preconditioner in FP64 iterative refinement, stage guess = "
                                            "linear extrapolation corrected by the BF16 network (trained on the "
                                            "GPU on stage solves of other initial packets), residual-minimising "
                                            "step"),
}
FORMS["mixed_fdm_extrap2"] = ("mixed", 3e-4, 2, "FP32-inner MINRES with the element fast-diagonalisation "
                                                "preconditioner in FP64 iterative refinement, stage guess "
                                                "extrapolated quadratically from the last three steps")
GUESS = {"mixed_extrap": 1, "mixed_diag_extrap": 1, "mixed_fdm_extrap": 1, "mixed_fdm_extrap2": 1,
         "mixed_fdm_learned": 2}
EXTRAP_ORDER = {"mixed_fdm_extrap2": 2}
# training trajectories of the learned form: packets (centre, sigma, momentum)
# other than the workload's, on the same mesh and potential
TRAIN_PACKETS = [((-3.0, 1.0), 1.2, (2.0, 1.0)), ((1.0, -2.0), 0.8, (-2.5, 2.0)), ((0.5, 2.5), 1.0, (1.0, -3.0))]
TRAIN_STEPS = 10


def set_form_options(ctx, form):
    from schrodingersem_gb300 import capi
    prec, itol, pc, _ = FORMS[form]
    ctx.set_option(capi.OPT_PRECOND, pc)
    ctx.set_option(capi.OPT_STAGE_GUESS, GUESS.get(form, 0))
    ctx.set_option(capi.OPT_EXTRAP_ORDER, EXTRAP_ORDER.get(form, 1))
    # the fast forms stop on the true FP64 residual below the reference's
    # threshold (half of it; a tenth with the element preconditioner, whose
    # extra digits cost few iterations), which keeps their states within 1e-8
    # of the FP64 solve
    ctx.set_option(capi.OPT_REFINE_TOL_SCALE, (0.1 if pc == 2 else 0.5) if prec == "mixed" else 1.0)
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED if prec == "mixed" else capi.PREC_FP64)
    if itol:
        ctx.set_option(capi.OPT_INNER_TOL, itol)


def train_learner(ctx, torch, Vd, X, Y):
    """record stage solves of TRAIN_PACKETS (extrapolated guesses), fit the
    network on them; returns the learner and a summary"""
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.learned import Learner
    from schrodingersem_gb300.meshgen import gaussian_packet
    t0 = time.time()
    ctx.set_option(capi.OPT_STAGE_GUESS, capi.GUESS_EXTRAPOLATE)
    ctx.record(ctx.E * 3 * (TRAIN_STEPS - 2) * len(TRAIN_PACKETS))
    dtr = DT / 2.0
    J, _, _, _ = ctx.metrics()
    _, w, _ = ctx.quadrature()
    for c, sg, k in TRAIN_PACKETS:
        re, im = gaussian_packet(X, Y, c, sg, k)
        nrm = mass_norm(J, w, re, im)
        dre, dim = ctx.to_device(re / nrm), ctx.to_device(-im / nrm)
        if not ctx.schrodinger("dirk4s3", dre, dim, Vd, (TRAIN_STEPS - 0.5) * dtr, dtr, 20 * ctx.dof(), TOL):
            raise RuntimeError("training trajectory did not converge")
    torch.cuda.synchronize()
    t_rec = time.time() - t0
    Xd, Td = ctx.dataset()
    ctx.record(0)
    t1 = time.time()
    L = Learner.for_mesh(ctx.N, hidden=256, seed=3)
    loss = L.fit(Xd, Td, epochs=4, batch=1024, lr=1e-3, seed=11)
    torch.cuda.synchronize()
    t_fit = time.time() - t1
    tv = float(Td.float().pow(2).mean())
    ctx.set_learner(L)
    return L, {"rows": int(Xd.shape[0]), "record_s": t_rec, "fit_s": t_fit, "final_mse": loss,
               "final_mse_rel": loss / tv if tv > 0 else None, "params": int(
                   L.d_in * L.hidden + L.hidden + L.hidden * L.hidden + L.hidden + L.hidden * L.d_out + L.d_out)}


def run_form(ctx, torch, form, re, im, Vr, steps, warmup, flush, clocks=None):
    """warm-up + timed steps of one solver form, state resident in HBM"""
    from schrodingersem_gb300 import capi
    set_form_options(ctx, form)
    dtr = DT / 2.0
    maxit = 20 * ctx.dof()
    dre, dim, dV = ctx.to_device(re), ctx.to_device(im), ctx.to_device(Vr)
    st = torch.cuda.current_stream()
    training = None
    if GUESS.get(form, 0) == 2:  # untimed: record training trajectories, fit the network
        X, Y = ctx.node_coords()
        _, training = train_learner(ctx, torch, dV, X, Y)
        set_form_options(ctx, form)

    def one_step(pr, pi, V):
        if not ctx.schrodinger("dirk4s3", pr, pi, V, 0.5 * dtr, dtr, maxit, TOL):
            raise RuntimeError(f"{form}: MINRES did not converge")

    for _ in range(warmup):
        one_step(dre, dim, dV)
    torch.cuda.synchronize()
    s0 = ctx.stats()
    times, iters, sweeps = [], [], []
    for _ in range(steps):
        flush_l2(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push(f"timed_{form}")  # profilers can select the timed steps of a form
        e0.record(st)
        one_step(dre, dim, dV)
        e1.record(st)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
        sts = ctx.stats()
        iters.append([int(sts.last_stage_iters[k]) for k in range(sts.last_step_stages)])
        sweeps.append([int(sts.last_stage_sweeps[k]) for k in range(sts.last_step_stages)])
    s1 = ctx.stats()
    return {
        "ms": float(np.mean(times)), "state": (dre.cpu().numpy(), dim.cpu().numpy()),
        "iters_per_step": float(np.mean([np.sum(i) for i in iters])),
        "iters_per_stage": float(np.mean([np.mean(i) for i in iters])),
        "sweeps_per_stage": float(np.mean([np.mean(i) for i in sweeps])),
        "launches": int(s1.kernel_launches - s0.kernel_launches),
        "solver_ms": s1.solver_kernel_ms - s0.solver_kernel_ms,
        "it64": s1.solver_iterations_fp64 - s0.solver_iterations_fp64,
        "it32": s1.solver_iterations_fp32 - s0.solver_iterations_fp32,
        "applies64": s1.fp64_applies - s0.fp64_applies,
        "learned": ({"guesses": s1.learned_guesses - s0.learned_guesses,
                     "accepted": s1.learned_accepted - s0.learned_accepted,
                     "last_residual_ratio": s1.last_guess_residual_ratio, "last_theta": s1.last_guess_theta,
                     "training": training} if training else None),
        "one_step": one_step,
    }


def run_ours(args):
    import torch

    import schrodingersem_gb300 as S
    from schrodingersem_gb300 import capi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    S.build()
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    co, el = workload_inputs()
    ctx = S.Context(P, coords=co, elements=el)
    ctx.set_option(capi.OPT_PROFILE, 1)
    X, Y, re, im = fields(ctx)
    J, _, _, _ = ctx.metrics()
    _, w, _ = ctx.quadrature()
    nrm = mass_norm(J, w, re, im)
    re, im = re / nrm, -im / nrm                     # psi' = conj(psi)
    Vr = X * X + Y * Y                               # V' = 2 * (x^2+y^2)/2
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    forms = [f for f in args.forms.split(",") if f]
    # accuracy reference: the same number of steps by the plain FP64 solver at
    # MINRES tolerance 1e-13 (untimed); every form is judged against it
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_FP64)
    ctx.set_option(capi.OPT_STAGE_GUESS, capi.GUESS_ZERO)
    o_re, o_im = ctx.to_device(re), ctx.to_device(im)
    dVo = ctx.to_device(Vr)
    for _ in range(args.warmup + args.steps):
        if not ctx.schrodinger("dirk4s3", o_re, o_im, dVo, 0.25 * DT, 0.5 * DT, 40 * ctx.dof(), ORACLE_TOL):
            raise RuntimeError("FP64 reference run did not converge")
    oracle_state = (o_re.cpu().numpy(), o_im.cpu().numpy())
    del o_re, o_im, dVo
    res = {}
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        for f in forms:
            res[f] = run_form(ctx, torch, f, re, im, Vr, args.steps, args.warmup, flush)
        if dist:
            dist.barrier()
    # accuracy of every form (M-weighted relative L2) against the FP64
    # reference run, and against the plain FP64 form at the workload tolerance
    def rel(a, b):
        return mass_norm(J, w, a[0] - b[0], a[1] - b[1]) / mass_norm(J, w, *b)

    for f, r in res.items():
        r["rel_err_vs_fp64"] = rel(r["state"], oracle_state)
        r["rel_err_vs_plain_fp64"] = rel(r["state"], res["fp64"]["state"]) if "fp64" in res else None
        r["norm_drift"] = abs(mass_norm(J, w, *r["state"]) - 1.0)
    valid = [f for f in forms if res[f]["rel_err_vs_fp64"] <= 1e-8]
    best = min(valid, key=lambda f: res[f]["ms"])
    # the metric is the learned-warm-start + FP32-inner form's step time; the
    # fastest form within the accuracy bar is reported beside it
    head = "mixed_fdm_learned" if "mixed_fdm_learned" in valid else best
    H = res[head]
    ms = H["ms"]
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())

    # e2e of the headline form through the C ABI with pinned host buffers
    h_re = torch.from_numpy(re.copy()).pin_memory()
    h_im = torch.from_numpy(im.copy()).pin_memory()
    h_V = torch.from_numpy(np.ascontiguousarray(Vr)).pin_memory()
    prec = FORMS[head][0]
    set_form_options(ctx, head)
    st = torch.cuda.current_stream()
    for _ in range(min(2, args.warmup)):
        H["one_step"](h_re.numpy(), h_im.numpy(), h_V.numpy())
    e2e_times = []
    for _ in range(args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        H["one_step"](h_re.numpy(), h_im.numpy(), h_V.numpy())
        e1.record(st)
        torch.cuda.synchronize()
        e2e_times.append(e0.elapsed_time(e1))
    e2e_s = float(np.mean(e2e_times)) / 1e3
    nbytes = ctx.n * 8
    if rank != 0:
        return
    app = apply_gbs(S, torch) if not args.no_apply else None
    # algorithmic bytes of the dominant kernel (the persistent solver):
    # per Krylov iteration one Res apply (9 words/node) + 13 two-plane vector
    # words; per FP64 refinement sweep one FP64 residual (apply + 5 words)
    n = ctx.n
    # (with the element preconditioner 16 two-plane vector words instead of
    # 13: its local solve reads y, r2 and writes y and the local result; the
    # apply pass reads that, writes z and reads y for beta; Phase B reads z
    # instead of r2 and the previous z instead of r1)
    b64 = n * 8 * (9 + 26)
    b32 = n * 4 * (9 + (32 if FORMS[head][2] == 2 else 26))
    sweeps_total = H["applies64"] if prec == "mixed" else 0
    alg_bytes = H["it64"] * b64 + H["it32"] * b32 + sweeps_total * n * 8 * 14
    achieved = alg_bytes / (H["solver_ms"] / 1e3) / 1e9 if H["solver_ms"] > 0 else None
    kern = "k_minres_mixed<9,RES>" if prec == "mixed" else "k_minres<9,double,RES>"
    forms_out = {f: {"s_per_step": r["ms"] / 1e3, "minres_iters_per_stage": r["iters_per_stage"],
                     "refine_sweeps_per_stage": r["sweeps_per_stage"], "rel_err_vs_fp64": r["rel_err_vs_fp64"],
                     "rel_err_vs_plain_fp64": r["rel_err_vs_plain_fp64"], "norm_drift": r["norm_drift"],
                     "description": FORMS[f][3], **({"learned": r["learned"]} if r.get("learned") else {})}
                 for f, r in res.items()}
    cpu = cpu_baseline_sample(res["fp64"]["iters_per_step"] if "fp64" in res else H["iters_per_step"]) \
        if not args.no_cpu else None
    # the batched-ensemble workload (1,024 seeded instances, BDF2)
    from schrodingersem_gb300.batch_bench import run_batch
    batch = run_batch(1024, steps=args.batch_steps, warmup=2) if args.batch_steps > 0 else None
    if batch and not args.no_cpu:
        batch["cpu_baseline"] = batch_cpu_baseline(1024)
        batch["speedup_vs_cpu"] = batch["value"] / batch["cpu_baseline"]["value"]
    flops64 = n * (2 * (8 * ctx.N + 14) + 6 + 2 * 13)
    line = {
        "metric": METRIC, "value": ms / 1e3, "unit": "s/step", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec == "fp64" else "f64+f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": head + ": " + FORMS[head][3],
                   "accuracy": f"M-weighted relative L2 of the state after warm-up + timed steps against the FP64 "
                               f"solver at MINRES tolerance {ORACLE_TOL:g} (headline forms must stay within 1e-8)",
                   "l2": "flushed before every step (256 MiB write)", "parallelism": "replicas only"},
        "forms": forms_out,
        "speedup_vs_plain_fp64": (res["fp64"]["ms"] / ms) if "fp64" in res else None,
        "fastest_form": {"form": best, "s_per_step": res[best]["ms"] / 1e3,
                         "speedup_vs_plain_fp64": (res["fp64"]["ms"] / res[best]["ms"]) if "fp64" in res else None},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": (achieved / hbm_peak) if achieved else None,
                     "traffic": SOLVER_DRAM_BYTES_PER_LAUNCH if FORMS[head][2] == 2 and prec == "mixed" else None,
                     "traffic_unit": "bytes per launch (ncu capture of the timed steps)",
                     "algorithmic_bytes_per_launch": alg_bytes / (3 * args.steps),
                     "launches": 3 * args.steps,
                     "kernel": kern + " (persistent cooperative solver)",
                     "algorithmic_bytes": alg_bytes, "fp64_iterations": H["it64"], "fp32_iterations": H["it32"],
                     "kernel_ms": H["solver_ms"], "peak_source": peak_src,
                     "fp64_pipe": ({"achieved_tflops": flops64 * H["it64"] / (H["solver_ms"] / 1e3) / 1e12,
                                    "peak_tflops": FP64_PEAK_TFLOPS, "peak_source": "FMA-chain probe on a GB300"}
                                   if prec == "fp64" and H["solver_ms"] > 0 else None)},
        "apply": ({"fp32_gbs": app["fp32"]["gbs"], "fp32_frac_hbm": app["fp32"]["gbs"] / hbm_peak,
                   "fp64_gbs": app["fp64"]["gbs"], "fp64_frac_hbm": app["fp64"]["gbs"] / hbm_peak,
                   "fp64_tflops": app["fp64"]["tflops"], "fp64_frac_fp64_pipe": app["fp64"]["frac_fp64"],
                   "detail": app, "note": "n_loc*s*9 algorithmic words and n_loc*(16N+23) flops per apply; "
                                          "the FP64 apply is bound by GB300's FP64 pipe, the FP32 apply by HBM"}
                  if app else None),
        "cpu_baseline": cpu,
        "batch": batch,
        "e2e": {"value": e2e_s, "unit": "s/step", "h2d_bytes_per_step": 3 * nbytes,
                "d2h_bytes_per_step": 2 * nbytes},
        "clocks": clk.summary(),
        "gpu_launches": H["launches"],
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--batch-steps", type=int, default=10,
                    help="timed steps of the batched-ensemble workload (0: skip it)")
    ap.add_argument("--no-apply", action="store_true", help="skip the 20M-node operator-apply measurement")
    ap.add_argument("--forms", default="fp64,mixed,mixed_fdm,mixed_fdm_extrap,mixed_fdm_extrap2,mixed_fdm_learned",
                    help="solver forms to time (comma list)")
    args = ap.parse_args()
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
