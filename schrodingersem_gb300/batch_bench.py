"""Batched-ensemble workload: many seeded independent Schroedinger instances
advanced by BDF2 in one sem_batch (one persistent launch per time step,
replayed from a captured CUDA graph).

    python -m schrodingersem_gb300.batch_bench [--instances 1024] [--steps 100]

Instance k (seeded): n x n jittered quads on [-6,6]^2 with n uniform in
[4,32], p drawn from {4,6,8}; potential a sum of six Gaussians (amplitude
U(-20,20), width U(0.3,1.5), centres uniform in the box); initial state a
unit-amplitude Gaussian packet (sigma U(0.5,1.5), momentum uniform in
[-4,4]^2, centre uniform in the inner half of the box).  The equation
i psi_t = -lap/2 psi + V psi is run in the reference's convention
(V' = 2V, dt' = dt/2, psi' = conj psi).  BDF2 with dt = 5e-3, MINRES to
1e-10, FP32 inner iterations with FP64 refinement and the element
preconditioner.  Prints one JSON line: instance-steps per second (device
time of the replayed steps) and iterations.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def make_instances(count: int, seed: int = 2026):
    from schrodingersem_gb300.meshgen import structured_quads
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(rng.integers(4, 33))
        p = int(rng.choice([4, 6, 8]))
        co, el = structured_quads(n, box=(-6.0, 6.0, -6.0, 6.0), jitter=0.1, seed=int(rng.integers(1 << 30)))
        gauss = [(rng.uniform(-20, 20), rng.uniform(0.3, 1.5), rng.uniform(-6, 6), rng.uniform(-6, 6))
                 for _ in range(6)]
        packet = (rng.uniform(0.5, 1.5), rng.uniform(-4, 4, 2), rng.uniform(-3, 3, 2))
        out.append({"n": n, "p": p, "coords": co, "elements": el, "gauss": gauss, "packet": packet})
    return out


def instance_fields(inst, X, Y):
    """reference-convention potential and state at the element-local nodes"""
    from schrodingersem_gb300.meshgen import gaussian_packet
    V = np.zeros_like(X)
    for A, w, cx, cy in inst["gauss"]:
        V += A * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * w * w))
    sg, k, c = inst["packet"]
    re, im = gaussian_packet(X, Y, (float(c[0]), float(c[1])), float(sg), (float(k[0]), float(k[1])))
    return 2.0 * V, re, -im


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    a = ap.parse_args()
    sys.path.insert(0, ROOT)
    insts = make_instances(a.instances)
    import torch

    import schrodingersem_gb300 as S
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.batch import Batch
    S.build()
    t0 = time.time()
    B = Batch([(i["p"], i["coords"], i["elements"]) for i in insts])
    setup_s = time.time() - t0
    B.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
    from schrodingersem_gb300.meshgen import element_node_coords
    z = {}
    for pp in sorted({i["p"] for i in insts}):  # GLL nodes of each degree
        c = S.Context(pp, coords=insts[0]["coords"], elements=insts[0]["elements"])
        z[pp] = c.quadrature()[0]
        c.close()
    fields = []
    for k, inst in enumerate(insts):
        X, Y = element_node_coords(inst["coords"], inst["elements"], z[inst["p"]])
        V, re, im = instance_fields(inst, X, Y)
        fields.append((torch.as_tensor(re, device="cuda"), torch.as_tensor(im, device="cuda"),
                       torch.as_tensor(V, device="cuda")))
    dt = 2.5e-3  # dt' = dt/2 of the workload's 5e-3
    maxit = 200000
    re = [f[0] for f in fields]
    im = [f[1] for f in fields]
    V = [f[2] for f in fields]
    ok = B.bdf2(re, im, V, (a.warmup - 0.5) * dt, dt, maxit, 1e-10)  # warm-up (graph capture)
    s0 = B.stats()
    torch.cuda.synchronize()
    t0 = time.time()
    ok = B.bdf2(re, im, V, (a.steps - 0.5) * dt, dt, maxit, 1e-10)
    torch.cuda.synchronize()
    wall = time.time() - t0
    s1 = B.stats()
    ms = s1.kernel_ms - s0.kernel_ms
    nodes = sum(i["n"] ** 2 * (i["p"] + 1) ** 2 for i in insts)
    line = {
        "metric": "batched BDF2 instance-steps per second", "value": a.instances * a.steps / (ms / 1e3),
        "unit": "instance-steps/s", "instances": a.instances, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms / a.steps, "wall_s": wall, "setup_s": setup_s,
        "local_nodes_per_component": nodes, "converged": int(sum(ok)),
        "inner_iterations_per_instance_step": (s1.krylov_iterations - s0.krylov_iterations) /
                                              (a.instances * a.steps),
        "graph_launches": s1.graph_launches - s0.graph_launches, "graphs_built": s1.graphs_built,
        "kmax_of_p": {p: s1.kmax_of_p[p] for p in (4, 6, 8)},
        "config": {"workload": "1,024 seeded instances: n~U{4..32} quads on [-6,6]^2, p in {4,6,8}, 6-Gaussian "
                               "potentials, Gaussian packets; BDF2 dt=5e-3, MINRES 1e-10, FP32 inner + FP64 "
                               "refinement, element preconditioner", "dtype": "f64+f32"},
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
