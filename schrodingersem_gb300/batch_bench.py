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


def run_batch(n_instances: int = 1024, steps: int = 100, warmup: int = 3, seed: int = 2026):
    """build the seeded ensemble, warm up (graph capture), time `steps` BDF2
    steps of all instances; returns the measurement as a dict"""
    import torch

    import schrodingersem_gb300 as S
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.batch import Batch
    from schrodingersem_gb300.meshgen import element_node_coords
    S.build()
    insts = make_instances(n_instances, seed)
    t0 = time.time()
    B = Batch([(i["p"], i["coords"], i["elements"]) for i in insts])
    setup_s = time.time() - t0
    B.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
    z = {}
    for pp in sorted({i["p"] for i in insts}):  # GLL nodes of each degree
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
    dt = 2.5e-3  # dt' = dt/2 of the workload's 5e-3
    maxit = 200000
    B.bdf2(re, im, V, (warmup - 0.5) * dt, dt, maxit, 1e-10)  # warm-up (graph capture)
    s0 = B.stats()
    torch.cuda.synchronize()
    t0 = time.time()
    ok = B.bdf2(re, im, V, (steps - 0.5) * dt, dt, maxit, 1e-10)
    torch.cuda.synchronize()
    wall = time.time() - t0
    s1 = B.stats()
    ms = s1.kernel_ms - s0.kernel_ms
    nodes = sum(i["n"] ** 2 * (i["p"] + 1) ** 2 for i in insts)
    return {
        "metric": "batched BDF2 instance-steps per second", "value": n_instances * steps / (ms / 1e3),
        "unit": "instance-steps/s", "instances": n_instances, "steps": steps, "warmup": warmup,
        "ms_per_step": ms / steps, "wall_s": wall, "setup_s": setup_s,
        "local_nodes_per_component": nodes, "converged": int(sum(ok)),
        "inner_iterations_per_instance_step": (s1.krylov_iterations - s0.krylov_iterations) / (n_instances * steps),
        "graph_launches": s1.graph_launches - s0.graph_launches, "graphs_built": s1.graphs_built,
        "kmax_of_p": {p: s1.kmax_of_p[p] for p in (4, 6, 8)},
        "config": {"workload": f"{n_instances:,} seeded instances: n~U{{4..32}} quads on [-6,6]^2, p in {{4,6,8}}, "
                               "6-Gaussian potentials, Gaussian packets; BDF2 dt=5e-3, MINRES 1e-10, FP32 inner + "
                               "FP64 refinement, element preconditioner", "dtype": "f64+f32"},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    a = ap.parse_args()
    sys.path.insert(0, ROOT)
    print(json.dumps(run_batch(a.instances, a.steps, a.warmup)))


if __name__ == "__main__":
    main()
