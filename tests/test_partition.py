"""Partitioned single-mesh path, host logic (CPU; gloo ranks).

``schrodingersem_gb300.partition`` splits one mesh's elements across ranks
(PCA median bisection, include/mpi_impl/distribute_mesh.hpp:82-132) and
provides the cross-rank global_sum / mask / dot of the reference's MPI path
(include/mpi_impl/global_sum.hpp:78-245, dot.hpp:11-68) and MINRES over
them.  Checked here: on one rank the operations equal the oracle's bit for
bit (dot to rounding); on 2 and 4 gloo ranks the gathered global_sum equals
the one-rank result bit for bit, and MINRES on a Schroedinger stage operator
(element kernel in NumPy over the oracle's metrics) takes the oracle's
iteration count and reaches its solution.  The per-rank device kernels are
not wired to this path; only the host logic is under test."""
import os
import socket

import numpy as np
import pytest

from schrodingersem_gb300 import partition as P
from tests.util import SMALL_MESH, structured


def _mesh(O, kind, p):
    if kind == "small":
        m = O.Mesh(p, folder=SMALL_MESH)
        return m, None, m.corner_ids
    co, el = structured(8, box=(-2.0, 2.0, -2.0, 2.0), jitter=0.15, seed=3)
    return O.Mesh(p, coords=co, elements=el), co, np.asarray(el)


def _local_res(m, V, alpha):
    """element-local (unassembled) Res = [M q0 + a L q1 ; a L q0 - M q1],
    L u = glaplace(u) + (W (u V) W) J, M u = (W u W) J (schrodinger.hpp)"""
    ww = np.outer(m.w, m.w)  # [j, i]

    def op(q, elems):
        q0, q1 = q
        o0, o1 = np.zeros_like(q0), np.zeros_like(q1)
        for k, e in enumerate(elems):
            mm = ww * m.J[e]
            mv = mm * V[e]
            l0 = m.glaplace(int(e), q0[k]) + mv * q0[k]
            l1 = m.glaplace(int(e), q1[k]) + mv * q1[k]
            o0[k] = mm * q0[k] + alpha * l1
            o1[k] = alpha * l0 - mm * q1[k]
        return o0, o1
    return op


def test_pca_bisection_balanced_and_deterministic():
    rng = np.random.default_rng(0)
    c = rng.uniform(-1, 1, size=(1000, 2)) * np.array([3.0, 1.0])
    for Pn in (1, 2, 4, 8):
        lab = P.pca_bisection(c, Pn)
        counts = np.bincount(lab, minlength=Pn)
        assert set(np.unique(lab)) == set(range(Pn))
        assert counts.max() - counts.min() <= Pn
        assert np.array_equal(lab, P.pca_bisection(c, Pn))
    # the first cut of an elongated cloud runs across its long axis
    lab = P.pca_bisection(c, 2)
    assert abs(c[lab == 0, 0].mean() - c[lab == 1, 0].mean()) > 2.0
    with pytest.raises(ValueError):
        P.pca_bisection(c, 3)


@pytest.mark.parametrize("kind,p", [("jit", 4), ("small", 3)])
def test_one_rank_equals_oracle(oracle, kind, p):
    m, co, el = _mesh(oracle, kind, p)
    part = P.Partition(el, m.N, np.zeros(m.n_el, dtype=int), 0, 1)
    rng = np.random.default_rng(5)
    a = rng.standard_normal(m.shape)
    b = rng.standard_normal(m.shape)
    assert np.array_equal(part.global_sum(a), m.global_sum(a))
    assert np.array_equal(part.mask(a), m.mask(a))
    assert abs(part.dot(a, b) - m.dot(a, b)) <= 1e-13 * abs(m.dot(np.abs(a), np.abs(b)))
    ones = np.ones(m.shape)
    assert part.dot(ones, ones) == m.dof()


def test_local_operator_assembles_to_oracle_res(oracle):
    m, co, el = _mesh(oracle, "jit", 4)
    X, Y = m.node_coords()
    V = X * X + Y * Y
    rng = np.random.default_rng(2)
    q = (m.mask(rng.standard_normal(m.shape)), m.mask(rng.standard_normal(m.shape)))
    part = P.Partition(el, m.N, np.zeros(m.n_el, dtype=int), 0, 1)
    A = part.operator(lambda u: _local_res(m, V, 0.01)(u, np.arange(m.n_el)))
    y = A(q)
    r0, r1 = m.schro_res(V, 0.01, *q)
    assert np.abs(y[0] - r0).max() <= 1e-12 * np.abs(r0).max()
    assert np.abs(y[1] - r1).max() <= 1e-12 * np.abs(r1).max()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import datetime

    import torch.distributed as dist

    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    try:
        O.set_threads(1)
        m, co, el = _mesh(O, "jit", 4)
        lab = P.pca_bisection(P.element_centres(co, el), world)
        part = P.Partition(el, m.N, lab, rank, world)
        loc = part.local
        rng = np.random.default_rng(7)
        a = rng.standard_normal(m.shape)
        gs = part.global_sum(a[loc], dist)
        d = part.dot(a[loc], a[loc], dist)
        X, Y = m.node_coords()
        V = X * X + Y * Y
        alpha = 0.005
        op = _local_res(m, V, alpha)
        fr, fi = m.schro_f(V, np.exp(-X * X - Y * Y) * np.cos(3 * X), np.exp(-X * X - Y * Y) * np.sin(3 * X))
        b = (0.005 * fr[loc], 0.005 * fi[loc])
        A = part.operator(lambda u: op(u, loc), dist)
        x, ok, it, res = P.minres(part, A, b, 2000, 1e-10, dist)
        q.put((rank, "ok", (loc, gs, d, x, ok, it)))
    except Exception as e:
        q.put((rank, "error", repr(e)))
    finally:
        dist.destroy_process_group()


def _run(world):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(world):
        r, status, v = q.get(timeout=300)
        out[r] = (status, v)
    for p in procs:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    return out


@pytest.mark.parametrize("world", [2, 4])
def test_distributed_ops_and_minres_gloo(oracle, world):
    m, co, el = _mesh(oracle, "jit", 4)
    rng = np.random.default_rng(7)
    a = rng.standard_normal(m.shape)
    ref_gs = m.global_sum(a)
    X, Y = m.node_coords()
    V = X * X + Y * Y
    fr, fi = m.schro_f(V, np.exp(-X * X - Y * Y) * np.cos(3 * X), np.exp(-X * X - Y * Y) * np.sin(3 * X))
    b = (0.005 * fr, 0.005 * fi)
    n = m.n_el * m.N * m.N
    # the oracle's MINRES (the reference's algorithm) on the same operator, one process
    apply = lambda v: np.concatenate([t.ravel() for t in m.schro_res(V, 0.005, v[:n].reshape(m.shape),  # noqa: E731
                                                                     v[n:].reshape(m.shape))])
    dot = lambda u, v: m.dot(u[:n].reshape(m.shape), v[:n].reshape(m.shape)) + \
        m.dot(u[n:].reshape(m.shape), v[n:].reshape(m.shape))  # noqa: E731
    xo, (oko, ito, _) = oracle.krylov("minres", apply, np.concatenate([b[0].ravel(), b[1].ravel()]),
                                      np.zeros(2 * n), 2000, 1e-10, dot)
    out = _run(world)
    for r in range(world):
        assert out[r][0] == "ok", out[r][1]
    x = (np.zeros(m.shape), np.zeros(m.shape))
    d_sum = None
    for r in range(world):
        loc, gs, d, xr, ok, it = out[r][1]
        assert np.array_equal(gs, ref_gs[loc])  # same bits as one rank
        d_sum = d if d_sum is None else d_sum
        assert d == d_sum  # every rank holds the same all-reduced value
        assert ok and abs(it - ito) <= 1, (it, ito)
        x[0][loc], x[1][loc] = xr
    assert abs(d_sum - m.dot(a, a)) <= 1e-12 * m.dot(a, a)
    xo0, xo1 = xo[:n].reshape(m.shape), xo[n:].reshape(m.shape)
    err = max(np.linalg.norm(x[0] - xo0) / np.linalg.norm(xo0), np.linalg.norm(x[1] - xo1) / np.linalg.norm(xo1))
    assert oko and err < 1e-9, err
