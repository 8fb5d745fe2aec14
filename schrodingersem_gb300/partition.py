"""Element partition of one mesh across ranks: the host side of a
partitioned multi-GPU run (the reference's ``include/mpi_impl``).

* ``pca_bisection`` splits the elements into P = 2^k groups by recursive
  median bisection of the element centres along their first principal
  direction (include/mpi_impl/distribute_mesh.hpp:82-132).
* ``Partition`` derives, from the global topology (element corner ids) and
  the element-to-rank map, every rank's elements and its interface with each
  other rank, then provides the three operations a Krylov solve needs across
  ranks, on a rank's element-local fields (E_r, N, N) in the reference's
  layout:

  - ``global_sum``: every copy of a shared node receives the sum of all its
    copies, formed from 0 in ascending global element order, which is the
    reference's ``connected_elements`` order for corners
    (include/openmp_impl/global_sum.hpp:56-59) and owner + other for sides,
    so every rank, and a single-rank run, obtain the same bits
    (include/mpi_impl/global_sum.hpp:78-245 exchanges the same values);
  - ``mask``: zero on the Dirichlet boundary and on every copy but the
    owner's (the copy of the lowest element id);
  - ``dot``: the unique-DOF dot (owner copies), summed on each rank and
    all-reduced (include/mpi_impl/dot.hpp:11-68).

  The exchange sends, to each neighbouring rank, this rank's copies of the
  nodes the two share, in one canonical order both sides derive from the
  global topology: one message per neighbour and direction.
* ``minres`` is include/minres.hpp:19-107 over those operations, for an
  operator given as a rank-local element kernel: A x = mask(global_sum(
  local_op(global_sum(x)))) on masked vectors (unmask equals global_sum on
  a masked vector).

Communication goes through ``torch.distributed`` point-to-point and
all-reduce calls (NCCL between GPUs, gloo between CPU processes).  This
module is the host logic only: the tests run it across CPU ranks with a
NumPy element kernel; the library's per-rank device kernels are not wired to
it.
"""
from __future__ import annotations

from collections import defaultdict
from typing import Callable

import numpy as np


# ------------------------------------------------------------------ partition
def pca_bisection(centres: np.ndarray, P: int) -> np.ndarray:
    """element -> group in [0, P), P a power of two: a queue of (range, parts)
    halves each range at the median of the projection on the range's first
    principal direction; the upper half takes the next new label"""
    n = centres.shape[0]
    if P < 1 or (P & (P - 1)):
        raise ValueError("P must be a power of two")
    order = np.arange(n)
    label = np.zeros(n, dtype=np.int64)
    queue = [(0, n, P)]
    nxt = 1
    while queue and P > 1:
        first, last, p = queue.pop(0)
        idx = order[first:last]
        c = centres[idx]
        d = c - c.mean(axis=0)
        cov = d.T @ d / max(1, len(idx) - 1)
        w, v = np.linalg.eigh(cov)
        u = v[:, np.argmax(w)]
        if u[1] < 0 or (u[1] == 0 and u[0] < 0):  # one sign on every host
            u = -u
        pc = d @ u
        mid = (first + last) // 2
        # stable: ties by element id, so every rank derives the same split
        srt = np.lexsort((idx, pc))
        order[first:last] = idx[srt]
        label[order[mid:last]] = nxt
        nxt += 1
        if p > 2:
            queue.append((first, mid, p // 2))
            queue.append((mid, last, p // 2))
    return label


def element_centres(coords: np.ndarray, elements: np.ndarray) -> np.ndarray:
    return coords[elements].mean(axis=1)


# ------------------------------------------------------------------ topology
def _node_keys(elements: np.ndarray, N: int):
    """global node id of every element-local slot (E, N, N) and boundary flag
    per node.  Slot (i, j) of element e; corners 0..3 at (0,0), (N-1,0),
    (N-1,N-1), (0,N-1); sides j=0, i=N-1, j=N-1, i=0 between those corners."""
    E = elements.shape[0]
    key = np.full((E, N, N), -1, dtype=np.int64)
    corner_pos = [(0, 0), (N - 1, 0), (N - 1, N - 1), (0, N - 1)]
    nodes: dict = {}
    side_count: dict = defaultdict(int)
    for e in range(E):
        c = elements[e]
        for s in range(4):
            a, b = int(c[s]), int(c[(s + 1) % 4])
            side_count[(min(a, b), max(a, b))] += 1

    def nid(k):
        v = nodes.get(k)
        if v is None:
            v = nodes[k] = len(nodes)
        return v

    for e in range(E):
        c = elements[e]
        for q, (i, j) in enumerate(corner_pos):
            key[e, j, i] = nid(("c", int(c[q])))
        for s in range(4):
            a, b = int(c[s]), int(c[(s + 1) % 4])
            (i0, j0), (i1, j1) = corner_pos[s], corner_pos[(s + 1) % 4]
            for t in range(1, N - 1):
                i = i0 + (i1 - i0) * t // (N - 1)
                j = j0 + (j1 - j0) * t // (N - 1)
                tt = t if a < b else N - 1 - t  # position counted from the smaller corner id
                key[e, j, i] = nid(("s", min(a, b), max(a, b), tt))
        for j in range(1, N - 1):
            for i in range(1, N - 1):
                key[e, j, i] = nid(("i", e, i, j))
    bnd = np.zeros(len(nodes), dtype=bool)
    for (a, b), cnt in side_count.items():
        if cnt == 1:  # boundary side: its nodes and both corners
            bnd[nodes[("c", a)]] = bnd[nodes[("c", b)]] = True
            for t in range(1, N - 1):
                bnd[nodes[("s", a, b, t)]] = True
    return key, bnd


class Partition:
    """one rank's view of a partitioned mesh (see the module docstring)"""

    def __init__(self, elements: np.ndarray, N: int, labels: np.ndarray, rank: int, world: int):
        elements = np.ascontiguousarray(elements, dtype=np.int64).reshape(-1, 4)
        self.N, self.rank, self.world = int(N), int(rank), int(world)
        labels = np.asarray(labels, dtype=np.int64)
        key, bnd = _node_keys(elements, self.N)
        E = elements.shape[0]
        self.local = np.flatnonzero(labels == rank)          # global ids of this rank's elements
        self.E = len(self.local)
        flat_key = key.reshape(E, -1)
        # copies of every node: (element, slot) in ascending element order
        order = np.argsort(flat_key.ravel(), kind="stable")
        keys_sorted = flat_key.ravel()[order]
        starts = np.flatnonzero(np.r_[True, keys_sorted[1:] != keys_sorted[:-1]])
        counts = np.diff(np.r_[starts, keys_sorted.size])
        el_of = order // (self.N * self.N)
        slot_of = order % (self.N * self.N)
        lpos = -np.ones(E, dtype=np.int64)
        lpos[self.local] = np.arange(self.E)
        nl = self.N * self.N
        # per shared node (2+ copies) touching this rank: the canonical list of
        # copies (global element order), each as (rank, local flat index)
        self._sum_nodes = []  # (list of (src, idx)) per node; src -1 local, else peer rank
        self._targets = []    # local flat indices that receive the node's sum
        send = defaultdict(list)   # peer -> local flat indices sent, canonical order
        recv = defaultdict(int)    # peer -> number of values received
        owner_local = np.zeros(self.E * nl, dtype=bool)
        bnd_local = np.zeros(self.E * nl, dtype=bool)
        for s0, cnt in zip(starts, counts):
            g = keys_sorted[s0]
            els = el_of[s0:s0 + cnt]
            slots = slot_of[s0:s0 + cnt]
            ranks = labels[els]
            mine = ranks == rank
            if not mine.any():
                continue
            # owner: the copy of the lowest element id (els ascending)
            if mine[0]:
                owner_local[lpos[els[0]] * nl + slots[0]] = True
            if bnd[g]:  # Dirichlet boundary: masked, never summed (global_sum.hpp)
                bnd_local[lpos[els[mine]] * nl + slots[mine]] = True
                continue
            if cnt < 2:
                continue
            peers = sorted(set(int(r) for r in ranks[~mine]))
            copies = []
            for e_, s_, r_ in zip(els, slots, ranks):
                if r_ == rank:
                    copies.append((-1, int(lpos[e_] * nl + s_)))
                else:
                    copies.append((int(r_), recv[int(r_)]))
                    recv[int(r_)] += 1
            for q in peers:
                send[q].extend(int(lpos[e_] * nl + s_) for e_, s_ in zip(els[mine], slots[mine]))
            self._sum_nodes.append(copies)
            self._targets.append(np.array([c[1] for c in copies if c[0] == -1], dtype=np.int64))
        self.peers = sorted(set(send) | set(recv))
        self._send = {q: np.array(send[q], dtype=np.int64) for q in self.peers}
        self._recv = {q: int(recv[q]) for q in self.peers}
        self._owner = owner_local
        self._keep = owner_local & ~bnd_local
        self._bnd = bnd_local

    # ---------------------------------------------------------- operations
    def shape(self):
        return (self.E, self.N, self.N)

    def _exchange(self, flat: np.ndarray, dist):
        import torch
        if not self.peers:
            return {}
        reqs, bufs = [], {}
        for q in self.peers:
            out = torch.from_numpy(np.ascontiguousarray(flat[self._send[q]]))
            bufs[q] = torch.empty(self._recv[q], dtype=torch.float64)
            reqs.append(dist.isend(out, dst=q))
            reqs.append(dist.irecv(bufs[q], src=q))
        for r in reqs:
            r.wait()
        return {q: b.numpy() for q, b in bufs.items()}

    def global_sum(self, a: np.ndarray, dist=None) -> np.ndarray:
        """every copy of a shared interior node gets the sum of all its copies;
        boundary copies stay as they are (include/openmp_impl/global_sum.hpp)"""
        flat = np.ascontiguousarray(a, dtype=np.float64).reshape(-1).copy()
        got = self._exchange(flat, dist) if self.world > 1 else {}
        src = flat.copy()
        for copies, tgt in zip(self._sum_nodes, self._targets):
            s = 0.0
            for r, i in copies:
                s += src[i] if r < 0 else got[r][i]
            flat[tgt] = s
        return flat.reshape(self.shape())

    def mask(self, a: np.ndarray) -> np.ndarray:
        """zero on the boundary and on every copy but the owner's"""
        flat = np.ascontiguousarray(a, dtype=np.float64).reshape(-1).copy()
        flat[~self._keep] = 0.0
        return flat.reshape(self.shape())

    def dot(self, a: np.ndarray, b: np.ndarray, dist=None) -> float:
        fa, fb = np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)
        s = float(np.dot(fa[self._owner], fb[self._owner]))
        if self.world > 1:
            import torch
            t = torch.tensor([s], dtype=torch.float64)
            dist.all_reduce(t)
            s = float(t.item())
        return s

    def operator(self, local_op: Callable, dist=None):
        """x (masked, tuple of planes) -> mask(global_sum(local_op(unmask x)))"""
        def A(x):
            u = tuple(self.global_sum(p, dist) for p in x)
            y = local_op(u)
            return tuple(self.mask(self.global_sum(p, dist)) for p in y)
        return A


def minres(part: Partition, A: Callable, b, maxit: int, tol: float, dist=None):
    """include/minres.hpp:19-107 (identity preconditioner) on tuples of
    element-local planes, with the partition's dot; x0 = 0.  Returns
    (x, success, n_iter, residual estimate)."""
    def dot(u, v):
        return sum(part.dot(p, q, dist) for p, q in zip(u, v))

    def lin(*terms):
        return tuple(sum(c * t[k] for c, t in terms) for k in range(len(terms[0][1])))

    x = tuple(np.zeros_like(p) for p in b)
    r1 = tuple(p.copy() for p in b)
    y = r1
    beta = np.sqrt(dot(r1, y))
    bnorm = beta
    r2 = r1
    oldb, dbar, epsln, phibar, cs, sn = 0.0, 0.0, 0.0, beta, -1.0, 0.0
    w = tuple(np.zeros_like(p) for p in b)
    w2 = w
    eps = np.finfo(np.float64).eps
    for it in range(1, maxit + 1):
        s = 1.0 / beta
        v = lin((s, y))
        y = A(v)
        if it >= 2:
            y = lin((1.0, y), (-beta / oldb, r1))
        alpha = dot(v, y)
        y = lin((1.0, y), (-alpha / beta, r2))
        r1, r2 = r2, y
        oldb, beta = beta, np.sqrt(dot(r2, y))
        oldeps = epsln
        delta = cs * dbar + sn * alpha
        gbar = sn * dbar - cs * alpha
        epsln = sn * beta
        dbar = -cs * beta
        gamma = max(np.sqrt(gbar * gbar + beta * beta), eps)
        cs, sn = gbar / gamma, beta / gamma
        phi = cs * phibar
        phibar *= sn
        w1, w2 = w2, w
        w = tuple((1.0 / gamma) * ((vk - oldeps * a1) - delta * a2) for vk, a1, a2 in zip(v, w1, w2))
        x = tuple(xk + phi * wk for xk, wk in zip(x, w))
        if phibar < tol * bnorm + tol:
            return x, True, it, phibar
    return x, False, maxit + 1, phibar
