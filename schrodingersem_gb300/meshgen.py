"""Synthetic meshes and fields in the reference's formats.

Meshes are n x n structured bilinear quads on a box with every interior
vertex jittered by an independent uniform offset in [-a*h, a*h] per
coordinate (numpy PCG64 seeded generator).  Elements list their corners
counter-clockwise (bottom-left, bottom-right, top-right, top-left), the
order ``load_mesh`` expects (include/load_mesh.hpp:65-71).

``write_mesh_folder`` / ``read_mesh_folder`` speak the reference's folder
format: ``info.txt`` ("n_nodes n_elements"), ``coordinates.txt`` (x y per
line) and ``elements.txt`` (4 corner ids per line).
"""
from __future__ import annotations

import os

import numpy as np


def structured_quads(n: int, box=(0.0, 1.0, 0.0, 1.0), jitter: float = 0.0, seed: int = 0):
    """Return (coords [(n+1)^2, 2] float64, elements [n^2, 4] int32)."""
    x0, x1, y0, y1 = box
    hx = (x1 - x0) / n
    hy = (y1 - y0) / n
    jj, ii = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    X = x0 + ii * hx
    Y = y0 + jj * hy
    rng = np.random.Generator(np.random.PCG64(seed))
    d = rng.uniform(-1.0, 1.0, size=(n + 1, n + 1, 2))
    interior = (ii > 0) & (ii < n) & (jj > 0) & (jj < n)
    X = np.where(interior, X + jitter * hx * d[..., 0], X)
    Y = np.where(interior, Y + jitter * hy * d[..., 1], Y)
    coords = np.stack([X.reshape(-1), Y.reshape(-1)], axis=1).astype(np.float64)
    v = lambda i, j: j * (n + 1) + i  # noqa: E731
    el = []
    for j in range(n):
        for i in range(n):
            el.append((v(i, j), v(i + 1, j), v(i + 1, j + 1), v(i, j + 1)))
    return coords, np.asarray(el, dtype=np.int32)


def write_mesh_folder(folder: str, coords: np.ndarray, elements: np.ndarray) -> None:
    os.makedirs(folder, exist_ok=True)
    with open(os.path.join(folder, "info.txt"), "w") as f:
        f.write(f"{coords.shape[0]} {elements.shape[0]}")
    np.savetxt(os.path.join(folder, "coordinates.txt"), coords, fmt="%.18e")
    np.savetxt(os.path.join(folder, "elements.txt"), elements, fmt="%d")


def read_mesh_folder(folder: str):
    with open(os.path.join(folder, "info.txt")) as f:
        n_nodes, n_el = (int(t) for t in f.read().split()[:2])
    coords = np.loadtxt(os.path.join(folder, "coordinates.txt"), dtype=np.float64).reshape(-1, 2)[:n_nodes]
    elements = np.loadtxt(os.path.join(folder, "elements.txt"), dtype=np.int64).reshape(-1, 4)[:n_el]
    return np.ascontiguousarray(coords), np.ascontiguousarray(elements.astype(np.int32))


def element_node_coords(coords: np.ndarray, elements: np.ndarray, z: np.ndarray):
    """Physical (x, y) of every element-local node, shape (E, N, N) indexed
    [e, j, i] -- the bilinear map of include/Quad.hpp:57-62."""
    xs = coords[elements, 0]  # [E, 4]
    ys = coords[elements, 1]
    xi = z[None, None, :]   # i index (last axis)
    eta = z[None, :, None]  # j index
    def m(c):
        c = c[:, :, None, None]
        return 0.25 * (c[:, 0] * (1 - xi) * (1 - eta) + c[:, 1] * (1 + xi) * (1 - eta)
                       + c[:, 2] * (1 + xi) * (1 + eta) + c[:, 3] * (1 - xi) * (1 + eta))
    return m(xs), m(ys)


def gaussian_packet(X, Y, center, sigma, k):
    """exp(-|r-r0|^2 / (2 sigma^2)) * exp(i k.r), unnormalised (re, im)."""
    r2 = (X - center[0]) ** 2 + (Y - center[1]) ** 2
    amp = np.exp(-r2 / (2.0 * sigma ** 2))
    ph = k[0] * X + k[1] * Y
    return amp * np.cos(ph), amp * np.sin(ph)


def gaussian_sum_potential(X, Y, rng, box, n_bumps=6, amp=(-20.0, 20.0), width=(0.3, 1.5)):
    """Sum of n_bumps Gaussians, amplitude U(amp), width U(width), centres U(box)."""
    V = np.zeros_like(X)
    x0, x1, y0, y1 = box
    for _ in range(n_bumps):
        A = rng.uniform(*amp)
        w = rng.uniform(*width)
        cx = rng.uniform(x0, x1)
        cy = rng.uniform(y0, y1)
        V += A * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * w * w))
    return V
