"""Helpers shared by the test modules."""
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
SMALL_MESH = os.path.join(GOLDEN, "small_mesh")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def structured(n, box=(0.0, 1.0, 0.0, 1.0), jitter=0.15, seed=0):
    from schrodingersem_gb300.meshgen import structured_quads
    return structured_quads(n, box=box, jitter=jitter, seed=seed)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))
