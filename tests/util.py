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


def det_field(shape, seed: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    """Pseudo-random float64 field from integer arithmetic only (SplitMix64 of
    the flat index and the seed), so the same inputs arise on every host and
    numpy version; used for the inputs of the reference fixtures."""
    n = int(np.prod(shape))
    with np.errstate(over="ignore"):
        z = np.arange(n, dtype=np.uint64) + np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15)
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return (lo + (hi - lo) * u).reshape(shape)


REF_GOLDEN = os.path.join(GOLDEN, "ref")

# meshes of the reference fixtures (tests/golden/make_ref_golden.py)
REF_MESHES = {
    "jit8": dict(n=8, box=(-4.0, 4.0, -4.0, 4.0), jitter=0.1, seed=1),
    "c1": dict(n=16, box=(0.0, 1.0, 0.0, 1.0), jitter=0.15, seed=0),
}


def ref_mesh_arrays(name: str):
    m = REF_MESHES[name]
    return structured(m["n"], box=m["box"], jitter=m["jitter"], seed=m["seed"])


def load_ref_fixture(name: str) -> dict:
    with np.load(os.path.join(REF_GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}
