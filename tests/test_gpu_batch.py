"""Batched ensembles: every instance of a sem_batch follows the reference's
BDF2 driver (schrodinger.hpp:22-128), so its state matches the
single-instance FP64 driver and the CPU oracle within the solver's
accuracy, with per-instance flags and iteration counts."""
import numpy as np
import pytest

from tests.util import rel_err, structured

pytestmark = pytest.mark.gpu

# (p, n, box half-width, jitter seed, potential scale, packet centre, momentum)
INSTANCES = [(2, 3, 2.0, 1, 1.0, (-0.3, 0.2), (2.0, 0.5)), (4, 5, 3.0, 2, 0.5, (0.5, -0.5), (-1.0, 2.0)),
             (6, 2, 2.5, 3, 2.0, (0.0, 0.3), (1.5, 1.5)), (8, 4, 4.0, 4, 0.25, (-1.0, 0.0), (3.0, 0.0)),
             (4, 7, 4.0, 5, 1.0, (1.0, 1.0), (0.0, -2.0)), (5, 3, 3.0, 6, 0.7, (0.2, -0.8), (-2.0, -1.0)),
             (3, 6, 3.0, 7, 1.5, (-0.5, 0.5), (1.0, -1.0)), (7, 3, 3.5, 8, 0.3, (0.3, 0.3), (2.5, 1.0))]


def _inputs(semlib):
    from schrodingersem_gb300.meshgen import gaussian_packet
    meshes, fields = [], []
    for p, n, h, seed, vs, c, k in INSTANCES:
        co, el = structured(n, box=(-h, h, -h, h), jitter=0.1, seed=seed)
        meshes.append((p, co, el))
        ctx = semlib.Context(p, coords=co, elements=el)
        X, Y = ctx.node_coords()
        re, im = gaussian_packet(X, Y, c, 0.8, k)
        fields.append((ctx, re, im, vs * (X * X + Y * Y)))
    return meshes, fields


def test_batch_bdf2_matches_single_instance_fp64(semlib):
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.batch import Batch
    meshes, fields = _inputs(semlib)
    dt, steps, tol = 5e-3, 5, 1e-10
    T = (steps - 0.5) * dt
    ref = []
    for ctx, re, im, V in fields:
        a, b = re.copy(), im.copy()
        assert ctx.schrodinger("bdf2", a, b, V, T, dt, 20 * ctx.dof(), tol)
        ref.append((a, b))
    B = Batch(meshes)
    B.set_option(capi.OPT_REFINE_TOL_SCALE, 0.1)
    re = [f[1].copy() for f in fields]
    im = [f[2].copy() for f in fields]
    V = [np.ascontiguousarray(f[3]) for f in fields]
    ok = B.bdf2(re, im, V, T, dt, 20 * max(f[0].dof() for f in fields), tol)
    assert all(ok)
    for i in range(len(fields)):
        steps_i, stopped, its = B.instance(i)
        assert steps_i == steps and not stopped and its > 0
        assert max(rel_err(re[i], ref[i][0]), rel_err(im[i], ref[i][1])) < 1e-8, i
    st = B.stats()
    assert st.steps == steps and st.graph_launches == steps and st.graphs_built == 1
    assert st.instance_steps == steps * len(fields)
    for p in {m[0] for m in meshes}:
        assert st.kmax_of_p[p] >= 1
    # a second call with the same arguments replays the captured step
    ok = B.bdf2(re, im, V, T, dt, 20 * max(f[0].dof() for f in fields), tol)
    assert all(ok) and B.stats().graphs_built == 1


def test_batch_bdf2_matches_oracle(semlib, oracle):
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.batch import Batch
    meshes, fields = _inputs(semlib)
    sel = [0, 2, 6]
    dt, steps, tol = 5e-3, 3, 1e-10
    T = (steps - 0.5) * dt
    B = Batch([meshes[i] for i in sel])
    B.set_option(capi.OPT_REFINE_TOL_SCALE, 0.1)
    re = [fields[i][1].copy() for i in sel]
    im = [fields[i][2].copy() for i in sel]
    V = [np.ascontiguousarray(fields[i][3]) for i in sel]
    assert all(B.bdf2(re, im, V, T, dt, 100000, tol))
    for k, i in enumerate(sel):
        p, co, el = meshes[i]
        om = oracle.Mesh(p, coords=co, elements=el)
        a, b, ok = om.schrodinger("bdf2", fields[i][1], fields[i][2], fields[i][3], T, dt, 100000, 1e-13)
        assert ok
        assert max(rel_err(re[k], a), rel_err(im[k], b)) < 1e-8, i


def test_batch_device_fields_and_failure_flags(semlib):
    import torch
    from schrodingersem_gb300.batch import Batch
    meshes, fields = _inputs(semlib)
    B = Batch(meshes[:4])
    re = [torch.as_tensor(f[1], device="cuda") for f in fields[:4]]
    im = [torch.as_tensor(f[2], device="cuda") for f in fields[:4]]
    V = [torch.as_tensor(f[3], device="cuda") for f in fields[:4]]
    # an iteration cap far below what the stage needs: every instance stops
    # after its first step and reports failure, as the reference's driver
    ok = B.bdf2(re, im, V, 3.5e-3 * 5, 3.5e-3, 3, 1e-14)
    assert not any(ok)
    for i in range(4):
        steps_i, stopped, _ = B.instance(i)
        assert stopped and steps_i == 1
    ok = B.bdf2(re, im, V, 3.5e-3 * 2.5, 3.5e-3, 100000, 1e-10)
    assert all(ok)
    assert all(torch.isfinite(x).all() for x in re + im)


def test_batch_rejects_unsupported_degree(semlib):
    from schrodingersem_gb300.batch import Batch
    from schrodingersem_gb300.capi import SemError
    co, el = structured(2)
    with pytest.raises(SemError):
        Batch([(1, co, el)])
    with pytest.raises(SemError):
        Batch([(12, co, el)])
