"""Periodic boundaries in the mixed form: sphere pairs take the nearest periodic image (prefilter,
neighbour cells that wrap around the box, double-float exact path, the FP64 tie band), and mobile
spheres go back into the box after every step with the reference's wrap
(Boundary::EnforceBoundaryConditions, Boundary.cpp:225-304).  Its lists are complete across the
faces, as the FP64 form's Leap consultant's are (LeapConsultant.h:147-446), so at identical states
the contact sets are that form's and the per-step impulses agree within 1e-5 relative; every form
of the tick gives the same bits.  The reference's Leap list holds some pairs twice on a periodic
axis (70 of 6,362 candidates in the layer below: a zone adjacent to another both directly and
through the periodic image), and a pair listed twice is applied twice there; the mixed form
applies each pair once, so the spheres of such pairs are left out of the impulse comparison."""
import os
import tempfile

import numpy as np
import pytest

from vedo_gb300 import scenes
from vedo_gb300.scene import SPHERE

pytestmark = pytest.mark.gpu


def _active(e):
    it = e.interactions()
    a = it["active"] == 1
    return set(zip(it["first"][a].tolist(), it["second"][a].tolist()))


def _layer(solver):
    return scenes.periodic_layer(nx=12, ny=12, layers=4, seed=21, steps=2000, solver=solver)


@pytest.mark.parametrize("solver", ["ISwBSDBF", "ISwHertz", "ISwH"])
def test_mixed_periodic_against_fp64_leap(solver, engine_lib):
    f64 = engine_lib.GpuEngine(_layer(solver), up_iact=5, consultant="leap")
    f64.run(150)                                   # spheres have crossed the faces, contacts formed
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "p.ido")
        f64.write_ido(path)
        a = engine_lib.GpuEngine(path, up_iact=5, consultant="leap")
        b = engine_lib.GpuEngine(path, up_iact=5, precision=1)
    A, B = _active(a), _active(b)
    assert len(A) > 20
    assert A == B
    # the spheres of active pairs that the Leap list holds more than once
    it = a.interactions()
    act = it["active"] == 1
    keys = [tuple(sorted(p)) for p in zip(it["first"][act].tolist(), it["second"][act].tolist())]
    twice = {p for p in keys if keys.count(p) > 1}
    skip = np.zeros(a.n, bool)
    for p, q in twice:
        skip[p] = skip[q] = True
    a.run(1)
    b.run(1)
    sa, sb = a.state(), b.state()
    for k in ("impact", "angular_impact"):
        x, y = sa[k][~skip], sb[k][~skip]
        ref = np.linalg.norm(x)
        assert np.linalg.norm(x - y) <= 1e-5 * ref + 1e-30, k
    assert np.linalg.norm(sa["impact"][~skip]) > 0


def test_mixed_periodic_forms_agree_and_stay_in_the_box(engine_lib):
    sc = _layer("ISwH")
    forms = [engine_lib.GpuEngine(sc, precision=1, **kw)
             for kw in ({}, {"split_tick": True}, {"pair_pass": True}, {"stored_splits": True, "pair_pass": True},
                        {"skin": 0.02, "check_interval": 1})]
    for n in (7, 1, 93, 150, 49):
        for e in forms:
            e.run(n)
        ref = forms[0].state()
        for e in forms[1:]:
            st = e.state()
            for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
                assert np.array_equal(st[k], ref[k]), k
    sph = np.array([sc.models[m].shape == SPHERE for m in sc.model_index])
    x0 = sc.position[sph]
    p = forms[0].state(("position",))["position"][sph]
    b = sc.sp.pbc
    for k in (0, 1):
        assert np.all((p[:, k] >= b.lower[k]) & (p[:, k] < b.upper[k]))
    assert np.sum(p[:, 0] < x0[:, 0] - 0.5 * (b.upper[0] - b.lower[0])) > 10   # out at the upper x face
    assert (forms[0].interactions()["active"] == 1).sum() > 20


def test_mixed_periodic_batch_equals_alone(engine_lib):
    scs = [_layer("ISwBSDBF"), scenes.cluster(n=64, solver="ISwBSDBF", seed=21), _layer("ISwHertz")]
    batch = engine_lib.BatchEngine(scs)
    batch.run(200)
    for q, sc in enumerate(scs):
        e = engine_lib.GpuEngine(sc, precision=1)
        e.run(200)
        st, sb = e.state(), batch.scene_state(q)
        for k in ("position", "velocity", "angular_velocity"):
            assert np.array_equal(st[k], sb[k]), (q, k)
        e.close()
    batch.close()
