"""Whole-run agreement on the 8,000-sphere linear spring-dashpot box (20,000 steps, dt 1e-6 s,
candidate list rebuilt every 20 steps) against the reference's own run of the same seeded scene
(tests/golden/wholerun/lsd_box.npz, made by tests/golden/wholerun/make_wholerun.py).

* FP64 form: the state after every 500 steps has the reference's SHA-256 (bit for bit), so
  kinetic energy, centre of mass, contact count and coordination number are the reference's.
* Mixed form: granular trajectories are chaotic, so the comparison is pointwise only for the
  first 100 steps (positions within 1e-12 m, velocities within 1e-7 relative) and, over the whole
  run, through the observables: translational kinetic energy within 2 % of the reference's
  (plus 1e-9 J for the nearly still end of the run), rotational kinetic energy within 10 % of the
  translational scale, centre of mass within 5 um, the average coordination number within 0.1,
  active contacts within 5 % (plus 20).
"""
import hashlib
import os

import numpy as np
import pytest

from vedo_gb300 import scenes

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "wholerun", "lsd_box.npz")


def _digest(st):
    h = hashlib.sha256()
    for k in ("position", "velocity", "angular_velocity"):
        h.update(np.ascontiguousarray(st[k], dtype="<f8").tobytes())
    return h.hexdigest()


def _observables(scene, st):
    from vedo_gb300.scene import SPHERE
    m = np.array([scene.models[k].analysis()[2] if scene.models[k].shape == SPHERE else 0.0
                  for k in scene.model_index])
    inertia = np.array([scene.models[k].analysis()[4][0] if scene.models[k].shape == SPHERE else 0.0
                        for k in scene.model_index])
    v, w, p = st["velocity"], st["angular_velocity"], st["position"]
    ke_t = float(np.sum(0.5 * m * np.sum(v * v, axis=1)))
    ke_r = float(np.sum(0.5 * inertia * np.sum(w * w, axis=1)))
    com = (m[:, None] * p).sum(axis=0) / m.sum()
    return ke_t, ke_r, com


def _run(engine_lib, precision):
    g = np.load(FIX)
    sc = scenes.lsd_box(steps=int(g["steps"]))
    e = engine_lib.GpuEngine(sc, up_iact=int(g["up_iact"]), precision=precision)
    box = tuple(g["box"])
    rows, digests, first = [], [], None
    done = 0
    for target in g["table"][:, 0].astype(int):
        e.run(int(target) - done)
        done = int(target)
        st = e.state(("position", "velocity", "angular_velocity"))
        if done == 100:
            first = st
        ke_t, ke_r, com = _observables(sc, st)
        contacts = int(e.observables()[9])
        cn = e.coordination(box)[2]
        rows.append([done, ke_t, ke_r, com[0], com[1], com[2], contacts, cn])
        digests.append(_digest(st))
    e.close()
    return g, np.array(rows), digests, first


def test_fp64_whole_run_is_the_reference_bit_for_bit(engine_lib):
    g, rows, digests, first = _run(engine_lib, 0)
    for k in ("position", "velocity", "angular_velocity"):
        np.testing.assert_array_equal(first[k], g[f"first100_{k}"], err_msg=k)
    bad = [int(r[0]) for r, a, b in zip(rows, digests, g["digests"]) if a != str(b)]
    assert not bad, f"state differs from the reference's at steps {bad[:5]}"
    np.testing.assert_array_equal(rows, g["table"])


def test_mixed_whole_run_observables_within_stated_tolerances(engine_lib):
    g, rows, _, first = _run(engine_lib, 1)
    ref = g["table"]
    np.testing.assert_allclose(first["position"], g["first100_position"], rtol=0, atol=1e-12)
    v0 = g["first100_velocity"]
    np.testing.assert_allclose(first["velocity"], v0, rtol=0, atol=1e-7 * np.abs(v0).max())
    ke_scale = ref[:, 1].max()
    for r, q in zip(rows, ref):
        step = int(q[0])
        assert abs(r[1] - q[1]) <= 0.02 * q[1] + 1e-9, (step, "translational KE", r[1], q[1])
        assert abs(r[2] - q[2]) <= 0.1 * ke_scale, (step, "rotational KE", r[2], q[2])
        assert np.all(np.abs(r[3:6] - q[3:6]) <= 5e-6), (step, "centre of mass", r[3:6], q[3:6])
        assert abs(r[6] - q[6]) <= 0.05 * q[6] + 20, (step, "active contacts", r[6], q[6])
        assert abs(r[7] - q[7]) <= 0.1, (step, "coordination number", r[7], q[7])
