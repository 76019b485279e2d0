"""Whole-run fixture of the 8,000-sphere linear spring-dashpot box, made by the reference itself.

Runs the reference DEM CPU path (compiled from its sources by ``make -C oracle ref``; needs
the reference checkout, default /root/reference or $VEDO_REFERENCE) on the seeded
`scenes.lsd_box()` scene (8,000 spheres, r = 1 mm, 5 fixed plates, ISwBSDBF, dt = 1e-6 s)
for the full 20,000 steps with the candidate list rebuilt every 20 steps, and stores:

* every SAMPLE steps: a SHA-256 of the state bytes (position, velocity, angular velocity,
  [n][3] FP64 little endian), translational and rotational kinetic energy (sum of 1/2 m v^2
  and 1/2 I w^2 over the spheres), the mass-weighted centre, the number of active contacts,
  and the average coordination number of the reference's CalcCoordinateNum over a box that
  holds the whole scene;
* the full state after the first 100 steps (pointwise comparison);

    python tests/golden/wholerun/make_wholerun.py          # -> tests/golden/wholerun/lsd_box.npz
"""
import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

from vedo_gb300 import scenes  # noqa: E402
from vedo_gb300.scene import Scene  # noqa: E402

STEPS = 20000
SAMPLE = 500
UP_IACT = 20
BOX = (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)


def state_digest(st):
    """SHA-256 over position, velocity and angular velocity as [n][3] little-endian doubles."""
    h = hashlib.sha256()
    for k in ("position", "velocity", "angular_velocity"):
        h.update(np.ascontiguousarray(st[k], dtype="<f8").tobytes())
    return h.hexdigest()


def sphere_observables(scene, st):
    """Kinetic energies and the mass-weighted centre of the spheres (mass and moment of
    inertia of each sphere's model, DOModel::Analysis)."""
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


def main():
    import oracle
    oracle.build_ref()
    from oracle import RefWorld, ref_coordination
    sc = scenes.lsd_box(steps=STEPS)
    w = RefWorld(sc, up_iact=UP_IACT)
    rows, digests = [], []
    first = None
    done = 0
    while done < STEPS:
        k = 100 if done == 0 else SAMPLE - (100 if done == 100 else 0)
        w.run(k)
        done += k
        st = w.state()
        if done == 100:
            first = st
        if done % SAMPLE and done != 100:
            continue
        ke_t, ke_r, com = sphere_observables(sc, st)
        it = w.interactions()
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "s.ido")
            w.write_ido(path)
            cn = ref_coordination(Scene.from_ido(path), BOX)
        rows.append([done, ke_t, ke_r, com[0], com[1], com[2], int(it["active"].sum()), cn])
        digests.append(state_digest(st))
        print(done, rows[-1][1:], digests[-1][:16], flush=True)
    w.close()
    np.savez_compressed(os.path.join(HERE, "lsd_box.npz"), steps=STEPS, up_iact=UP_IACT,
                        sample=SAMPLE, box=np.array(BOX), table=np.array(rows, dtype=np.float64),
                        digests=np.array(digests),
                        **{f"first100_{k}": first[k] for k in ("position", "velocity", "angular_velocity")})


if __name__ == "__main__":
    main()
