"""The seeded scene generators start without overlaps (CPU).

An overlap at t = 0 is a contact the reference would never have let form; with stiff Hertz
contacts it blows the packing up in a few steps.  Clearances are computed with the reference's
own contact geometry: sphere-sphere centre distance; the rounded-slab plate of
CDSphere2QuasiPlate.cpp:15-97 (closest point of the mid-plane rectangle); the rod of
CDSphere2QuasiCylinder.cpp:16-80 (closest point of the axis segment)."""
import numpy as np
import pytest

from vedo_gb300 import scenes
from vedo_gb300.scene import INNER_CYLINDER, QUASI_CYLINDER, QUASI_PLATE, SPHERE

spatial = pytest.importorskip("scipy.spatial")


def _unit(v):
    return v / np.linalg.norm(v)


def min_clearance(sc):
    kind = np.array([sc.models[m].shape for m in sc.model_index])
    sph = np.flatnonzero(kind == SPHERE)
    P = sc.position[sph]
    r = np.array([sc.models[sc.model_index[i]].attrs[0] for i in sph])
    gaps = []
    tree = spatial.cKDTree(P)
    pairs = tree.query_pairs(2.0 * r.max() * 1.001, output_type="ndarray")
    if len(pairs):
        d = np.linalg.norm(P[pairs[:, 0]] - P[pairs[:, 1]], axis=1) - r[pairs[:, 0]] - r[pairs[:, 1]]
        gaps.append(d.min())
    for w in np.flatnonzero(kind != SPHERE):
        m = sc.models[sc.model_index[w]]
        c, oz = sc.position[w], _unit(sc.orientation_z[w])
        if m.shape == QUASI_PLATE:
            ox = _unit(sc.orientation_x[w])
            oy = np.cross(oz, ox)
            width, height, length = m.attrs[:3]
            q = P - c
            dx = np.clip(q @ ox, -0.5 * width, 0.5 * width)
            dy = np.clip(q @ oy, -0.5 * length, 0.5 * length)
            closest = c + dx[:, None] * ox + dy[:, None] * oy
            gaps.append((np.linalg.norm(P - closest, axis=1) - r - 0.5 * height).min())
        elif m.shape == QUASI_CYLINDER:
            rc, h = m.attrs[:2]
            t = np.clip((P - c) @ oz, -0.5 * h, 0.5 * h)
            closest = c + t[:, None] * oz
            gaps.append((np.linalg.norm(P - closest, axis=1) - r - rc).min())
        elif m.shape == INNER_CYLINDER:              # inside the shell: R - axis distance - r
            rc = m.attrs[0]
            t = (P - c) @ oz
            gaps.append((rc - np.linalg.norm((P - c) - t[:, None] * oz, axis=1) - r).min())
    return min(gaps)


@pytest.mark.parametrize("name,make", [
    ("lsd_box", lambda: scenes.lsd_box(n_side=10)),
    ("hertz_drum", lambda: scenes.hertz_drum(n=20000, seed=3)),
    ("hopper", lambda: scenes.hopper(n=3000, seed=1)),
    ("settle_lsd", lambda: scenes.serving_job("settle", 3000, "lsd", 1)),
    ("projectile_hertz", lambda: scenes.serving_job("projectile", 3000, "hertz", 2)),
    ("compressed_bed", lambda: scenes.compressed_bed(n=50000, box=0.06, cylinders=4, packing="fcc")),
])
def test_scene_starts_without_overlaps(name, make):
    assert min_clearance(make()) > 0.0, name


def test_drum_has_a_largest_sphere_last():
    """The reference's NBS cell size comes from the last local object's radius
    (NBSConsultant.cpp:140); the drum generator puts a largest-class sphere there."""
    sc = scenes.hertz_drum(n=20000, seed=3)
    r = np.array([sc.models[m].attrs[0] if sc.models[m].shape == SPHERE else 0.0 for m in sc.model_index])
    last_sphere = np.flatnonzero(r > 0)[-1]
    assert r[last_sphere] == r.max()


@pytest.mark.parametrize("name,make", [
    ("compressed_bed", lambda: scenes.compressed_bed(n=50000, box=0.06, cylinders=4)),
    ("hopper", lambda: scenes.hopper(n=3000, seed=1, touching=True)),
])
def test_touching_packings_touch_without_overlap(name, make):
    """The contact-bearing stand-ins (a simple cubic lattice whose neighbours, floor and walls
    touch): every sphere's nearest neighbour lies at 2 r to rounding, and no wall overlaps."""
    sc = make()
    sph = np.array([sc.models[m].shape == SPHERE for m in sc.model_index])
    p = sc.position[sph]
    r = sc.models[sc.model_index[np.flatnonzero(sph)[0]]].attrs[0]
    d, _ = spatial.cKDTree(p).query(p, k=2)
    np.testing.assert_allclose(d[:, 1], 2 * r, rtol=1e-12)
    assert min_clearance(sc) > -1e-12 * r, name
