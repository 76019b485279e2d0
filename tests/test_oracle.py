"""CPU tests: the C oracle against the reference's golden vectors, the .ido format, the
scene generators and the C ABI library's exported symbols.  No GPU needed."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from vedo_gb300 import scenes
from vedo_gb300.scene import Scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))
EXACT_CASES = ("box_lsd", "cluster_ISwBSDBF", "cluster_ISwBtSDBF", "cluster_ISwBSDB2F", "cluster_bsdbf_upiact1",
               "cluster_zoi", "holed_plate_lsd", "periodic_lsd",
               "periodic_far_lsd", "periodic_btsdbf", "periodic_bsdb2f", "leap_box_lsd",
               "leap_periodic_lsd", "leap_periodic_wide", "leap_wide_y", "leap_column_z", "leap_single")


def _name(p):
    return os.path.splitext(os.path.basename(p))[0]


@pytest.mark.parametrize("path", GOLDEN, ids=[_name(p) for p in GOLDEN])
def test_port_matches_reference_golden(path, port_lib):
    """The C restatement reproduces the reference's own outputs: candidate list (order included),
    active set and shear-history pairing exactly; state bit for bit for the linear laws with fixed
    walls, and within 1e-9 relative where libm pow/cos/sin enter (Hertz, ISwH, orbital walls)."""
    from oracle import PortWorld
    g = np.load(path)
    sc = Scene.from_ido(g["ido"].tobytes())
    w = PortWorld(sc, up_iact=int(g["up_iact"]), consultant=str(g["consultant"]) if "consultant" in g else "nbs")
    f0, s0 = w.candidates()
    assert np.array_equal(f0, g["cand0_first"]) and np.array_equal(s0, g["cand0_second"])
    w.run(int(g["steps"]))
    f, s = w.candidates()
    assert np.array_equal(f, g["cand_first"]) and np.array_equal(s, g["cand_second"])
    it = w.interactions()
    assert np.array_equal(it["active"], g["iact_active"])
    assert np.array_equal(it["slave"], g["iact_slave"]) and np.array_equal(it["master"], g["iact_master"])
    assert np.array_equal(it["contact"], g["iact_contact"])
    st = w.state()
    exact = _name(path) in EXACT_CASES
    for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact", "orientation_x",
              "orientation_z"):
        ref = g[f"state_{k}"]
        if exact:
            np.testing.assert_array_equal(st[k], ref, err_msg=k)
        else:
            np.testing.assert_allclose(st[k], ref, rtol=1e-9, atol=1e-12 * (np.abs(ref).max() + 1e-300), err_msg=k)
    if exact:
        np.testing.assert_array_equal(it["shear"], g["iact_shear"])
    else:
        np.testing.assert_allclose(it["shear"], g["iact_shear"], rtol=1e-8, atol=1e-14)
    assert w.time() == float(g["time"])


def test_port_energy_matches_reference(port_lib):
    """DOWorld::CalculateSystemEnergy restated (the reference computes it at the last reset)."""
    from oracle import PortWorld
    g = np.load(os.path.join(ROOT, "tests", "golden", "box_lsd.npz"))
    w = PortWorld(Scene.from_ido(g["ido"].tobytes()), up_iact=int(g["up_iact"]))
    w.run(int(g["steps"]))
    np.testing.assert_array_equal(w.energy(), g["energy"])


def test_ido_roundtrip_bytes():
    """Scene -> .ido -> Scene -> .ido is byte-identical (records included)."""
    sc = scenes.cluster(n=20, solver="ISwH", polydisperse=True, cylinders=2)
    from vedo_gb300.scene import Records
    m = 3
    sc.records = Records(np.array([0, 1, 2], np.uint32), np.array([5, 6, 7], np.uint32),
                         np.array([1, 0, 1], bool), np.array([0, 0, 1], bool), np.arange(m) * 1.5,
                         np.arange(m) * 0.25, np.arange(9.0).reshape(3, 3), np.ones((3, 3)), np.zeros((3, 3)),
                         np.full((3, 3), 2.0), np.full((3, 3), -1.0), np.arange(m) * 1e-6)
    b1 = sc.to_ido()
    sc2 = Scene.from_ido(b1)
    assert sc2.to_ido() == b1
    assert len(sc2.records) == 3 and sc2.records.contact.tolist() == [True, False, True]


def test_golden_ido_parses():
    """Every fixture's .ido (written by our writer, read by the reference when the fixtures were
    made) parses back into the same object count and models (less the objects a zone of interest
    erased before the first step)."""
    for p in GOLDEN:
        g = np.load(p)
        sc = Scene.from_ido(g["ido"].tobytes())
        if not sc.sp.zoi.active:
            assert sc.num_objects == g["state_position"].shape[0]
        else:
            assert sc.num_objects > g["state_position"].shape[0]
        assert sc.to_ido() == g["ido"].tobytes()


def test_zoi_cleanup_erases_and_rekeys_like_the_reference(port_lib):
    """The zone-of-interest fixture: the reference erased the mobile objects above the zone
    before its first step and re-keyed the contact records; the oracle does the same (its
    candidate list at step 0 equals the reference's, record aliasing included)."""
    from oracle import PortWorld
    g = np.load(os.path.join(ROOT, "tests", "golden", "cluster_zoi.npz"))
    sc = Scene.from_ido(g["ido"].tobytes())
    mobile = [k for k, m in enumerate(sc.model_index) if sc.models[m].behavior == 3]
    above = [k for k in mobile if sc.position[k, 2] > sc.sp.zoi.upper[2]]
    assert len(above) > 0 and any(a in above or b in above for a, b in zip(sc.records.first, sc.records.second))
    w = PortWorld(sc, up_iact=int(g["up_iact"]))
    assert w.n == sc.num_objects - len(above) == g["state_position"].shape[0]
    f0, s0 = w.candidates()
    assert np.array_equal(f0, g["cand0_first"]) and np.array_equal(s0, g["cand0_second"])


def test_truncated_ido_rejected():
    b = scenes.cluster(n=8).to_ido()
    with pytest.raises(ValueError):
        Scene.from_ido(b[: len(b) // 2])


def test_time_control_runs_exact_step_count(port_lib):
    """t_stop = (steps - 1/2) dt makes Run() return false exactly after `steps` steps."""
    from oracle import PortWorld
    sc = scenes.cluster(n=8, steps=37)
    w = PortWorld(sc, up_iact=4)
    conts = [w.run(1) for _ in range(37)]
    assert all(conts[:-1]) and not conts[-1]


def test_generators_are_deterministic():
    a, b = scenes.lsd_box(n_side=6), scenes.lsd_box(n_side=6)
    assert a.to_ido() == b.to_ido()
    d1 = scenes.hertz_drum(n=20000, seed=3)
    d2 = scenes.hertz_drum(n=20000, seed=3)
    assert np.array_equal(d1.position, d2.position) and np.array_equal(d1.model_index, d2.model_index)


def test_drum_has_no_initial_overlap():
    sc = scenes.hertz_drum(n=30000, seed=1)
    p = sc.position[: 30000]
    r = np.array([m.attrs[0] for m in sc.models])[sc.model_index[:30000]]
    from scipy.spatial import cKDTree
    pairs = cKDTree(p).query_pairs(2 * r.max(), output_type="ndarray")
    d = np.linalg.norm(p[pairs[:, 0]] - p[pairs[:, 1]], axis=1)
    assert np.all(d > r[pairs[:, 0]] + r[pairs[:, 1]])


def test_lsd_box_matches_stated_config():
    sc = scenes.lsd_box()
    n = 8000
    assert sc.num_objects == n + 5
    assert sc.models[0].attrs[0] == 1e-3 and sc.models[0].density == 2500.0
    assert abs(sc.velocity[:n].std() - 0.05) < 0.002
    assert sc.iact_models[0].get("NormalStiffness") == 1e4 and sc.iact_models[0].get("ShearStiffness") == 8e3
    assert sc.iact_models[0].get("FrictionCoefficient") == 0.5
    assert sc.sp.time_interval == 1e-6


def test_abi_library_exports_every_declared_symbol(engine_lib):
    """libvedogpu.so loads without a GPU and exports every function include/vedo_gpu.h declares."""
    hdr = open(os.path.join(ROOT, "include", "vedo_gpu.h")).read()
    names = sorted(set(re.findall(r"\b(vedo_gpu_\w+)\s*\(", hdr)))
    assert len(names) >= 15
    lib = ctypes.CDLL(engine_lib.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    lib.vedo_gpu_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.vedo_gpu_version()


def test_abi_rejects_null_arguments(engine_lib):
    """Status codes instead of exit(): NULL handles and paths are INVALID_ARGUMENT (no GPU touched)."""
    lib = engine_lib.lib()
    assert lib.vedo_gpu_run(None, 1, None) == 1
    assert lib.vedo_gpu_create_from_ido(None, None, ctypes.byref(ctypes.c_void_p())) == 1
    assert lib.vedo_gpu_get_observables(None, None) == 1


def test_abi_bad_ido_is_reported(engine_lib, tmp_path):
    """A truncated .ido is BAD_IDO before any device work."""
    p = tmp_path / "bad.ido"
    p.write_bytes(scenes.cluster(n=8).to_ido()[:100])
    lib = engine_lib.lib()
    h = ctypes.c_void_p()
    rc = lib.vedo_gpu_create_from_ido(str(p).encode(), None, ctypes.byref(h))
    assert rc == 7
    assert b"truncated" in lib.vedo_gpu_last_error(None)


def test_holed_plate_model_analysis():
    """DOModel::Analysis of a plate with a circular hole (DOModel.cpp:90-119): the range of a
    plate, the hole's volume taken out, no inertia; a hole outside the plate is an error."""
    from vedo_gb300.scene import DOModel, FIXED, GLOBAL, QUASI_PLATE_WITH_CIRCULAR_HOLE
    m = DOModel("H", "W", FIXED, GLOBAL, 7800.0, 1.0, QUASI_PLATE_WITH_CIRCULAR_HOLE, (0.1, 0.01, 0.2, 0.02, 0.01, -0.03))
    rng, vol, mass, sm, inertia = m.analysis()
    assert rng == 0.5 * 0.01 and vol == 0.1 * 0.01 * 0.2 - 0.02 * 0.02 * np.pi * 0.01 and inertia == (0.0, 0.0, 0.0)
    bad = DOModel("H", "W", FIXED, GLOBAL, 7800.0, 1.0, QUASI_PLATE_WITH_CIRCULAR_HOLE, (0.1, 0.01, 0.2, 0.04, 0.02, 0.0))
    with pytest.raises(ValueError):
        bad.analysis()


def test_leap_cleans_the_zone_at_every_reset(port_lib):
    """The Leap consultant erases the mobile objects outside the zone of interest at every reset
    (LeapConsultant.cpp:61-68), the NBS consultant only once, at the start (SimMediator.cpp:125-134):
    with spheres flying out of the zone, the Leap world shrinks during the run and the NBS world
    keeps its objects after the start (the golden fixtures leap_zoi*.npz pin the Leap run to the
    reference's, records included)."""
    from oracle import PortWorld
    from vedo_gb300.scene import Boundary
    sc = scenes.cluster(n=27, seed=2, vel_sigma=1.0)
    mobile = [k for k, m in enumerate(sc.model_index) if sc.models[m].behavior == 3]
    x = sc.position[mobile, 0]
    sc.sp.zoi = Boundary(switch=(True, False, False), lower=(float(x.min()) - 5e-5, 0.0, 0.0),
                         upper=(float(x.max()) + 5e-5, 0.0, 0.0))
    leap, nbs = PortWorld(sc, up_iact=5, consultant="leap"), PortWorld(sc, up_iact=5, consultant="nbs")
    n0 = leap.n
    assert n0 == nbs.n == sc.num_objects
    leap.run(600)
    nbs.run(600)
    assert leap.n < n0 and nbs.n == n0
    assert leap.state()["position"].shape == (leap.n, 3)


def _one_zone_periodic_layer():
    """A layer whose periodic y axis is one Leap zone wide (two rows of spheres)."""
    return scenes.periodic_layer(nx=6, ny=2, layers=3, solver="ISwBSDBF", seed=32, periodic_y=True,
                                 drift=(-0.74, -1.06))


def test_leap_self_pairs_are_refused(port_lib):
    """With a periodic axis one zone wide, the reference's Leap consultant pairs a zone with its own
    periodic image, so its list holds pairs (i, i); CreateInteraction drops them (Assembler.cpp:27-30)
    and the pair table no longer lines up with the interactions.  The oracle refuses such a list."""
    import oracle
    from oracle import PortWorld
    sc = _one_zone_periodic_layer()
    with pytest.raises(ValueError, match="unsupported interaction"):
        PortWorld(sc, up_iact=4, consultant="leap")
    if oracle.ref_available() or oracle.build_ref() is not None:
        from oracle import RefWorld
        a, b = RefWorld(sc, up_iact=4, consultant="leap").candidates()
        assert np.any(a == b)


@pytest.mark.parametrize("seed", [31, 33, 34, 35])
def test_leap_oracle_equals_the_reference_on_random_layouts(seed, port_lib):
    """Seeded layouts (zone counts, periodic axes, drift) run by the reference's own Leap consultant
    and by the oracle: candidate lists element for element at the start and after 120 steps,
    states bit for bit.  Needs the reference compiled from its sources (skipped elsewhere)."""
    import oracle
    if not oracle.ref_available() and oracle.build_ref() is None:
        pytest.skip("reference sources not available")
    from oracle import PortWorld, RefWorld
    rng = np.random.default_rng(seed)
    # (at least three rows on each axis: a periodic axis one zone wide makes self pairs, above)
    sc = scenes.periodic_layer(nx=int(rng.integers(3, 7)), ny=int(rng.integers(3, 7)), layers=int(rng.integers(1, 4)),
                               solver="ISwBSDBF", seed=seed, periodic_y=bool(rng.integers(0, 2)),
                               drift=(float(rng.uniform(-3, 3)), float(rng.uniform(-3, 3))))
    r, p = RefWorld(sc, up_iact=4, consultant="leap"), PortWorld(sc, up_iact=4, consultant="leap")
    for _ in range(2):
        ra, rb = r.candidates()
        pa, pb = p.candidates()
        assert np.array_equal(ra, pa) and np.array_equal(rb, pb)
        r.run(60)
        p.run(60)
    a, b = r.state(), p.state()
    for k in ("position", "velocity", "angular_velocity"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    r.close()


@pytest.mark.parametrize("consultant", ["nbs", "leap"])
@pytest.mark.parametrize("seed", [41, 42, 43])
def test_oracle_equals_the_reference_on_random_clusters(seed, consultant, port_lib):
    """Seeded polydisperse clusters (sphere count, law, orbital walls, rods) run by the reference's
    own consultant and by the oracle: candidate lists element for element at the start and after
    each of two 60-step legs; states bit for bit for the linear law, within 1e-9 where pow and
    cos/sin enter.  Needs the reference compiled from its sources (skipped elsewhere)."""
    import oracle
    if not oracle.ref_available() and oracle.build_ref() is None:
        pytest.skip("reference sources not available")
    from oracle import PortWorld, RefWorld
    rng = np.random.default_rng(seed)
    solver = ("ISwBSDBF", "ISwH", "ISwHertz")[int(rng.integers(0, 3))]
    orbital = bool(rng.integers(0, 2))
    sc = scenes.cluster(n=int(rng.integers(20, 80)), solver=solver, polydisperse=True, orbital=orbital,
                        cylinders=int(rng.integers(0, 4)), steps=300, seed=seed)
    up = int(rng.integers(1, 8))
    r, p = RefWorld(sc, up_iact=up, consultant=consultant), PortWorld(sc, up_iact=up, consultant=consultant)
    for _ in range(3):
        ra, rb = r.candidates()
        pa, pb = p.candidates()
        assert np.array_equal(ra, pa) and np.array_equal(rb, pb)
        r.run(60)
        p.run(60)
    a, b = r.state(), p.state()
    exact = solver == "ISwBSDBF" and not orbital
    for k in ("position", "velocity", "angular_velocity"):
        if exact:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
        else:
            np.testing.assert_allclose(a[k], b[k], rtol=1e-9, atol=1e-12 * (np.abs(a[k]).max() + 1e-300), err_msg=k)
    r.close()


def test_port_matches_reference_whole_run_start(port_lib):
    """The first 2,000 steps of the 8,000-sphere box's whole run: the C restatement's state has
    the reference's SHA-256 after 100, 500, 1,000, 1,500 and 2,000 steps
    (tests/golden/wholerun/lsd_box.npz, made by the reference itself)."""
    import hashlib
    from oracle import PortWorld
    g = np.load(os.path.join(ROOT, "tests", "golden", "wholerun", "lsd_box.npz"))
    want = {int(s): str(d) for s, d in zip(g["table"][:, 0], g["digests"])}
    w = PortWorld(scenes.lsd_box(steps=int(g["steps"])), up_iact=int(g["up_iact"]))
    done = 0
    for target in (100, 500, 1000, 1500, 2000):
        w.run(target - done)
        done = target
        st = w.state()
        h = hashlib.sha256()
        for k in ("position", "velocity", "angular_velocity"):
            h.update(np.ascontiguousarray(st[k], dtype="<f8").tobytes())
        assert h.hexdigest() == want[target], target
        if target == 100:
            for k in ("position", "velocity", "angular_velocity"):
                np.testing.assert_array_equal(st[k], g[f"first100_{k}"], err_msg=k)
    w.close()


def test_inner_cylinder_detector_analytic(port_lib):
    """The hollow-cylinder extension (a drum shell; the reference has none): a sphere resting on
    the bottom at the linear law's equilibrium depth m g / kn, and a sphere pressed 1 um into the
    side.  Depths and outward radial normals are the analytic ones, and after one step the
    resting sphere's total impulse (contact + field) vanishes to rounding."""
    from oracle import PortWorld
    sc = scenes.shell_rest()
    m = 2500.0 * 4.0 / 3.0 * np.pi * 1e-9
    w = PortWorld(sc, up_iact=1)
    it = w.interactions()
    assert list(it["master"]) == [2, 2] and list(it["active"]) == [1, 1]
    np.testing.assert_allclose(it["depth"], [m * 9.81 / 1e4, 1e-6], rtol=1e-6)
    np.testing.assert_allclose(it["normal"], [[0.0, 0.0, -1.0], [0.0, 1.0, 0.0]], atol=1e-12)
    w.run(1)
    J = w.state()["impact"]
    assert np.abs(J[0]).max() <= 1e-9 * m * 9.81 * 1e-6
    np.testing.assert_allclose(J[1, 1], -1e4 * 1e-6 * 1e-6, rtol=1e-6)
    w.close()


def test_inner_cylinder_scene_keeps_every_sphere_inside_and_reaches_the_shell(port_lib):
    """shell_drop (the scene of the GPU shell tests): spheres start clear of the shell and of one
    another, and within 1,000 steps of the oracle they reach it and bounce off it."""
    from oracle import PortWorld
    sc = scenes.shell_drop()
    w = PortWorld(sc, up_iact=5)
    hits = 0
    for _ in range(10):
        w.run(100)
        it = w.interactions()
        hits += int(it["active"][it["master"] == 150].sum())
    assert hits > 10
    v = w.state()["velocity"][:150]
    assert np.abs(v).max() < 3.0
    w.close()
