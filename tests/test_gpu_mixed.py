"""GPU tests of the mixed-precision form (VEDO_PRECISION_MIXED) against the FP64 engine, whose
results are pinned to the reference by test_gpu_parity.py.

Bars (from the engine's contract): the contact set at identical positions is identical;
per-step impulses from identical state (positions, velocities, shear history) agree within
1e-5 relative (L2 over all objects); energy after 2,000 steps within 1 %; runs are
deterministic."""
import os

import numpy as np
import pytest

from vedo_gb300 import scenes

pytestmark = pytest.mark.gpu


def _active_set(it):
    a = it["active"] == 1
    return set(zip(it["first"][a].tolist(), it["second"][a].tolist()))


@pytest.mark.parametrize("which", ["box", "drum"])
def test_mixed_contact_set_equals_fp64(which, box_ido, drum_ido, engine_lib):
    path = box_ido if which == "box" else drum_ido
    a = engine_lib.GpuEngine(path, up_iact=20)
    b = engine_lib.GpuEngine(path, up_iact=20, precision=1)
    A, B = _active_set(a.interactions()), _active_set(b.interactions())
    assert len(A) > 10
    assert A == B


@pytest.mark.parametrize("which", ["box", "drum"])
def test_mixed_per_step_impulse_error(which, box_ido, drum_ido, engine_lib):
    path = box_ido if which == "box" else drum_ido
    a = engine_lib.GpuEngine(path, up_iact=20)
    b = engine_lib.GpuEngine(path, up_iact=20, precision=1)
    a.run(1)
    b.run(1)
    sa, sb = a.state(), b.state()
    for k in ("impact", "angular_impact"):
        ref = np.linalg.norm(sa[k])
        assert ref > 0, k
        err = np.linalg.norm(sa[k] - sb[k]) / ref
        assert err <= 1e-5, (k, err)


def test_mixed_energy_within_one_percent(box_ido, engine_lib):
    a = engine_lib.GpuEngine(box_ido, up_iact=20)
    b = engine_lib.GpuEngine(box_ido, up_iact=20, precision=1)
    a.run(2000)
    b.run(2000)
    oa, ob = a.observables(), b.observables()
    ea, eb = oa[0] + oa[1] + oa[2], ob[0] + ob[1] + ob[2]
    assert abs(ea - eb) <= 0.01 * abs(ea)
    assert abs(oa[1] - ob[1]) <= 0.01 * oa[1]


def test_mixed_deterministic(drum_ido, engine_lib):
    r = []
    for _ in range(2):
        e = engine_lib.GpuEngine(drum_ido, up_iact=20, precision=1)
        e.run(300)
        r.append(e.state())
        e.close()
    for k in r[0]:
        assert np.array_equal(r[0][k], r[1][k]), k


def test_mixed_results_independent_of_rebuilds(box_ido, engine_lib):
    """Neighbour lists are kept in canonical order and histories are carried, so a tiny skin
    (a rebuild every step or two) and a wide one (rare rebuilds) give bit-identical results."""
    a = engine_lib.GpuEngine(box_ido, precision=1, skin=0.5)
    b = engine_lib.GpuEngine(box_ido, precision=1, skin=0.002, check_interval=1)
    a.run(400)
    b.run(400)
    sa, sb = a.state(), b.state()
    for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
        assert np.array_equal(sa[k], sb[k]), k


def test_mixed_matches_oracle_trajectory_start(engine_lib, port_lib):
    """Mixed vs the C oracle (= the reference) for the first 100 steps of a colliding cluster."""
    from oracle import PortWorld
    sc = scenes.cluster(n=64, solver="ISwBSDBF", steps=500, seed=21)
    e = engine_lib.GpuEngine(sc, up_iact=5, precision=1)
    p = PortWorld(sc, up_iact=5)
    e.run(100)
    p.run(100)
    a, b = e.state(), p.state()
    assert np.linalg.norm(a["velocity"] - b["velocity"]) <= 1e-5 * np.linalg.norm(b["velocity"])
    assert np.abs(a["position"] - b["position"]).max() <= 1e-9


@pytest.mark.parametrize("behavior,solver", [("mobile", "ISwBSDBF"), ("constrained", "ISwH")])
def test_mixed_mobile_and_constrained_walls_against_fp64(behavior, solver, engine_lib):
    """A lid moved by its impulses (a mobile plate: translation and rotation; a constrained one:
    along its normal) in the mixed form: the wall shares are summed exactly every step and the
    lid responds as the FP64 form's respond_object.  From the FP64 form's state at step 450 (lid
    in contact): identical contact sets, the lid's and the spheres' step impulses within 1e-5,
    and after 100 more steps the lid within 1e-8 m and 1e-3 relative in velocity of the FP64
    form's (the lid rests on many spheres: the force errors add up in its small sideways motion);
    every form of the tick gives the same bits."""
    import os
    import tempfile
    sc = scenes.piston(behavior=behavior, solver=solver, steps=3000)
    lid = sc.num_objects - 1
    f64 = engine_lib.GpuEngine(sc, up_iact=5)
    f64.run(450)                                   # the lid has reached the spheres
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "p.ido")
        f64.write_ido(path)
        a = engine_lib.GpuEngine(path, up_iact=5)
        forms = [engine_lib.GpuEngine(path, up_iact=5, precision=1, **kw)
                 for kw in ({}, {"split_tick": True}, {"pair_pass": True}, {"skin": 0.02, "check_interval": 1})]
    b = forms[0]
    A, B = _active_set(a.interactions()), _active_set(b.interactions())
    assert A == B and any(lid in p for p in A)
    a.run(1)
    for e in forms:
        e.run(1)
    sa, sb = a.state(), b.state()
    for k in ("impact", "angular_impact"):
        ref = np.linalg.norm(sa[k])
        assert np.linalg.norm(sa[k] - sb[k]) <= 1e-5 * ref, k
    assert np.linalg.norm(sa["impact"][lid] - sb["impact"][lid]) <= 1e-5 * np.linalg.norm(sa["impact"][lid])
    a.run(100)
    for e in forms:
        e.run(100)
    sa, sb = a.state(), b.state()
    assert np.abs(sa["position"][lid] - sb["position"][lid]).max() <= 1e-8
    assert np.linalg.norm(sa["velocity"][lid] - sb["velocity"][lid]) <= 1e-3 * np.linalg.norm(sa["velocity"][lid])
    assert abs(sa["position"][lid][2] - sc.position[lid][2]) > 1e-5          # the lid did move
    for e in forms[1:]:
        st = e.state()
        for k in ("position", "velocity", "angular_velocity", "orientation_x", "orientation_z"):
            assert np.array_equal(st[k], sb[k]), k


@pytest.mark.parametrize("which", ["dense", "box"])
def test_stored_and_formed_position_splits_agree(which, box_ido, engine_lib):
    """The sphere-pair overlap test's hi/lo position splits, stored once per step or formed per
    pair, give bit-identical results (the autotuner may pick either)."""
    sc = scenes.dense_pack(n=20000) if which == "dense" else box_ido
    a = engine_lib.GpuEngine(sc, precision=1, stored_splits=False)
    b = engine_lib.GpuEngine(sc, precision=1, stored_splits=True)
    assert b.tuning()["stored_splits"] and not a.tuning()["stored_splits"]
    a.run(300)
    b.run(300)
    sa, sb = a.state(), b.state()
    for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
        assert np.array_equal(sa[k], sb[k]), k
    assert (a.interactions()["active"] == 1).sum() > 1000 if which == "dense" else True


@pytest.mark.parametrize("which", ["dense", "box", "drum"])
def test_split_tick_agrees_with_one_tick(which, box_ido, drum_ido, engine_lib):
    """The split tick (light prefilter tick at full occupancy + the full tick over the deferred
    spheres) gives the single tick's results bit for bit."""
    sc = {"dense": lambda: scenes.dense_pack(n=20000), "box": lambda: box_ido, "drum": lambda: drum_ido}[which]()
    a = engine_lib.GpuEngine(sc, precision=1, split_tick=False)
    b = engine_lib.GpuEngine(sc, precision=1, split_tick=True, stored_splits=True)
    assert b.tuning()["split_tick"] and not a.tuning()["split_tick"]
    a.run(300)
    b.run(300)
    sa, sb = a.state(), b.state()
    for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.parametrize("which", ["dense", "box", "drum", "hopper", "bed", "holed", "shell"])
@pytest.mark.parametrize("stored", [False, True])
def test_pair_pass_agrees_with_one_tick(which, stored, box_ido, drum_ido, engine_lib):
    """The pair pass (prefilter pass, each pair on the exact path evaluated once, per-sphere sums
    of the pair records in list order) gives the single tick's state, impulses and contact
    history bit for bit, over calls of uneven length (impulses written on each call's last step),
    rebuilds, walls (fixed plates, rods, a holed plate, an orbital top plate) and contacts that
    form and break."""
    sc = {"dense": lambda: scenes.dense_pack(n=20000), "box": lambda: box_ido, "drum": lambda: drum_ido,
          "hopper": lambda: scenes.hopper(n=6000, touching=True),
          "bed": lambda: scenes.compressed_bed(n=20000, box=0.03, cylinders=1, plate_speed=0.5),
          "holed": lambda: scenes.holed_plate_drop(), "shell": lambda: scenes.shell_drop(rpm=30.0)}[which]()
    a = engine_lib.GpuEngine(sc, precision=1, stored_splits=stored)
    b = engine_lib.GpuEngine(sc, precision=1, stored_splits=stored, pair_pass=True)
    assert b.tuning()["pair_pass"] and not a.tuning()["pair_pass"] and not b.tuning()["split_tick"]
    for n in (7, 1, 33, 100, 2, 157):
        a.run(n)
        b.run(n)
        _same_run(a, b)
    if which in ("dense", "bed"):
        assert (b.interactions()["active"] == 1).sum() > 100
    elif which == "box":
        assert (b.interactions()["active"] == 1).sum() > 10


def test_pair_pass_batch_equals_alone(engine_lib):
    """A scene's slice of a pair-pass batch equals the scene run alone in the single tick."""
    hs = [scenes.hopper(n=n, seed=s, touching=True) for n, s in ((3000, 1), (5000, 2), (1200, 3))]
    b = engine_lib.BatchEngine(hs, pair_pass=True)
    b.run(250)
    for q, h in enumerate(hs):
        e = engine_lib.GpuEngine(h, precision=1)
        e.run(250)
        st, sb = e.state(), b.scene_state(q)
        for k in ("position", "velocity", "angular_velocity"):
            assert np.array_equal(st[k], sb[k]), (q, k)
        e.close()
    b.close()


def test_split_tick_and_pair_pass_are_exclusive(engine_lib):
    with pytest.raises(ValueError):
        engine_lib.GpuEngine(scenes.dense_pack(n=2000), precision=1, split_tick=True, pair_pass=True)


def test_mixed_orientations_follow_the_fp64_form(box_ido, engine_lib):
    """With `orientations` the mixed form turns every sphere's Ox, Oz by dt (w + dw/2) per step
    as DOSphere::Response does: on the settled box (spheres rolling and spinning) they stay
    within 1e-5 of the FP64 form's after 300 steps (the angular velocities themselves differ at
    the mixed form's force error), stay unit and orthogonal, and are the same in every form of
    the tick; without the option they are left as they were."""
    f64 = engine_lib.GpuEngine(box_ido, up_iact=1)
    mixed = [engine_lib.GpuEngine(box_ido, precision=1, orientations=True, **kw)
             for kw in ({}, {"split_tick": True}, {"pair_pass": True})]
    still = engine_lib.GpuEngine(box_ido, precision=1)
    o0 = still.state(("orientation_x", "orientation_z"))
    for e in [f64, still] + mixed:
        e.run(300)
    ref = f64.state(("orientation_x", "orientation_z", "angular_velocity"))
    assert np.abs(ref["angular_velocity"]).max() > 1.0          # the spheres do spin
    moved = np.abs(ref["orientation_x"] - o0["orientation_x"]).max()
    assert moved > 1e-3
    first = mixed[0].state(("orientation_x", "orientation_z"))
    for e in mixed[1:]:
        st = e.state(("orientation_x", "orientation_z"))
        for k in st:
            assert np.array_equal(st[k], first[k]), k
    for k in ("orientation_x", "orientation_z"):
        np.testing.assert_allclose(first[k], ref[k], rtol=0, atol=1e-5, err_msg=k)
        assert np.allclose(np.linalg.norm(first[k], axis=1), 1.0, atol=1e-12)
    assert np.abs(np.sum(first["orientation_x"] * first["orientation_z"], axis=1)).max() < 1e-12
    left = still.state(("orientation_x", "orientation_z"))
    for k in left:
        assert np.array_equal(left[k], o0[k]), k


def _active_history(e):
    it = e.interactions()
    a = np.nonzero(it["active"] == 1)[0]
    return {(int(it["first"][q]), int(it["second"][q])): (tuple(it["shear"][q]), float(it["kn"][q])) for q in a}


def _same_run(a, b):
    sa, sb = a.state(), b.state()
    for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
        assert np.array_equal(sa[k], sb[k]), k
    ia, ib = a.interactions(), b.interactions()
    for k in ia:
        assert np.array_equal(ia[k], ib[k]), k


@pytest.mark.parametrize("which,split", [("fresh_drum", True), ("fresh_drum", False), ("drum", True),
                                         ("hopper", True), ("hopper", False), ("box", True)])
def test_quiet_spheres_skip_the_walk_with_identical_results(which, split, box_ido, drum_ido, engine_lib):
    """A sphere whose pairs have all been certainly apart since the rebuild, with clean history,
    skips its neighbour-list walk; state, impulses and contact history equal those of full walks
    bit for bit, over calls of uneven length (impulses written on each call's last step),
    rebuilds, and contacts that form and break."""
    sc = {"fresh_drum": lambda: scenes.hertz_drum(n=20000), "drum": lambda: drum_ido,
          "hopper": lambda: scenes.hopper(n=6000), "box": lambda: box_ido}[which]()
    a = engine_lib.GpuEngine(sc, precision=1, split_tick=split, full_walks=True)
    b = engine_lib.GpuEngine(sc, precision=1, split_tick=split)
    quiet = 0
    for n in (7, 1, 33, 100, 2, 157, 60):
        a.run(n)
        b.run(n)
        _same_run(a, b)
        assert a.quiet_spheres() == 0
        quiet = max(quiet, b.quiet_spheres())
    if which in ("fresh_drum", "hopper"):       # free fall: most spheres are quiet
        assert quiet > b.n // 2, quiet


def test_orbital_wall_closing_in_independent_of_skin(engine_lib):
    """A fast orbital top plate closing on a bed: its entries are gathered with the wider wall
    skin and tested with their own displacement bound.  A tiny skin (rebuilds every few steps), a
    wide one, and full walks give bit-identical results, the plate does reach the bed, and its
    impulse agrees with the FP64 engine's."""
    sc = scenes.compressed_bed(n=20000, box=0.03, cylinders=1, plate_speed=0.5, packing="fcc")
    plate = sc.position.shape[0] - 1
    wide = engine_lib.GpuEngine(sc, precision=1, skin=0.5)
    tiny = engine_lib.GpuEngine(sc, precision=1, skin=0.002, check_interval=1)
    full = engine_lib.GpuEngine(sc, precision=1, skin=0.5, split_tick=True, full_walks=True)
    f64 = engine_lib.GpuEngine(sc, up_iact=1)
    touched = 0
    for n in (50, 1, 99, 150):
        for e in (wide, tiny, full, f64):
            e.run(n)
        _same_run(wide, full)
        sa, sb = wide.state(), tiny.state()
        for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
            assert np.array_equal(sa[k], sb[k]), k
        assert _active_history(wide) == _active_history(tiny)      # the candidate lists differ
        jm, jf = sa["impact"][plate], f64.state(("impact",))["impact"][plate]
        if jf[2] != 0.0:
            touched += 1
            assert np.linalg.norm(jm - jf) <= 1e-3 * np.linalg.norm(jf)
    assert touched >= 2


def test_profiled_graph_replay_times_kernels_without_changing_results(engine_lib):
    """Per-kernel timing events ride inside the replayed graphs: the tick and wall times are
    reported, and the results are those of an unprofiled run."""
    sc = scenes.hertz_drum(n=20000)
    a = engine_lib.GpuEngine(sc, precision=1, split_tick=True)
    b = engine_lib.GpuEngine(sc, precision=1, split_tick=True)
    b.set_profiling(True)
    for n in (40, 100):
        a.run(n)
        b.run(n)
    p = b.last_run_profile()
    assert p["pair_ms"] > 0.0 and p["object_ms"] > 0.0 and p["pair_ms"] + p["object_ms"] <= p["total_ms"]
    _same_run(a, b)


def test_set_state_keeps_the_list_when_the_bound_absorbs_the_jump(engine_lib):
    """vedo_gpu_set_state adds the spheres' largest jump to the displacement bound instead of
    rebuilding (a moved wall, or a jump the skin cannot absorb, still rebuilds).  A wide-skin
    engine that keeps its list and a tiny-skin one that rebuilds every step or two stay
    bit-identical through unchanged, slightly moved and far moved states."""
    sc = scenes.hopper(n=4000, steps=3000)
    a = engine_lib.GpuEngine(sc, precision=1, skin=0.5, split_tick=True)
    c = engine_lib.GpuEngine(sc, precision=1, skin=0.002, check_interval=1)
    fields = ("position", "velocity", "angular_velocity")
    for jump in (0.0, 2e-7, 3e-4):
        a.run(37)
        c.run(37)
        sa, sc_ = a.state(fields), c.state(fields)
        for k in fields:
            assert np.array_equal(sa[k], sc_[k]), (jump, k)
        sa["position"][5] += jump
        sa["velocity"][7] *= 1.5
        a.set_state(**sa)
        c.set_state(**sa)
        a.run(25)
        c.run(25)
        ra, rc = a.state(), c.state()
        for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
            assert np.array_equal(ra[k], rc[k]), (jump, k)
        assert _active_history(a) == _active_history(c)


def test_spinning_plate_corners_reach_spheres_beyond_its_list(engine_lib):
    """A plate spinning in its own plane keeps its plane but sweeps its corners: spheres near the
    plane outside its inscribed circle make the wall's approach bound the full |omega| R, so a
    moderate skin (spheres first listed late) and a tiny one (rebuilt every step or two) stay
    bit-identical, and the corners do hit the spheres."""
    sc = scenes.spinning_plate()
    a = engine_lib.GpuEngine(sc, precision=1, skin=0.05, split_tick=True)
    b = engine_lib.GpuEngine(sc, precision=1, skin=0.002, check_interval=1)
    for n in (1000, 700, 700, 599):
        a.run(n)
        b.run(n)
        sa, sb = a.state(), b.state()
        for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
            assert np.array_equal(sa[k], sb[k]), (n, k)
    v = a.state(("velocity",))["velocity"][:8]
    assert (np.linalg.norm(v, axis=1) > 0.1).sum() >= 4          # the first four were struck


def test_plate_with_circular_hole_mixed_against_fp64(engine_lib, tmp_path):
    """Spheres on a plate with an off-centre circular hole (the reference's
    QuasiPlateWithCircularHole): from identical state, the mixed form's contact set equals the
    FP64 form's (pinned to the reference by the golden fixture) and its one-step impulses agree
    within 1e-5."""
    sc = scenes.holed_plate_drop(steps=2000)
    f64 = engine_lib.GpuEngine(sc, up_iact=5)
    f64.run(150)
    path = str(tmp_path / "h.ido")
    f64.write_ido(path)
    a = engine_lib.GpuEngine(path, up_iact=5)
    b = engine_lib.GpuEngine(path, up_iact=5, precision=1)
    A, B = _active_set(a.interactions()), _active_set(b.interactions())
    assert len(A) >= 4 and A == B
    a.run(1)
    b.run(1)
    sa, sb = a.state(("impact",)), b.state(("impact",))
    assert np.linalg.norm(sa["impact"] - sb["impact"]) <= 1e-5 * np.linalg.norm(sa["impact"])
