"""The persistent tick: a check interval of steps as ONE cooperative launch whose stages (the
per-step kernels' device functions) are separated by grid barriers, in place of a replayed graph
of per-step kernels.  Same operations per sphere, pair and wall in the same order, so the same
bits: state, impulses and contact history, alone and in batches, for the full tick and the pair
pass.  The barrier's wait is bounded: a barrier that cannot complete expires, records where, and
the kernel ends with the device still usable."""
import ctypes as C
import time

import numpy as np
import pytest

from vedo_gb300 import scenes

pytestmark = pytest.mark.gpu


def _same_run(a, b):
    sa, sb = a.state(), b.state()
    for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact", "orientation_x",
              "orientation_z"):
        assert np.array_equal(sa[k], sb[k]), k
    ia, ib = a.interactions(), b.interactions()
    for k in ia:
        assert np.array_equal(ia[k], ib[k]), k


def _scene(which, box_ido, drum_ido):
    return {"dense": lambda: scenes.dense_pack(n=20000), "box": lambda: box_ido, "drum": lambda: drum_ido,
            "hopper": lambda: scenes.hopper(n=6000, touching=True),
            "bed": lambda: scenes.compressed_bed(n=20000, box=0.03, cylinders=1, plate_speed=0.5),
            "shell": lambda: scenes.shell_drop(rpm=30.0),
            "periodic": lambda: scenes.periodic_layer(nx=12, ny=12, layers=4, seed=21, steps=2000,
                                                      solver="ISwH")}[which]()


@pytest.mark.parametrize("which", ["dense", "box", "drum", "hopper", "bed", "shell", "periodic"])
@pytest.mark.parametrize("form", ["single", "pair"])
def test_persistent_tick_equals_per_step_kernels(which, form, box_ido, drum_ido, engine_lib):
    """Calls of uneven length (partial check intervals; each call's last step writes the impulses
    and runs as per-step kernels), rebuilds, walls, periodic wrap and sphere orientations: the
    persistent launch gives the per-step kernels' bits, with one launch per check interval."""
    sc = _scene(which, box_ido, drum_ido)
    kw = dict(precision=1, pair_pass=form == "pair", stored_splits=which != "box",
              orientations=which in ("periodic", "box"))
    a = engine_lib.GpuEngine(sc, **kw)
    b = engine_lib.GpuEngine(sc, persistent=True, **kw)
    assert b.tuning()["persistent"] and not a.tuning()["persistent"]
    for n in (7, 1, 33, 100, 2, 157):
        a.run(n)
        b.run(n)
        _same_run(a, b)
    la, lb = a.last_run_profile()["launches"], b.last_run_profile()["launches"]
    assert lb < la, (la, lb)
    if which in ("dense", "bed"):
        assert (b.interactions()["active"] == 1).sum() > 100


def test_persistent_batch_equals_alone(engine_lib):
    """A scene's slice of a persistent pair-pass batch equals the scene run alone with per-step
    kernels."""
    hs = [scenes.hopper(n=n, seed=s, touching=True) for n, s in ((3000, 1), (5000, 2), (1200, 3))]
    b = engine_lib.BatchEngine(hs, pair_pass=True, persistent=True)
    assert b.tuning()["persistent"]
    b.run(250)
    for q, h in enumerate(hs):
        e = engine_lib.GpuEngine(h, precision=1)
        e.run(250)
        st, sb = e.state(), b.scene_state(q)
        for k in ("position", "velocity", "angular_velocity"):
            assert np.array_equal(st[k], sb[k]), (q, k)
        e.close()
    b.close()


def test_persistent_tick_steps_past_its_list(engine_lib):
    """A check interval whose list runs out part way: the remaining steps of the launch are
    identity steps, taken again after the rebuild, as with per-step kernels (a fast, loose
    scene with a thin skin rebuilds often)."""
    sc = scenes.lsd_box(n_side=10, vel_sigma=3.0, spacing=2.2e-3)
    a = engine_lib.GpuEngine(sc, precision=1, skin=0.05, check_interval=25)
    b = engine_lib.GpuEngine(sc, precision=1, skin=0.05, check_interval=25, persistent=True)
    a.run(400)
    b.run(400)
    _same_run(a, b)
    assert b.list_status()["rebuilds"] > 5


def test_grid_barrier_counts_and_expires(engine_lib):
    """The barrier alone: 2,000 barriers over every block the device holds, each block checking
    the arrivals of every round; then a barrier that expects one block more than the grid has
    (nothing completes it) expires after its 50 ms limit, records the round, and the kernel ends;
    the device then runs an engine as before."""
    lib = engine_lib.lib()
    out = (C.c_uint32 * 4)()
    assert lib.vedo_gpu_barrier_check(0, 2000, 0, 2_000_000_000, out) == 0
    assert list(out) == [2000, 0, 0, 0]
    t0 = time.perf_counter()
    assert lib.vedo_gpu_barrier_check(0, 5, 1, 50_000_000, out) == 0
    waited = time.perf_counter() - t0
    assert out[0] == 0 and out[1] == 0 and out[2] == 1 and out[3] == 1, list(out)
    assert 0.05 <= waited < 2.0, waited
    e = engine_lib.GpuEngine(scenes.dense_pack(n=2000), precision=1, persistent=True)
    e.run(30)
    assert np.isfinite(e.state()["position"]).all()
    e.close()
