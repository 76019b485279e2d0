"""GPU parity tests: the CUDA engine, called through the C ABI, against the reference's golden
vectors (tests/golden, produced by the reference itself) and against the C oracle.

Tolerances: the linear spring-dashpot laws with fixed walls use only IEEE-rounded +,-,*,/
and sqrt, evaluated in the reference's order without FMA, so the engine must agree bit for
bit.  Hertz and ISwH call pow(), orbital walls call cos()/sin(); CUDA's and glibc's results
may differ in the last ulp, so those cases use rtol 1e-9 on short runs (per-step forces agree
to ~1e-15 relative); the contact set and history pairing stay exact."""
import glob
import os

import numpy as np
import pytest

from vedo_gb300 import scenes
from vedo_gb300.scene import Scene

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))
EXACT_CASES = ("box_lsd", "cluster_ISwBSDBF", "cluster_ISwBtSDBF", "cluster_ISwBSDB2F", "cluster_bsdbf_upiact1",
               "cluster_zoi", "holed_plate_lsd", "periodic_lsd",
               "periodic_far_lsd", "periodic_btsdbf", "periodic_bsdb2f", "leap_box_lsd",
               "leap_periodic_lsd", "leap_periodic_wide", "leap_wide_y", "leap_column_z", "leap_single", "leap_zoi")
STATE = ("position", "velocity", "angular_velocity", "impact", "angular_impact", "orientation_x", "orientation_z")


def _name(p):
    return os.path.splitext(os.path.basename(p))[0]


@pytest.mark.parametrize("path", GOLDEN, ids=[_name(p) for p in GOLDEN])
def test_engine_matches_reference_golden(path, engine_lib):
    g = np.load(path)
    sc = Scene.from_ido(g["ido"].tobytes())
    e = engine_lib.GpuEngine(sc, up_iact=int(g["up_iact"]),
                             consultant=str(g["consultant"]) if "consultant" in g else "nbs")
    it0 = e.interactions()
    assert np.array_equal(it0["first"], g["cand0_first"]) and np.array_equal(it0["second"], g["cand0_second"])
    e.run(int(g["steps"]))
    it = e.interactions()
    assert np.array_equal(it["first"], g["cand_first"]) and np.array_equal(it["second"], g["cand_second"])
    assert np.array_equal(it["active"], g["iact_active"])
    assert np.array_equal(it["slave"], g["iact_slave"]) and np.array_equal(it["master"], g["iact_master"])
    assert np.array_equal(it["contact"], g["iact_contact"])
    st = e.state()
    exact = _name(path) in EXACT_CASES
    for k in STATE:
        ref = g[f"state_{k}"]
        if exact and not k.startswith("orientation"):
            np.testing.assert_array_equal(st[k], ref, err_msg=k)
        else:
            np.testing.assert_allclose(st[k], ref, rtol=1e-9, atol=1e-12 * (np.abs(ref).max() + 1e-300), err_msg=k)
    if exact:
        np.testing.assert_array_equal(it["shear"], g["iact_shear"])
    else:
        np.testing.assert_allclose(it["shear"], g["iact_shear"], rtol=1e-8, atol=1e-14)
    assert e.time() == float(g["time"])
    e.close()


@pytest.mark.parametrize("solver", ["ISwBSDBF", "ISwBtSDBF", "ISwBSDB2F", "ISwHertz", "ISwH"])
def test_per_step_impulses_at_identical_state(solver, engine_lib, port_lib):
    """From identical state, one step: per-object impulse and angular impulse agree with the
    oracle within 1e-10 relative (exactly for the linear laws)."""
    from oracle import PortWorld
    sc = scenes.cluster(n=64, solver=solver, steps=500, seed=21)
    e = engine_lib.GpuEngine(sc, up_iact=4)
    p = PortWorld(sc, up_iact=4)
    e.run(120)
    p.run(120)
    s = p.state()
    sc2 = sc.copy()
    for k in ("position", "velocity", "angular_velocity", "orientation_x", "orientation_z"):
        setattr(sc2, k, s[k])
    e2 = engine_lib.GpuEngine(sc2, up_iact=4)
    p2 = PortWorld(sc2, up_iact=4)
    e2.run(1)
    p2.run(1)
    a, b = e2.state(), p2.state()
    for k in ("impact", "angular_impact"):
        scale = np.abs(b[k]).max() + 1e-300
        if solver in ("ISwHertz", "ISwH"):
            np.testing.assert_allclose(a[k], b[k], rtol=1e-10, atol=1e-10 * scale, err_msg=k)
        else:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    ia, ib = e2.interactions(), p2.interactions()
    assert np.array_equal(ia["active"], ib["active"].astype(np.uint8))
    assert ia["active"].sum() > 0


def test_lsd_box_full_size_bitexact(engine_lib, port_lib):
    """The 8,000-sphere box: 600 steps with rebuilds every 20, bit for bit against the oracle."""
    from oracle import PortWorld
    sc = scenes.lsd_box()
    e = engine_lib.GpuEngine(sc, up_iact=20)
    p = PortWorld(sc, up_iact=20)
    e.run(600)
    p.run(600)
    a, b = e.state(), p.state()
    for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    ia = e.interactions()
    f, s = p.candidates()
    assert np.array_equal(ia["first"], f) and np.array_equal(ia["second"], s)


def test_two_pass_pair_kernel_bitexact(engine_lib, port_lib):
    """A box of 39,304 spheres thrown together (about 50,000 contacts after 200 steps), whose
    candidate list is longer than the one-pass pair kernel takes: the prefilter pass compacts the pairs that may touch and the exact pass evaluates them in full
    warps; 200 steps with rebuilds every 20, bit for bit against the oracle."""
    from oracle import PortWorld
    sc = scenes.lsd_box(n_side=34, box_width=0.08, box_height=0.1, steps=400, spacing=2.005e-3, vel_sigma=0.3)
    e = engine_lib.GpuEngine(sc, up_iact=20)
    p = PortWorld(sc, up_iact=20)
    assert len(e.interactions()["first"]) > (1 << 17)
    e.run(200)
    p.run(200)
    a, b = e.state(), p.state()
    for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    ia, ib = e.interactions(), p.interactions()
    f, s = p.candidates()
    assert np.array_equal(ia["first"], f) and np.array_equal(ia["second"], s)
    assert np.array_equal(ia["active"], ib["active"].astype(np.uint8))
    assert ia["active"].sum() > 10000


def test_first_100_steps_pointwise_hertz_drum_small(engine_lib, port_lib):
    """Polydisperse ISwH drum (orbital end plates, polygon shell), 20k spheres: pointwise agreement
    for the first 100 steps (1e-9 relative), exact contact set."""
    from oracle import PortWorld
    sc = scenes.hertz_drum(n=20000, seed=5, steps=200)
    e = engine_lib.GpuEngine(sc, up_iact=10)
    p = PortWorld(sc, up_iact=10)
    for _ in range(4):
        e.run(25)
        p.run(25)
        a, b = e.state(), p.state()
        for k in ("position", "velocity"):
            np.testing.assert_allclose(a[k], b[k], rtol=1e-9, atol=1e-12 * np.abs(b[k]).max() + 1e-300, err_msg=k)
    ia, ib = e.interactions(), p.interactions()
    f, s = p.candidates()
    assert np.array_equal(ia["first"], f) and np.array_equal(ia["second"], s)
    assert np.array_equal(ia["active"], ib["active"].astype(np.uint8))


def test_create_from_ido_equals_create(engine_lib, tmp_path):
    sc = scenes.cluster(n=40, solver="ISwH", polydisperse=True, cylinders=2, seed=4)
    path = tmp_path / "s.ido"
    sc.to_ido(str(path))
    a = engine_lib.GpuEngine(sc, up_iact=3)
    b = engine_lib.GpuEngine(str(path), up_iact=3)
    a.run(150)
    b.run(150)
    sa, sb = a.state(), b.state()
    for k in sa:
        np.testing.assert_array_equal(sa[k], sb[k])


def test_history_survives_ido_restart(engine_lib, tmp_path):
    """run(2k) == run(k) + write_ido + reload + run(k): the IDO carries the shear history."""
    sc = scenes.cluster(n=64, solver="ISwBSDBF", steps=1000, seed=8)
    a = engine_lib.GpuEngine(sc, up_iact=5)
    a.run(300)
    assert a.interactions()["active"].sum() > 0
    path = tmp_path / "mid.ido"
    a.write_ido(str(path))
    a.run(300)
    b = engine_lib.GpuEngine(str(path), up_iact=5)
    b.run(300)
    sa, sb = a.state(), b.state()
    for k in ("position", "velocity", "angular_velocity"):
        np.testing.assert_array_equal(sa[k], sb[k])


def test_deterministic_reruns(engine_lib):
    sc = scenes.hertz_drum(n=30000, seed=2, steps=100)
    r = []
    for _ in range(2):
        e = engine_lib.GpuEngine(sc, up_iact=10)
        e.run(60)
        r.append(e.state())
        e.close()
    for k in r[0]:
        assert np.array_equal(r[0][k], r[1][k])


def test_observables_match_oracle(engine_lib, port_lib):
    from oracle import PortWorld
    sc = scenes.lsd_box(n_side=10)
    e = engine_lib.GpuEngine(sc, up_iact=10)
    p = PortWorld(sc, up_iact=10)
    e.run(200)
    p.run(200)
    o, q = e.observables(), p.energy()
    np.testing.assert_allclose(o[:9], q, rtol=1e-12)


def test_unsupported_model_is_an_error(engine_lib):
    sc = scenes.cluster(n=8)
    sc.iact_models[0].equation_type = "ISwNoSuchLaw"
    with pytest.raises(engine_lib.EngineError) as ex:
        engine_lib.GpuEngine(sc)
    assert ex.value.code == 3


def test_missing_mechanism_is_an_error(engine_lib):
    sc = scenes.cluster(n=8)
    sc.iact_models[0].mechanisms = [m for m in sc.iact_models[0].mechanisms if m[0] != "ShearStiffness"]
    with pytest.raises(engine_lib.EngineError) as ex:
        engine_lib.GpuEngine(sc)
    assert ex.value.code == 2


def test_engine_native_library_is_the_one_loaded(engine_lib):
    """The product path is the in-tree CUDA library: no fallback exists."""
    import ctypes
    e = engine_lib.GpuEngine(scenes.cluster(n=8))
    e.run(2)
    assert engine_lib._lib is not None and engine_lib._lib._name.endswith("libvedogpu.so")
    prof = e.last_run_profile()
    assert prof["launches"] >= 4
    del ctypes


def test_engine_from_xml_equals_engine_from_ido(engine_lib, tmp_path):
    """DOWorldSchema XML input (vedo_gpu_create_from_xml) runs exactly as the same scene's .ido."""
    sc = scenes.cluster(n=64, solver="ISwBSDBF", steps=300, seed=12)
    ido, xml = str(tmp_path / "s.ido"), str(tmp_path / "s.xml")
    sc.to_ido(ido)
    engine_lib.convert_scene(ido, xml)
    a = engine_lib.GpuEngine(ido, up_iact=5)
    b = engine_lib.GpuEngine(xml, up_iact=5)
    a.run(200)
    b.run(200)
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


def test_zone_of_interest_cleanup_in_both_forms(engine_lib):
    """A world with a zone of interest loses its mobile objects outside the zone before the first
    step, in both forms, and the survivors' contact sets agree."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "cluster_zoi.npz"))
    sc = Scene.from_ido(g["ido"].tobytes())
    a = engine_lib.GpuEngine(sc, up_iact=int(g["up_iact"]))
    b = engine_lib.GpuEngine(sc, up_iact=int(g["up_iact"]), precision=1)
    assert a.n == b.n == g["state_position"].shape[0] < sc.num_objects
    ia, ib = a.interactions(), b.interactions()
    A = set(zip(ia["first"][ia["active"] == 1].tolist(), ia["second"][ia["active"] == 1].tolist()))
    B = set(zip(ib["first"][ib["active"] == 1].tolist(), ib["second"][ib["active"] == 1].tolist()))
    assert A == B
    np.testing.assert_array_equal(a.state(("position",))["position"], b.state(("position",))["position"])


@pytest.mark.parametrize("precision", [0, 1])
def test_external_impulses_equal_a_constant_external_force(precision, engine_lib):
    """vedo_gpu_run_with_impulses (SimMediator::Run with external impacts): a step that adds
    F dt to every sphere equals a step of the same world whose sphere model carries the external
    force F (DiscreteObject::AddConstrainedImpact adds dt F just before): bit for bit in the
    FP64 form (the same sums in the same order), within FP32 roundings in the MIXED form."""
    import copy
    F = np.array([0.02, -0.01, 0.005])
    sa = scenes.cluster(n=48, solver="ISwBSDBF", steps=400, seed=5)
    sb = copy.deepcopy(sa)
    sa.models[0].external_force = tuple(F)
    dt = sa.sp.time_interval
    a = engine_lib.GpuEngine(sa, up_iact=5, precision=precision)
    b = engine_lib.GpuEngine(sb, up_iact=5, precision=precision)
    imp = np.zeros((b.n, 3))
    imp[sb.model_index == 0] = F * dt
    for _ in range(120 if precision == 0 else 3):   # FP32 roundings grow along a chaotic trajectory
        a.run(1)
        b.run_with_impulses(imp, None)
    ra, rb = a.state(), b.state()
    for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
        if precision == 0:
            np.testing.assert_array_equal(ra[k], rb[k], err_msg=k)
        else:
            np.testing.assert_allclose(ra[k], rb[k], rtol=1e-5, atol=1e-7 * (np.abs(ra[k]).max() + 1e-30),
                                       err_msg=k)
    assert np.abs(ra["velocity"] - scenes.cluster(n=48, solver="ISwBSDBF", steps=400, seed=5).velocity).max() > 0


def test_periodic_layer_at_size_bitexact(engine_lib, port_lib):
    """A 12 x 12 x 4 layer drifting across both periodic faces: 300 steps with rebuilds every 5,
    the FP64 form bit for bit against the oracle (the wrap after Response, the minimum image in
    the sphere detector and in the lever arms, the FP32 prefilter's periodic distance bound)."""
    from oracle import PortWorld
    sc = scenes.periodic_layer(nx=12, ny=12, layers=4, seed=21, steps=400)
    e = engine_lib.GpuEngine(sc, up_iact=5)
    p = PortWorld(sc, up_iact=5)
    x0 = sc.position[:, 0].copy()
    for _ in range(3):
        e.run(100)
        p.run(100)
        a, b = e.state(), p.state()
        for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
        ia = e.interactions()
        f, s = p.candidates()
        assert np.array_equal(ia["first"], f) and np.array_equal(ia["second"], s)
        assert np.array_equal(ia["active"].astype(bool), p.interactions()["active"].astype(bool))
    lo, hi = sc.sp.pbc.lower[0], sc.sp.pbc.upper[0]
    x = a["position"][:-1, 0]
    assert np.all((x >= lo) & (x < hi))
    assert np.sum(x < x0[:-1] - 0.5 * (hi - lo)) > 10          # spheres that went out at the upper face


def test_mixed_form_refuses_periodic_layouts_it_cannot_run(engine_lib):
    """The mixed form runs periodic scenes (tests/test_gpu_periodic_mixed.py) but refuses, with
    VEDO_ERR_UNSUPPORTED_MODEL, a periodic range shorter than three cells of 2 r_max + skin and
    walls outside the periodic box (the reference's wrap would move them; the mixed form keeps
    walls where they are)."""
    small = scenes.periodic_layer(nx=3, ny=3, layers=2, seed=3)       # 3 spheres per period
    with pytest.raises(engine_lib.EngineError) as ex:
        engine_lib.GpuEngine(small, precision=1, skin=0.5)
    assert ex.value.code == 3
    walls_out = scenes.periodic_layer(nx=8, ny=8, layers=2, periodic_y=False, side_walls=True, seed=9)
    with pytest.raises(engine_lib.EngineError) as ex:
        engine_lib.BatchEngine([walls_out])
    assert ex.value.code == 3


def test_step_and_contacts_entry_points_equal_run_and_interactions(engine_lib):
    """vedo_gpu_step / vedo_gpu_get_contacts (the names of the step and contacts contract) do what
    vedo_gpu_run / vedo_gpu_get_interactions do."""
    import ctypes as C
    from vedo_gb300.engine import lib
    L = lib()
    L.vedo_gpu_step.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_int)]
    L.vedo_gpu_get_contacts.argtypes = [C.c_void_p, C.POINTER(engine_lib.ContactView)]
    sc = scenes.cluster(n=48, solver="ISwBSDBF", steps=400, seed=5)
    a, b = engine_lib.GpuEngine(sc, up_iact=5), engine_lib.GpuEngine(sc, up_iact=5)
    keep = C.c_int(0)
    assert L.vedo_gpu_step(a.h, 150, C.byref(keep)) == 0 and keep.value == 1
    b.run(150)
    for k, v in a.state().items():
        np.testing.assert_array_equal(v, b.state()[k], err_msg=k)
    ib = b.interactions()
    m = len(ib["first"])
    first, second = np.zeros(m, np.uint32), np.zeros(m, np.uint32)
    active = np.zeros(m, np.uint8)
    shear = np.zeros((m, 3))
    view = engine_lib.ContactView()
    view.first = first.ctypes.data_as(C.POINTER(C.c_uint32))
    view.second = second.ctypes.data_as(C.POINTER(C.c_uint32))
    view.active = active.ctypes.data_as(C.POINTER(C.c_uint8))
    view.shear = shear.ctypes.data_as(C.POINTER(C.c_double))
    assert L.vedo_gpu_get_contacts(a.h, C.byref(view)) == 0
    np.testing.assert_array_equal(first, ib["first"])
    np.testing.assert_array_equal(second, ib["second"])
    np.testing.assert_array_equal(active.astype(bool), ib["active"].astype(bool))
    np.testing.assert_array_equal(shear, ib["shear"])
    a.close()
    b.close()


@pytest.mark.parametrize("which", ["periodic", "box"])
def test_leap_consultant_at_size_bitexact(which, engine_lib, port_lib):
    """The Leap consultant's candidate list on the device: a 12 x 12 x 4 periodic layer (neighbour
    zones wrapping across both periodic faces) and the 8,000-sphere box; candidate lists element
    for element and states bit for bit against the oracle, with rebuilds every 5 / 20 steps."""
    from oracle import PortWorld
    if which == "periodic":
        sc, up, steps = scenes.periodic_layer(nx=12, ny=12, layers=4, seed=21, steps=400), 5, 200
    else:
        sc, up, steps = scenes.lsd_box(), 20, 200
    e = engine_lib.GpuEngine(sc, up_iact=up, consultant="leap")
    p = PortWorld(sc, up_iact=up, consultant="leap")
    for _ in range(2):
        ia = e.interactions()
        f, s = p.candidates()
        assert np.array_equal(ia["first"], f) and np.array_equal(ia["second"], s)
        e.run(steps // 2)
        p.run(steps // 2)
    a, b = e.state(), p.state()
    for k in ("position", "velocity", "angular_velocity", "impact", "angular_impact"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    nbs = engine_lib.GpuEngine(sc, up_iact=up)
    assert len(nbs.interactions()["first"]) != len(e.interactions()["first"]) or which == "box"
    e.close()
    nbs.close()


def test_leap_self_pairs_are_refused_by_the_engine(engine_lib):
    """A periodic axis one Leap zone wide gives the reference's list pairs (i, i): the engine refuses
    the scene with VEDO_ERR_UNSUPPORTED_MODEL, as the oracle does, instead of building an
    interaction of a sphere with itself."""
    sc = scenes.periodic_layer(nx=6, ny=2, layers=3, solver="ISwBSDBF", seed=32, periodic_y=True,
                               drift=(-0.74, -1.06))
    with pytest.raises(engine_lib.EngineError) as ex:
        engine_lib.GpuEngine(sc, up_iact=4, consultant="leap")
    assert ex.value.code == 3
    engine_lib.GpuEngine(sc, up_iact=4).close()     # the NBS list of the same layer is fine


@pytest.mark.parametrize("case", ["box_lsd", "cluster_ISwH"])
def test_system_status_csv_matches_reference(case, engine_lib, tmp_path):
    """With an output prefix the FP64 form writes SystemStatus.csv as SimMediator does
    (SimMediator.cpp:46-123): the same header, a line at creation and at every reset, the same
    record and contact counts, and energies that print the same to the reference's 6 digits
    (compared as numbers: the reductions add in another order)."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "status", f"{case}.npz"))
    sc = Scene.from_ido(g["ido"].tobytes())
    e = engine_lib.GpuEngine(sc, up_iact=int(g["up_iact"]), output_prefix=str(tmp_path / "w"))
    e.run(int(g["steps"]))
    e.close()
    got = (tmp_path / "SystemStatus.csv").read_text().splitlines()
    ref = g["csv"].tobytes().decode().splitlines()
    assert got[0] == ref[0]
    assert len(got) == len(ref)
    for a, b in zip(got[1:], ref[1:]):
        fa, fb = [x.strip() for x in a.split(",")], [x.strip() for x in b.split(",")]
        assert len(fa) == len(fb)
        assert fa[1:4] == fb[1:4], (a, b)                 # objects, records, contacts
        np.testing.assert_allclose([float(x) for x in fa], [float(x) for x in fb], rtol=1e-5, atol=1e-300,
                                   err_msg=f"{a} | {b}")
