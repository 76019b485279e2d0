"""GPU tests of scene batches (vedo_gpu_create_batch): many independent scenes advanced by one
MIXED-form engine with one fused launch per step.

The bar is isolation: a scene's results inside a batch are bit-identical to the same scene run
alone, whatever else shares the batch and in whatever order."""
import numpy as np
import pytest

from vedo_gb300 import scenes

pytestmark = pytest.mark.gpu

FIELDS = ("position", "velocity", "angular_velocity", "impact", "angular_impact")


def _alone(engine_lib, sc, steps):
    e = engine_lib.GpuEngine(sc, precision=1)
    e.run(steps)
    st = e.state(FIELDS)
    it = e.interactions()
    t = e.time()
    e.close()
    return st, it, t


def _contact_rows(it, off=0, count=None):
    a = it["active"] == 1
    f, s = it["first"][a].astype(np.int64) - off, it["second"][a].astype(np.int64) - off
    keep = (f >= 0) & (f < count) if count is not None else np.ones_like(f, bool)
    return sorted(zip(f[keep].tolist(), s[keep].tolist(), it["kn"][a][keep].tolist()))


@pytest.fixture(scope="module")
def mix(box_ido, drum_ido):
    from vedo_gb300.scene import Scene
    return [Scene.from_ido(box_ido), scenes.cluster(n=64, solver="ISwBSDBF", steps=500, seed=21),
            Scene.from_ido(drum_ido), scenes.cluster(n=48, solver="ISwH", steps=500, seed=5, walls="box")]


def test_batch_scene_equals_alone(engine_lib, mix):
    steps = 300
    b = engine_lib.BatchEngine(mix)
    assert b.num_scenes == len(mix)
    b.run(steps)
    st = b.state(FIELDS)
    it = b.interactions()
    for s, sc in enumerate(mix):
        ref, rit, rt = _alone(engine_lib, sc, steps)
        f, c, t = b.scene_range(s)
        assert c == sc.num_objects
        assert t == rt
        for k in FIELDS:
            assert np.array_equal(st[k][f:f + c], ref[k]), (s, k)
        assert _contact_rows(it, f, c) == _contact_rows(rit), s


def test_batch_order_does_not_matter(engine_lib, mix):
    a = engine_lib.BatchEngine(mix)
    b = engine_lib.BatchEngine(mix[::-1])
    a.run(200)
    b.run(200)
    sa, sb = a.state(FIELDS), b.state(FIELDS)
    S = len(mix)
    for s in range(S):
        fa, ca, _ = a.scene_range(s)
        fb, cb, _ = b.scene_range(S - 1 - s)
        for k in FIELDS:
            assert np.array_equal(sa[k][fa:fa + ca], sb[k][fb:fb + cb]), (s, k)


def test_batch_rejects_fp64_and_empty(engine_lib, mix):
    import ctypes as C
    L = engine_lib.lib()
    h = C.c_void_p()
    opts = engine_lib._opts(1, 0, 0, 0, None, None, None)
    arr = (C.POINTER(engine_lib._abi.SceneDesc) * 1)()
    assert L.vedo_gpu_create_batch(arr, 0, C.byref(opts), C.byref(h)) == 1
    d, keep = engine_lib.scene_to_desc(mix[1])
    arr[0] = C.pointer(d)
    assert L.vedo_gpu_create_batch(arr, 1, C.byref(opts), C.byref(h)) == 1     # FP64 form
    assert not h.value


def test_autotuned_graph_batch_equals_plain_alone(engine_lib):
    """Hoppers of uneven sizes in one autotuned batch whose check intervals replay as CUDA
    graphs, against each hopper alone with fixed settings and direct launches: bit-identical,
    because neither the tuned skin, cell scale and block size nor graph replay change a result."""
    steps = 500                                   # the tuner needs about 400 steps of the call
    hs = [scenes.hopper(n=n, seed=s, friction=mu, restitution=e, orifice=w, steps=steps)
          for n, s, mu, e, w in scenes.hopper_params(4, seed=7, n_lo=1000, n_hi=6000)]
    b = engine_lib.BatchEngine(hs, autotune=True)
    b.run(steps)
    tune = b.tuning()
    assert tune["tick_block"] in (64, 128, 256) and tune["cell_scale"] >= 1.0 and tune["skin"] > 0
    st = b.state(FIELDS)
    for s, sc in enumerate(hs):
        e = engine_lib.GpuEngine(sc, precision=1, graphs=False, skin=0.15, tick_block=256)
        e.run(steps)
        ref = e.state(FIELDS)
        e.close()
        f, c, t = b.scene_range(s)
        for k in FIELDS:
            assert np.array_equal(st[k][f:f + c], ref[k]), (s, k)
    # the spheres are falling: the discharge is under way
    assert (st["velocity"][:, 2] < -0.01).sum() > 0
