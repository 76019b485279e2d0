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
