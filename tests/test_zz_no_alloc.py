"""vedo_gpu_system_energy_noalloc (no device allocation, fixed scratch array) against the
engine's vedo_gpu_get_observables on the same state, through the C ABI.

Tolerance: sums agree within 1e-12 relative (the two reductions add in different orders);
minima and maxima are exact."""
import ctypes as C

import numpy as np
import pytest

from vedo_gb300 import scenes
from vedo_gb300.scene import MOBILE


def _entry(engine_lib):
    f = engine_lib.lib().vedo_gpu_system_energy_noalloc
    f.argtypes = [C.c_void_p] * 6 + [C.c_uint32, C.POINTER(C.c_double), C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _per_object(sc):
    n = sc.num_objects
    mass, inertia, mobile = np.zeros(n), np.zeros((n, 3)), np.zeros(n, np.uint8)
    for k, m in enumerate(sc.models):
        sel = np.asarray(sc.model_index) == k
        _, _, mk, _, inr = m.analysis()
        mass[sel], inertia[sel], mobile[sel] = mk, inr, 1 if m.behavior == MOBILE else 0
    return mass, inertia, mobile


def _check(got, ref):
    scale = np.abs(ref).max()
    for k in (0, 1, 2, 7, 8):
        assert abs(got[k] - ref[k]) <= 1e-12 * max(abs(ref[k]), 1e-30 * scale), (k, got[k], ref[k])
    for k in (3, 4, 5, 6):
        assert got[k] == ref[k], (k, got[k], ref[k])
    for k in range(3):
        assert abs(got[9 + k] - ref[10 + k]) <= 1e-12 * np.abs(ref[10:13]).max(), (k, got[9 + k], ref[10 + k])


@pytest.mark.gpu
def test_noalloc_energy_equals_engine_observables_twice(engine_lib):
    torch = pytest.importorskip("torch")
    f = _entry(engine_lib)
    sc = scenes.cluster(n=3000, solver="ISwBSDBF", polydisperse=True, steps=2000, seed=3)
    mass, inertia, mobile = _per_object(sc)
    dev = {k: torch.from_numpy(np.ascontiguousarray(a)).cuda() for k, a in
           (("mass", mass), ("inertia", inertia), ("mobile", mobile))}
    out = torch.full((12,), float("nan"), dtype=torch.float64, device="cuda")
    g = (C.c_double * 3)(*sc.sp.field_acceleration)
    e = engine_lib.GpuEngine(sc, up_iact=5)
    for call in range(2):                       # two calls in a row, on different states
        e.run(200)
        st = e.state(("position", "velocity", "angular_velocity"))
        ref = e.observables()
        x = {k: torch.from_numpy(st[k]).cuda() for k in st}
        stream = torch.cuda.current_stream()
        rc = f(x["position"].data_ptr(), x["velocity"].data_ptr(), x["angular_velocity"].data_ptr(),
               dev["mass"].data_ptr(), dev["inertia"].data_ptr(), dev["mobile"].data_ptr(), sc.num_objects, g,
               out.data_ptr(), stream.cuda_stream)
        assert rc == 0, engine_lib.lib().vedo_gpu_last_error(None)
        stream.synchronize()
        got = out.cpu().numpy()
        assert ref[1] > 0.0 and ref[2] > 0.0, call
        _check(got, ref)
    e.close()


@pytest.mark.gpu
def test_noalloc_many_blocks_without_mobile_flags_and_no_new_memory(engine_lib):
    """100,000 objects (more than 32 blocks of partial sums) with every object counted
    (mobile = NULL), against a plain FP64 reduction of the same arrays; after a warm-up call,
    a second call leaves the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    f = _entry(engine_lib)
    rng = np.random.default_rng(11)
    n = 100_000
    p, v, w = rng.normal(0, 0.1, (n, 3)), rng.normal(0, 1.0, (n, 3)), rng.normal(0, 50.0, (n, 3))
    m = rng.uniform(1e-6, 1e-5, n)
    inertia = np.repeat((0.4 * m * 1e-6)[:, None], 3, axis=1)
    x = {k: torch.from_numpy(np.ascontiguousarray(a)).cuda() for k, a in
         (("p", p), ("v", v), ("w", w), ("m", m), ("i", inertia))}
    out = torch.full((12,), float("nan"), dtype=torch.float64, device="cuda")
    g = (C.c_double * 3)(0.0, 0.0, -9.81)
    stream = torch.cuda.current_stream()
    args = (x["p"].data_ptr(), x["v"].data_ptr(), x["w"].data_ptr(), x["m"].data_ptr(), x["i"].data_ptr(), None,
            n, g, out.data_ptr(), stream.cuda_stream)
    assert f(*args) == 0, engine_lib.lib().vedo_gpu_last_error(None)        # warm-up call
    stream.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    assert f(*args) == 0, engine_lib.lib().vedo_gpu_last_error(None)
    stream.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    got = out.cpu().numpy()
    ke_t = np.sum(0.5 * m * np.sum(v * v, axis=1))
    ke_r = np.sum(0.5 * inertia * w * w)
    pe = -np.sum(m * (p @ np.array([0.0, 0.0, -9.81])))
    com = (m[:, None] * p).sum(axis=0) / m.sum()
    for k, ref in ((0, pe), (1, ke_t), (2, ke_r)):
        assert abs(got[k] - ref) <= 1e-12 * abs(ref), (k, got[k], ref)
    speed, spin = np.linalg.norm(v, axis=1), np.linalg.norm(w, axis=1)
    for k, ref in ((3, speed.min()), (4, speed.max()), (5, spin.min()), (6, spin.max())):
        assert abs(got[k] - ref) <= 1e-15 * ref, (k, got[k], ref)        # one rounding of the norm
    np.testing.assert_allclose(got[9:12], com, rtol=0, atol=1e-12 * np.abs(p).max())


@pytest.mark.gpu
def test_noalloc_rejects_host_buffers(engine_lib):
    f = _entry(engine_lib)
    g = (C.c_double * 3)(0.0, 0.0, -9.81)
    host = np.zeros((4, 3))
    hp = host.ctypes.data
    rc = f(hp, hp, hp, hp, hp, None, 4, g, hp, None)
    assert rc == 1
    assert b"device memory" in engine_lib.lib().vedo_gpu_last_error(None)


def test_noalloc_rejects_more_objects_than_its_scratch(engine_lib):
    """Refused before any CUDA call: runs without a GPU."""
    f = _entry(engine_lib)
    g = (C.c_double * 3)(0.0, 0.0, -9.81)
    too_many = 16777216 + 1
    rc = f(1, 1, 1, 1, 1, None, too_many, g, 1, None)
    assert rc == 1
    assert b"16777216" in engine_lib.lib().vedo_gpu_last_error(None)
