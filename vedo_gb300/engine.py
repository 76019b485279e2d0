"""ctypes binding of the GPU engine (``vedo_gb300/_build/libvedogpu.so``, C ABI of include/vedo_gpu.h).

:class:`GpuEngine` is the host-side mirror of the reference's ``SimMediator``
(src/vedo/framework/SimMediator.h:22-36): construct it from a scene (or an ``.ido``
file, as ``anne`` does) and call :meth:`Run` once per time step, or :meth:`run` for
many steps at a time.  There is no CPU fallback: if the CUDA library is missing or no
GPU is present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, Optional

import numpy as np

from . import _abi
from ._abi import ContactView, EngineOpts, StateView, dptr, scene_to_desc
from .scene import Scene

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libvedogpu.so")

_lib = None


class EngineError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load the engine library (fails loudly when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m vedo_gb300.build`")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.vedo_gpu_default_opts.argtypes = [C.POINTER(EngineOpts)]
        L.vedo_gpu_create.argtypes = [C.POINTER(_abi.SceneDesc), C.POINTER(EngineOpts), C.POINTER(vp)]
        L.vedo_gpu_create_from_ido.argtypes = [C.c_char_p, C.POINTER(EngineOpts), C.POINTER(vp)]
        L.vedo_gpu_create_from_xml.argtypes = [C.c_char_p, C.POINTER(EngineOpts), C.POINTER(vp)]
        L.vedo_convert_scene.argtypes = [C.c_char_p, C.c_char_p]
        L.vedo_gpu_run.argtypes = [vp, C.c_uint32, C.POINTER(C.c_int)]
        L.vedo_gpu_num_objects.argtypes = [vp]
        L.vedo_gpu_num_objects.restype = C.c_uint32
        L.vedo_gpu_get_state.argtypes = [vp, C.POINTER(StateView)]
        L.vedo_gpu_set_state.argtypes = [vp, C.POINTER(StateView)]
        L.vedo_gpu_num_interactions.argtypes = [vp, C.POINTER(C.c_uint32)]
        L.vedo_gpu_get_interactions.argtypes = [vp, C.POINTER(ContactView)]
        L.vedo_gpu_get_observables.argtypes = [vp, C.POINTER(C.c_double)]
        L.vedo_gpu_time.argtypes = [vp]
        L.vedo_gpu_time.restype = C.c_double
        L.vedo_gpu_step_count.argtypes = [vp]
        L.vedo_gpu_step_count.restype = C.c_uint64
        L.vedo_gpu_steps_remaining.argtypes = [vp]
        L.vedo_gpu_steps_remaining.restype = C.c_uint64
        L.vedo_gpu_write_ido.argtypes = [vp, C.c_char_p]
        L.vedo_gpu_coordination.argtypes = [vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]
        L.vedo_gpu_write_vtk.argtypes = [vp, C.c_char_p, C.c_int]
        L.vedo_gpu_last_run_profile.argtypes = [vp, C.POINTER(C.c_double)]
        L.vedo_gpu_last_run_profile.restype = C.c_uint64
        L.vedo_gpu_set_profiling.argtypes = [vp, C.c_int]
        L.vedo_gpu_last_error.argtypes = [vp]
        L.vedo_gpu_last_error.restype = C.c_char_p
        L.vedo_gpu_destroy.argtypes = [vp]
        L.vedo_gpu_version.restype = C.c_char_p
        L.vedo_gpu_create_batch.argtypes = [C.POINTER(C.POINTER(_abi.SceneDesc)), C.c_uint32,
                                            C.POINTER(EngineOpts), C.POINTER(vp)]
        L.vedo_gpu_num_scenes.argtypes = [vp]
        L.vedo_gpu_num_scenes.restype = C.c_uint32
        L.vedo_gpu_scene_range.argtypes = [vp, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                           C.POINTER(C.c_double)]
        L.vedo_gpu_get_tuning.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_uint32),
                                          C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.vedo_gpu_barrier_check.argtypes = [C.c_int32, C.c_uint32, C.c_uint32, C.c_uint64,
                                             C.POINTER(C.c_uint32)]
        _lib = L
    return _lib


STATE_FIELDS = ("position", "velocity", "angular_velocity", "orientation_x", "orientation_z", "impact",
                "angular_impact")


def _opts(up_iact, record, precision, device, prefix, skin, check_interval, tick_block=None, cell_scale=None,
          autotune=False, graphs=True, stored_splits=False, split_tick=False, full_walks=False,
          consultant="nbs", pair_pass=False, orientations=False, persistent=False) -> EngineOpts:
    opts = EngineOpts()
    lib().vedo_gpu_default_opts(C.byref(opts))
    opts.up_iact, opts.record, opts.precision, opts.device = up_iact, record, precision, device
    if skin is not None:
        opts.skin = skin
    if check_interval is not None:
        opts.check_interval = check_interval
    if tick_block is not None:
        opts.tick_block = tick_block
    if cell_scale is not None:
        opts.cell_scale = cell_scale
    opts.autotune = 1 if autotune else 0
    opts.graphs = 1 if graphs else 0
    opts.stored_splits = 1 if stored_splits else 0
    if split_tick and pair_pass:
        raise ValueError("split_tick and pair_pass are two forms of the tick: choose one")
    opts.split_tick = 2 if pair_pass else (1 if split_tick else 0)
    opts.full_walks = 1 if full_walks else 0
    opts.orientations = 1 if orientations else 0
    opts.persistent = 1 if persistent else 0
    if consultant not in ("nbs", "leap"):
        raise ValueError(f"consultant must be 'nbs' or 'leap', not {consultant!r}")
    opts.consultant = 1 if consultant == "leap" else 0
    opts.output_prefix = prefix
    return opts


class GpuEngine:
    """One scene on one GPU.

    Parameters mirror ``anne analysis <ido> <nbs|leap> <Record> <UpIact>`` (Anne.cpp:38-128):
    `up_iact` is the candidate-list rebuild interval, `record` the IDO record interval
    (0 = never), `output_prefix` where record/terminate IDO files go (None = none) and
    `consultant` whose candidate list the FP64 form builds.
    """

    def __init__(self, scene, up_iact: int = 1, record: int = 0, precision: int = _abi.PRECISION_FP64,
                 device: int = 0, output_prefix: Optional[str] = None, skin: Optional[float] = None,
                 check_interval: Optional[int] = None, tick_block: Optional[int] = None,
                 cell_scale: Optional[float] = None, autotune: bool = False, graphs: bool = True,
                 stored_splits: bool = False, split_tick: bool = False, full_walks: bool = False,
                 consultant: str = "nbs", pair_pass: bool = False, orientations: bool = False,
                 persistent: bool = False):
        L = lib()
        self._prefix = output_prefix.encode() if output_prefix else None
        opts = _opts(up_iact, record, precision, device, self._prefix, skin, check_interval, tick_block, cell_scale,
                     autotune, graphs, stored_splits, split_tick, full_walks, consultant, pair_pass, orientations,
                     persistent)
        h = C.c_void_p()
        if isinstance(scene, (str, bytes, os.PathLike)):
            path = os.fsencode(scene)
            make = L.vedo_gpu_create_from_xml if path.endswith(b".xml") else L.vedo_gpu_create_from_ido
            rc = make(path, C.byref(opts), C.byref(h))
        else:
            desc, keep = scene_to_desc(scene)
            rc = L.vedo_gpu_create(C.byref(desc), C.byref(opts), C.byref(h))
            del keep
        if rc != 0:
            raise EngineError(rc, L.vedo_gpu_last_error(None).decode())
        self.h = h

    @property
    def n(self) -> int:
        """Objects now: the Leap consultant's zone-of-interest clean-up erases objects at resets
        (LeapConsultant.cpp:61-68), so the count is read after every call that steps."""
        return lib().vedo_gpu_num_objects(self.h)

    def _check(self, rc: int):
        if rc != 0:
            raise EngineError(rc, lib().vedo_gpu_last_error(self.h).decode())

    # SimMediator::Run (SimMediator.cpp:714-842): one step, returns t < t_stop
    def Run(self) -> bool:
        return self.run(1)

    def run(self, nsteps: int) -> bool:
        keep = C.c_int(0)
        self._check(lib().vedo_gpu_run(self.h, nsteps, C.byref(keep)))
        return bool(keep.value)

    def state(self, fields=STATE_FIELDS, out: Optional[Dict[str, np.ndarray]] = None) -> Dict[str, np.ndarray]:
        """Copy object state to host arrays ([n][3] float64); `out` may supply (pinned) buffers."""
        if out is None:
            out = {f: np.zeros((self.n, 3)) for f in fields}
        for f in fields:
            a = out[f]
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != (self.n, 3):
                raise ValueError(f"out[{f!r}] must be a C-contiguous float64 array of shape ({self.n}, 3)")
        v = StateView()
        for f in fields:
            setattr(v, f, dptr(out[f]))
        self._check(lib().vedo_gpu_get_state(self.h, C.byref(v)))
        return out

    def set_state(self, **arrays):
        v = StateView()
        keep = []
        for f, a in arrays.items():
            a = np.ascontiguousarray(a, dtype=np.float64).reshape(self.n, 3)
            keep.append(a)
            setattr(v, f, dptr(a))
        self._check(lib().vedo_gpu_set_state(self.h, C.byref(v)))

    def interactions(self) -> Dict[str, np.ndarray]:
        n = C.c_uint32(0)
        self._check(lib().vedo_gpu_num_interactions(self.h, C.byref(n)))
        m = n.value
        out = dict(first=np.zeros(m, np.uint32), second=np.zeros(m, np.uint32), slave=np.zeros(m, np.uint32),
                   master=np.zeros(m, np.uint32), active=np.zeros(m, np.uint8), shear=np.zeros((m, 3)),
                   kn=np.zeros(m), contact=np.zeros(m, np.uint8))
        v = ContactView()
        for k in ("first", "second", "slave", "master"):
            setattr(v, k, _abi.uptr(out[k]))
        v.active, v.contact = _abi.bptr(out["active"]), _abi.bptr(out["contact"])
        v.shear, v.kn = dptr(out["shear"]), dptr(out["kn"])
        self._check(lib().vedo_gpu_get_interactions(self.h, C.byref(v)))
        return out

    def observables(self) -> np.ndarray:
        o = np.zeros(13)
        self._check(lib().vedo_gpu_get_observables(self.h, dptr(o)))
        return o

    def time(self) -> float:
        return lib().vedo_gpu_time(self.h)

    def step_count(self) -> int:
        return lib().vedo_gpu_step_count(self.h)

    def steps_remaining(self) -> int:
        """Run() calls left before t >= t_stop."""
        return lib().vedo_gpu_steps_remaining(self.h)

    def write_ido(self, path: str):
        self._check(lib().vedo_gpu_write_ido(self.h, os.fsencode(path)))

    def coordination(self, box=None):
        """CalcCoordinateNum on the device: (below, touching, average) - per object the other
        spheres whose centre distance is below / at most the radius sum (0 for walls), and with
        box = (xmin, xmax, ymin, ymax, zmin, zmax) computeAvgCoordinateNum over it (else None)."""
        below = np.zeros(self.n, np.uint32)
        touching = np.zeros(self.n, np.uint32)
        up = C.POINTER(C.c_uint32)
        if box is None:
            self._check(lib().vedo_gpu_coordination(self.h, below.ctypes.data_as(up), touching.ctypes.data_as(up),
                                                     None, None))
            return below, touching, None
        b = np.ascontiguousarray(box, dtype=np.float64)
        avg = C.c_double(0.0)
        self._check(lib().vedo_gpu_coordination(self.h, below.ctypes.data_as(up), touching.ctypes.data_as(up),
                                                 dptr(b), C.byref(avg)))
        return below, touching, float(avg.value)

    def write_vtk(self, path: str, with_coordination: bool = False):
        """The current state as a VTK file (DOWorld::WriteVTK), with the spheres' coordination
        numbers when asked (CalcCoordinateNum::outputCoordinateNumVTK)."""
        self._check(lib().vedo_gpu_write_vtk(self.h, os.fsencode(path), 1 if with_coordination else 0))

    def tuning(self):
        """Skin (fraction of r_max), cell scale, tick block size, split storage, the form of the
        tick (single, split or pair pass) and whether a check interval is one persistent launch,
        in use (MIXED form)."""
        sk, cs, tb, ss, st, pe = (C.c_float(0), C.c_float(0), C.c_uint32(0), C.c_uint32(0), C.c_uint32(0),
                                  C.c_uint32(0))
        self._check(lib().vedo_gpu_get_tuning(self.h, C.byref(sk), C.byref(cs), C.byref(tb), C.byref(ss),
                                              C.byref(st), C.byref(pe)))
        return {"skin": float(sk.value), "cell_scale": float(cs.value), "tick_block": int(tb.value),
                "stored_splits": bool(ss.value), "split_tick": st.value == 1, "pair_pass": st.value == 2,
                "persistent": bool(pe.value)}

    def run_with_impulses(self, impulse=None, angular_impulse=None) -> bool:
        """One step with an external impulse and angular impulse per object ([n, 3] arrays in
        object order; None = zeros), as the reference's SimMediator::Run(external impacts)."""
        keep = C.c_int(0)
        args = []
        for a in (impulse, angular_impulse):
            if a is None:
                args.append(None)
            else:
                a = np.ascontiguousarray(a, dtype=np.float64).reshape(self.n, 3)
                args.append(a)
        self._check(lib().vedo_gpu_run_with_impulses(self.h, dptr(args[0]) if args[0] is not None else None,
                                                     dptr(args[1]) if args[1] is not None else None,
                                                     C.byref(keep)))
        return bool(keep.value)

    def list_status(self) -> Dict[str, float]:
        """Neighbour-list state (MIXED form): steps since the rebuild, rebuilds, displacement
        bounds (relative to the scene frame, absolute, orbital walls) and the share of the
        list's life used."""
        o = np.zeros(6)
        self._check(lib().vedo_gpu_list_status(self.h, dptr(o)))
        return {"steps": int(o[0]), "rebuilds": int(o[1]), "rel": float(o[2]), "abs": float(o[3]),
                "wall": float(o[4]), "use": float(o[5])}

    def quiet_spheres(self) -> int:
        """Spheres whose next step skips the neighbour-list walk (MIXED form; 0 for FP64)."""
        c = C.c_uint64(0)
        self._check(lib().vedo_gpu_quiet_spheres(self.h, C.byref(c)))
        return int(c.value)

    def set_profiling(self, on: bool):
        lib().vedo_gpu_set_profiling(self.h, 1 if on else 0)

    def last_run_profile(self):
        o = np.zeros(4)
        launches = lib().vedo_gpu_last_run_profile(self.h, dptr(o))
        return {"pair_ms": float(o[0]), "object_ms": float(o[1]), "rebuild_ms": float(o[2]),
                "total_ms": float(o[3]), "launches": int(launches)}

    def close(self):
        if getattr(self, "h", None):
            lib().vedo_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def convert_scene(src: str, dst: str):
    """Convert a scene file between .ido and DOWorldSchema .xml, or write it as a VTK .vtu file
    (by extension); no GPU needed."""
    L = lib()
    rc = L.vedo_convert_scene(os.fsencode(src), os.fsencode(dst))
    if rc != 0:
        raise EngineError(rc, L.vedo_gpu_last_error(None).decode())


class BatchEngine(GpuEngine):
    """Many independent scenes advanced together by one MIXED-form engine.

    Objects are numbered scene after scene; :meth:`scene_range` gives a scene's
    ``(first, count, time)`` and :meth:`scene_state` its slice of the state.  Each
    scene's results are bit-identical to the same scene run alone in the MIXED form.
    """

    def __init__(self, scene_list, device: int = 0, skin: Optional[float] = None,
                 check_interval: Optional[int] = None, tick_block: Optional[int] = None,
                 cell_scale: Optional[float] = None, autotune: bool = False, graphs: bool = True,
                 full_walks: bool = False, split_tick: bool = False, pair_pass: bool = False,
                 orientations: bool = False, persistent: bool = False, stored_splits: bool = False):
        L = lib()
        self._prefix = None
        opts = _opts(1, 0, _abi.PRECISION_MIXED, device, None, skin, check_interval, tick_block, cell_scale,
                     autotune, graphs, stored_splits=stored_splits, split_tick=split_tick, full_walks=full_walks,
                     pair_pass=pair_pass, orientations=orientations, persistent=persistent)
        descs, keeps = [], []
        for sc in scene_list:
            if isinstance(sc, (str, bytes, os.PathLike)):
                sc = Scene.from_ido(sc)
            d, k = scene_to_desc(sc)
            descs.append(d)
            keeps.append(k)
        arr = (C.POINTER(_abi.SceneDesc) * max(1, len(descs)))(*[C.pointer(d) for d in descs])
        h = C.c_void_p()
        rc = L.vedo_gpu_create_batch(arr, len(descs), C.byref(opts), C.byref(h))
        del keeps
        if rc != 0:
            raise EngineError(rc, L.vedo_gpu_last_error(None).decode())
        self.h = h
        self.num_scenes = L.vedo_gpu_num_scenes(h)

    def scene_range(self, s: int):
        f, c, t = C.c_uint32(0), C.c_uint32(0), C.c_double(0)
        self._check(lib().vedo_gpu_scene_range(self.h, s, C.byref(f), C.byref(c), C.byref(t)))
        return int(f.value), int(c.value), float(t.value)

    def scene_state(self, s: int, fields=STATE_FIELDS, state: Optional[Dict[str, np.ndarray]] = None):
        f, c, _ = self.scene_range(s)
        st = state if state is not None else self.state(fields)
        return {k: st[k][f:f + c] for k in fields}
