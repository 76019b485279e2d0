"""Python handles on the two CPU oracles (TEST INFRASTRUCTURE ONLY).

* :class:`PortWorld` drives ``oracle/_build/libdemport.so``, the plain-C
  restatement of the reference step (dem_oracle.c).  It builds on any host.
* :class:`RefWorld` drives ``oracle/_ref/libvedoref.so``, the reference's own
  CPU code compiled from its sources by ``make -C oracle ref``.  Only available
  where the reference sources are.

Both expose the same methods so that tests can compare them with each other
and with the GPU engine.  Only tests/, __graft_entry__.smoke() and the CPU
baseline of bench.py use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libdemport.so")
REF_LIB = os.path.join(HERE, "_ref", "libvedoref.so")
REF_SRC = os.environ.get("VEDO_REFERENCE", "/root/reference")

_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint32)
_ip = C.POINTER(C.c_int)


def build_port() -> str:
    """Compile the C oracle (make -C oracle port)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


def build_ref() -> Optional[str]:
    """Compile the reference CPU path when its sources are present; None otherwise."""
    if not os.path.isdir(os.path.join(REF_SRC, "src", "vedo")):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}", "-j8"], check=True)
    return REF_LIB


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def _d(a):
    return a.ctypes.data_as(_dp)


class _World:
    @property
    def n(self) -> int:
        """Objects now (the Leap consultant's zone-of-interest clean-up erases some at resets)."""
        return self._num_objects()

    def state(self) -> Dict[str, np.ndarray]:
        out = {k: np.zeros((self.n, 3)) for k in ("position", "velocity", "angular_velocity", "orientation_x",
                                                   "orientation_z", "impact", "angular_impact")}
        self._get_state(*[_d(out[k]) for k in ("position", "velocity", "angular_velocity", "orientation_x",
                                               "orientation_z", "impact", "angular_impact")])
        return out


class PortWorld(_World):
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(PORT_LIB):
                build_port()
            L = C.CDLL(PORT_LIB)
            L.dp_create.restype = C.c_void_p
            L.dp_create.argtypes = [C.c_void_p, C.c_uint, C.c_int, C.c_char_p, C.c_size_t]
            L.dp_run.argtypes = [C.c_void_p, C.c_uint]
            L.dp_num_objects.argtypes = [C.c_void_p]
            L.dp_num_objects.restype = C.c_uint
            L.dp_get_state.argtypes = [C.c_void_p] + [_dp] * 7
            L.dp_set_state.argtypes = [C.c_void_p] + [_dp] * 5
            L.dp_num_candidates.argtypes = [C.c_void_p]
            L.dp_num_candidates.restype = C.c_uint
            L.dp_get_candidates.argtypes = [C.c_void_p, _up, _up]
            L.dp_get_interactions.argtypes = [C.c_void_p, _up, _up, _ip, _dp, _dp, _dp, _dp, _ip]
            L.dp_time.argtypes = [C.c_void_p]
            L.dp_time.restype = C.c_double
            L.dp_energy.argtypes = [C.c_void_p, _dp]
            L.dp_coordination.argtypes = [C.c_void_p, _dp, _up, _up]
            L.dp_coordination.restype = C.c_double
            L.dp_destroy.argtypes = [C.c_void_p]
            cls._lib = L
        return cls._lib

    def __init__(self, scene, up_iact: int = 1, consultant: str = "nbs"):
        from vedo_gb300._abi import scene_to_desc
        L = self.lib()
        desc, keep = scene_to_desc(scene)
        err = C.create_string_buffer(256)
        self.h = L.dp_create(C.byref(desc), up_iact, 1 if consultant == "leap" else 0, err, 256)
        if not self.h:
            raise ValueError("oracle rejected the scene: " + err.value.decode())

    def _num_objects(self) -> int:
        return self.lib().dp_num_objects(self.h)

    def run(self, nsteps: int) -> int:
        return self.lib().dp_run(self.h, nsteps)

    def _get_state(self, *ptrs):
        self.lib().dp_get_state(self.h, *ptrs)

    def set_state(self, position=None, velocity=None, angular_velocity=None, orientation_x=None,
                  orientation_z=None):
        conv = [None if a is None else np.ascontiguousarray(a, np.float64) for a in
                (position, velocity, angular_velocity, orientation_x, orientation_z)]
        self.lib().dp_set_state(self.h, *[None if a is None else _d(a) for a in conv])

    def candidates(self):
        m = self.lib().dp_num_candidates(self.h)
        a = np.zeros(m, np.uint32)
        b = np.zeros(m, np.uint32)
        self.lib().dp_get_candidates(self.h, a.ctypes.data_as(_up), b.ctypes.data_as(_up))
        return a, b

    def interactions(self):
        m = self.lib().dp_num_candidates(self.h)
        out = dict(slave=np.zeros(m, np.uint32), master=np.zeros(m, np.uint32), active=np.zeros(m, np.int32),
                   depth=np.zeros(m), normal=np.zeros((m, 3)), shear=np.zeros((m, 3)), kn=np.zeros(m),
                   contact=np.zeros(m, np.int32))
        self.lib().dp_get_interactions(self.h, out["slave"].ctypes.data_as(_up), out["master"].ctypes.data_as(_up),
                                       out["active"].ctypes.data_as(_ip), _d(out["depth"]), _d(out["normal"]),
                                       _d(out["shear"]), _d(out["kn"]), out["contact"].ctypes.data_as(_ip))
        return out

    def time(self) -> float:
        return self.lib().dp_time(self.h)

    def energy(self) -> np.ndarray:
        e = np.zeros(9)
        self.lib().dp_energy(self.h, _d(e))
        return e

    def coordination(self, box=(0.0, 0.0, 0.0, 0.0, 0.0, 0.0)):
        """(below, touching, average): CalcCoordinateNum's per-object counts and box average."""
        below = np.zeros(self.n, np.uint32)
        touching = np.zeros(self.n, np.uint32)
        b = np.ascontiguousarray(box, dtype=np.float64)
        avg = self.lib().dp_coordination(self.h, _d(b), below.ctypes.data_as(_up), touching.ctypes.data_as(_up))
        return below, touching, avg

    def close(self):
        if getattr(self, "h", None):
            self.lib().dp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ref_coordination(scene, box, coord_vtk: Optional[str] = None, world_vtk: Optional[str] = None) -> float:
    """The reference's CalcCoordinateNum on `scene` (written as an IDO file): returns
    computeAvgCoordinateNum over box = (xmin, xmax, ymin, ymax, zmin, zmax); writes the
    coordination VTK file and the plain world VTK file when paths are given."""
    L = RefWorld.lib()
    with tempfile.TemporaryDirectory(prefix="vref_cn_") as td:
        path = os.path.join(td, "scene.ido")
        scene.to_ido(path)
        b = np.ascontiguousarray(box, dtype=np.float64)
        return L.vref_coordination(path.encode(), _d(b), (coord_vtk or "").encode(), (world_vtk or "").encode())


class RefWorld(_World):
    """The reference's own SimMediator loop (see ref_harness.cpp).  The reference keeps global
    state (the aries::Constants singleton) and writes files into the working directory, so each
    instance runs in a temporary directory and instances should not be interleaved with
    different safety factors."""
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(REF_LIB):
                if build_ref() is None:
                    raise RuntimeError("reference sources not available; RefWorld cannot be built")
            L = C.CDLL(REF_LIB)
            L.vref_open.restype = C.c_void_p
            L.vref_open.argtypes = [C.c_char_p, C.c_char_p, C.c_uint, C.c_uint, C.c_char_p]
            L.vref_run.argtypes = [C.c_void_p, C.c_uint]
            L.vref_num_do.argtypes = [C.c_void_p]
            L.vref_num_do.restype = C.c_uint
            L.vref_get_state.argtypes = [C.c_void_p] + [_dp] * 7
            L.vref_num_candidates.argtypes = [C.c_void_p]
            L.vref_num_candidates.restype = C.c_uint
            L.vref_get_candidates.argtypes = [C.c_void_p, _up, _up]
            L.vref_num_interactions.argtypes = [C.c_void_p]
            L.vref_num_interactions.restype = C.c_uint
            L.vref_get_interactions.argtypes = [C.c_void_p, _up, _up, _ip, _dp, _dp, _dp, _dp, _ip]
            L.vref_time.argtypes = [C.c_void_p]
            L.vref_time.restype = C.c_double
            L.vref_energy.argtypes = [C.c_void_p, _dp]
            L.vref_write_ido.argtypes = [C.c_void_p, C.c_char_p]
            L.vref_write_xml.argtypes = [C.c_void_p, C.c_char_p]
            L.vref_close.argtypes = [C.c_void_p]
            L.vref_coordination.argtypes = [C.c_char_p, _dp, C.c_char_p, C.c_char_p]
            L.vref_coordination.restype = C.c_double
            cls._lib = L
        return cls._lib

    def __init__(self, scene, up_iact: int = 1, consultant: str = "nbs", record: int = 1 << 30):
        L = self.lib()
        self.tmp = tempfile.TemporaryDirectory(prefix="vref_")
        path = os.path.join(self.tmp.name, "scene.ido")
        scene.to_ido(path)
        cwd = os.getcwd()
        try:
            self.h = L.vref_open(path.encode(), consultant.encode(), record, up_iact, self.tmp.name.encode())
        finally:
            os.chdir(cwd)
        if not self.h:
            raise ValueError("reference could not read the scene")

    def _num_objects(self) -> int:
        return self.lib().vref_num_do(self.h)

    def run(self, nsteps: int) -> int:
        cwd = os.getcwd()
        os.chdir(self.tmp.name)
        try:
            return self.lib().vref_run(self.h, nsteps)
        finally:
            os.chdir(cwd)

    def _get_state(self, *ptrs):
        self.lib().vref_get_state(self.h, *ptrs)

    def candidates(self):
        m = self.lib().vref_num_candidates(self.h)
        a = np.zeros(m, np.uint32)
        b = np.zeros(m, np.uint32)
        self.lib().vref_get_candidates(self.h, a.ctypes.data_as(_up), b.ctypes.data_as(_up))
        return a, b

    def interactions(self):
        m = self.lib().vref_num_interactions(self.h)
        out = dict(slave=np.zeros(m, np.uint32), master=np.zeros(m, np.uint32), active=np.zeros(m, np.int32),
                   depth=np.zeros(m), normal=np.zeros((m, 3)), shear=np.zeros((m, 3)), kn=np.zeros(m),
                   contact=np.zeros(m, np.int32))
        self.lib().vref_get_interactions(self.h, out["slave"].ctypes.data_as(_up),
                                         out["master"].ctypes.data_as(_up), out["active"].ctypes.data_as(_ip),
                                         _d(out["depth"]), _d(out["normal"]), _d(out["shear"]), _d(out["kn"]),
                                         out["contact"].ctypes.data_as(_ip))
        return out

    def time(self) -> float:
        return self.lib().vref_time(self.h)

    def energy(self) -> np.ndarray:
        e = np.zeros(9)
        self.lib().vref_energy(self.h, _d(e))
        return e

    def write_ido(self, path: str):
        self.lib().vref_write_ido(self.h, path.encode())

    def write_xml(self, path: str):
        """The reference's own DOWorld::WriteXML (6 significant digits, as it writes them)."""
        self.lib().vref_write_xml(self.h, path.encode())

    def close(self):
        if getattr(self, "h", None):
            cwd = os.getcwd()
            try:
                self.lib().vref_close(self.h)
            finally:
                os.chdir(cwd)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
