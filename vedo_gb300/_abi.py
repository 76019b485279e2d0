"""ctypes mirror of include/vedo_gpu.h and the Scene -> ``vedo_scene_desc`` conversion."""
from __future__ import annotations

import ctypes as C
from typing import List, Tuple

import numpy as np

from .scene import Scene

c_double_p = C.POINTER(C.c_double)
c_uint32_p = C.POINTER(C.c_uint32)
c_uint8_p = C.POINTER(C.c_uint8)

VEDO_OK = 0
STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARGUMENT", 2: "INVALID_SCENE", 3: "UNSUPPORTED_MODEL", 4: "OUT_OF_MEMORY",
    5: "CUDA_ERROR", 6: "DEVICE_TIMEOUT", 7: "BAD_IDO", 8: "IO_ERROR",
}
PRECISION_FP64 = 0
PRECISION_MIXED = 1


class DOModelDesc(C.Structure):
    _fields_ = [("name", C.c_char_p), ("group", C.c_char_p), ("behavior", C.c_uint32), ("scope", C.c_uint32),
                ("shape", C.c_uint32), ("reserved", C.c_uint32), ("density", C.c_double),
                ("density_factor", C.c_double), ("external_force", C.c_double * 3), ("attrs", C.c_double * 10)]


class IactModelDesc(C.Structure):
    _fields_ = [("master_group", C.c_char_p), ("slave_group", C.c_char_p), ("equation_type", C.c_char_p),
                ("num_mechanisms", C.c_uint32), ("mechanism_names", C.POINTER(C.c_char_p)),
                ("mechanism_values", c_double_p)]


class SceneDesc(C.Structure):
    _fields_ = [("time_start", C.c_double), ("time_stop", C.c_double), ("time_interval", C.c_double),
                ("time_current", C.c_double), ("field_acceleration", C.c_double * 3),
                ("safety_factor", C.c_double), ("zoi_switch", C.c_uint8 * 3), ("pbc_switch", C.c_uint8 * 3),
                ("reserved", C.c_uint8 * 2), ("zoi_lower", C.c_double * 3), ("zoi_upper", C.c_double * 3),
                ("pbc_lower", C.c_double * 3), ("pbc_upper", C.c_double * 3), ("max_id_of_do", C.c_uint32),
                ("num_models", C.c_uint32), ("models", C.POINTER(DOModelDesc)),
                ("num_iact_models", C.c_uint32), ("iact_models", C.POINTER(IactModelDesc)),
                ("num_objects", C.c_uint32), ("object_model", c_uint32_p), ("object_id", c_uint32_p),
                ("position", c_double_p), ("velocity", c_double_p), ("orientation_x", c_double_p),
                ("orientation_z", c_double_p), ("angular_velocity", c_double_p), ("impact", c_double_p),
                ("angular_impact", c_double_p),
                ("num_records", C.c_uint32), ("record_first", c_uint32_p), ("record_second", c_uint32_p),
                ("record_contact", c_uint8_p), ("record_bond", c_uint8_p), ("record_kn", c_double_p),
                ("record_initial_velocity", c_double_p), ("record_shear", c_double_p)]


class EngineOpts(C.Structure):
    _fields_ = [("up_iact", C.c_uint32), ("record", C.c_uint32), ("precision", C.c_uint32), ("device", C.c_int32),
                ("output_prefix", C.c_char_p), ("skin", C.c_float), ("check_interval", C.c_uint32),
                ("tick_block", C.c_uint32), ("cell_scale", C.c_float), ("autotune", C.c_uint32),
                ("graphs", C.c_uint32), ("stored_splits", C.c_uint32), ("split_tick", C.c_uint32),
                ("full_walks", C.c_uint32), ("consultant", C.c_uint32), ("orientations", C.c_uint32),
                ("persistent", C.c_uint32)]


class StateView(C.Structure):
    _fields_ = [("position", c_double_p), ("velocity", c_double_p), ("angular_velocity", c_double_p),
                ("orientation_x", c_double_p), ("orientation_z", c_double_p), ("impact", c_double_p),
                ("angular_impact", c_double_p)]


class ContactView(C.Structure):
    _fields_ = [("first", c_uint32_p), ("second", c_uint32_p), ("slave", c_uint32_p), ("master", c_uint32_p),
                ("active", c_uint8_p), ("shear", c_double_p), ("kn", c_double_p), ("contact", c_uint8_p)]


def dptr(a: np.ndarray):
    return None if a is None else a.ctypes.data_as(c_double_p)


def uptr(a: np.ndarray):
    return None if a is None else a.ctypes.data_as(c_uint32_p)


def bptr(a: np.ndarray):
    return None if a is None else a.ctypes.data_as(c_uint8_p)


def scene_to_desc(scene: Scene) -> Tuple[SceneDesc, List[object]]:
    """Flatten a Scene into the C descriptor.  The returned list keeps every buffer alive."""
    keep: List[object] = []
    sp = scene.sp
    d = SceneDesc()
    d.time_start, d.time_stop, d.time_interval, d.time_current = sp.time_start, sp.time_stop, sp.time_interval, \
        sp.time_current
    d.field_acceleration[:] = list(sp.field_acceleration)
    d.safety_factor = sp.safety_factor
    d.zoi_switch[:] = [int(b) for b in sp.zoi.switch]
    d.pbc_switch[:] = [int(b) for b in sp.pbc.switch]
    d.zoi_lower[:], d.zoi_upper[:] = list(sp.zoi.lower), list(sp.zoi.upper)
    d.pbc_lower[:], d.pbc_upper[:] = list(sp.pbc.lower), list(sp.pbc.upper)
    d.max_id_of_do = sp.max_id_of_do
    models = (DOModelDesc * max(1, len(scene.models)))()
    for k, m in enumerate(scene.models):
        nm, gr = m.name.encode(), m.group.encode()
        keep += [nm, gr]
        models[k].name, models[k].group = nm, gr
        models[k].behavior, models[k].scope, models[k].shape = m.behavior, m.scope, m.shape
        models[k].density, models[k].density_factor = m.density, m.density_factor
        models[k].external_force[:] = list(m.external_force)
        a = list(m.attrs) + [0.0] * (10 - len(m.attrs))
        models[k].attrs[:] = a[:10]
    keep.append(models)
    d.num_models = len(scene.models)
    d.models = C.cast(models, C.POINTER(DOModelDesc))
    iacts = (IactModelDesc * max(1, len(scene.iact_models)))()
    for k, im in enumerate(scene.iact_models):
        mg, sg, eq = im.master_group.encode(), im.slave_group.encode(), im.equation_type.encode()
        names = (C.c_char_p * max(1, len(im.mechanisms)))(*[n.encode() for n, _ in im.mechanisms])
        vals = np.array([v for _, v in im.mechanisms] or [0.0], dtype=np.float64)
        keep += [mg, sg, eq, names, vals]
        iacts[k].master_group, iacts[k].slave_group, iacts[k].equation_type = mg, sg, eq
        iacts[k].num_mechanisms = len(im.mechanisms)
        iacts[k].mechanism_names = C.cast(names, C.POINTER(C.c_char_p))
        iacts[k].mechanism_values = dptr(vals)
    keep.append(iacts)
    d.num_iact_models = len(scene.iact_models)
    d.iact_models = C.cast(iacts, C.POINTER(IactModelDesc))
    arrays = {}
    for name in ("position", "velocity", "orientation_x", "orientation_z", "angular_velocity", "impact",
                 "angular_impact"):
        a = np.ascontiguousarray(getattr(scene, name), dtype=np.float64)
        arrays[name] = a
        setattr(d, name, dptr(a))
    keep.append(arrays)
    mi = np.ascontiguousarray(scene.model_index, dtype=np.uint32)
    ids = np.ascontiguousarray(scene.ids, dtype=np.uint32)
    keep += [mi, ids]
    d.num_objects = scene.num_objects
    d.object_model, d.object_id = uptr(mi), uptr(ids)
    r = scene.records
    d.num_records = len(r)
    if len(r):
        ra = [np.ascontiguousarray(r.first, np.uint32), np.ascontiguousarray(r.second, np.uint32),
              np.ascontiguousarray(r.contact, np.uint8), np.ascontiguousarray(r.bond, np.uint8),
              np.ascontiguousarray(r.kn, np.float64), np.ascontiguousarray(r.initial_velocity, np.float64),
              np.ascontiguousarray(r.shear, np.float64)]
        keep.append(ra)
        d.record_first, d.record_second = uptr(ra[0]), uptr(ra[1])
        d.record_contact, d.record_bond = bptr(ra[2]), bptr(ra[3])
        d.record_kn, d.record_initial_velocity, d.record_shear = dptr(ra[4]), dptr(ra[5]), dptr(ra[6])
    return d, keep
