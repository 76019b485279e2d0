"""Scene model of a VEDO DEM world and its binary ``.ido`` format.

A :class:`Scene` holds what ``vedo::DOWorld`` holds (src/vedo/framework/DOWorld.h):
the ``SystemParameter`` (time control, field acceleration, zone of interest,
periodic boundary), the ``DOModel`` list (shape, material, behaviour, scope),
the ``IactModel`` list (group pair -> equation type + named mechanism values),
the per-object ``DOStatus`` (SoA arrays here) and the ``IactRecordTab`` shear
history records.

``to_ido``/``from_ido`` are byte-compatible with the reference writer and
reader (DOWorld_RWIDO.cpp:9-202, SystemParameter.cpp:61-140,
DOModel.cpp:267-347, IactModel.cpp:102-137, DOStatus.cpp:176-200,
IactRecordTab.cpp:346-530) for the reference's ``-D_INT32 -D_FLOAT64
-D_STD_CPP_11`` build: every unsigned is 4 bytes, every float 8 bytes, bool 1
byte, little endian, strings are a uint32 length followed by the bytes.

Large scenes are written with vectorised numpy records: all DOStatus entries
whose model names have the same length form fixed-size records.
"""
from __future__ import annotations

import io
import math
import struct
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

# enum DOShapeType : _uint_t (DOModel.h:25, C++11 build)
NO_SHAPE, SPHERE, DMSPHERE, ELLIPSOID, POLYHEDRA, POLYHEDRA_BREP, QUASI_CYLINDER, QUASI_PLATE, \
    QUASI_PLATE_WITH_CIRCULAR_HOLE, TRIANGLE = range(10)
# No counterpart in the reference: the inside of a hollow cylinder (a drum shell), attrs
# (radius, length) about OrientationZ, global scope, fixed or orbital.  An engine extension;
# scenes that use it cannot be read by the reference.
INNER_CYLINDER = 32
# enum DOBehaviorType : _uint_t (DOModel.h:26)
NO_BEHAVIOR, CONSTRAINED, FIXED, MOBILE, ORBITAL = range(5)
# enum DOScopeType : _uint_t (DOModel.h:27)
NO_SCOPE, GLOBAL, LOCAL = range(3)

RELEASE_DATE = "2016-09-23"          # aries::information::_ReleaseDate (Constants.h:42)
SHAPE_ATTR_DOUBLES = 10              # sizeof(DOShapeAttributes) / 8: the triangle member is largest

PI = 4.0 * math.atan(1.0)            # aries::math::_PI (Constants.h:22)
FOURTH_THIRDS_PI = 4.0 / 3.0 * PI    # aries::math::_FourthThirdsPI (Constants.h:32)


@dataclass
class Boundary:
    """``vedo::Boundary`` as stored in an IDO file: three axis switches and a box."""
    switch: Tuple[bool, bool, bool] = (False, False, False)
    lower: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    upper: Tuple[float, float, float] = (0.0, 0.0, 0.0)

    @property
    def active(self) -> bool:
        return any(self.switch)


@dataclass
class SystemParameter:
    time_start: float = 0.0
    time_stop: float = 0.0
    time_interval: float = 1e-6
    time_current: float = 0.0
    field_acceleration: Tuple[float, float, float] = (0.0, 0.0, -9.81)
    zoi: Boundary = field(default_factory=Boundary)
    pbc: Boundary = field(default_factory=Boundary)
    safety_factor: float = 1.1          # aries::Constants SafetyFactor (Constants.h:184)
    num_udd_do: int = 0
    num_udd_impact: int = 0
    max_id_of_do: int = 0


@dataclass
class DOModel:
    name: str
    group: str
    behavior: int
    scope: int
    density: float
    density_factor: float
    shape: int
    attrs: Tuple[float, ...]            # shape attributes in union order, e.g. (radius,) for a sphere
    external_force: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    color: int = 0
    materials: List[Tuple[str, float]] = field(default_factory=list)

    def analysis(self):
        """Mass, SudoMass, inertia and range exactly as DOModel::Analysis (DOModel.cpp:17-149).

        Returns (range, volume, mass, sudo_mass, (Ix, Iy, Iz)).
        """
        a = list(self.attrs) + [0.0] * (SHAPE_ATTR_DOUBLES - len(self.attrs))
        if self.shape == SPHERE:
            r = a[0]
            rng = r
            vol = FOURTH_THIRDS_PI * r * r * r
            m = self.density * vol
            sm = self.density_factor * m
            mmi = 0.4 * m * r * r
            return rng, vol, m, sm, (mmi, mmi, mmi)
        if self.shape == QUASI_CYLINDER:
            r, h = a[0], a[1]
            rng = max(r, 0.5 * h) if self.scope == LOCAL else r
            vol = PI * r * r * h
            m = self.density * vol
            sm = self.density_factor * m
            mmi = m * (3.0 * r * r + h * h) / 12.0
            return rng, vol, m, sm, (mmi, mmi, 0.5 * m * r * r)
        if self.shape == INNER_CYLINDER:
            if self.scope != GLOBAL:
                raise ValueError(f"model {self.name!r}: an inner cylinder must have global scope")
            return 0.0, 0.0, 0.0, 0.0, (0.0, 0.0, 0.0)
        if self.shape == QUASI_PLATE:
            w, h, l = a[0], a[1], a[2]
            rng = 0.5 * max(max(w, h), l) if self.scope == LOCAL else 0.5 * h
            vol = w * h * l
            m = self.density * vol
            sm = self.density_factor * m
            k = m / 12.0
            return rng, vol, m, sm, (k * (h * h + l * l), k * (w * w + l * l), k * (h * h + w * w))
        if self.shape == QUASI_PLATE_WITH_CIRCULAR_HOLE:
            w, h, l, hr, hxo, hyo = a[0], a[1], a[2], a[3], a[4], a[5]
            rng = 0.5 * max(max(w, h), l) if self.scope == LOCAL else 0.5 * h
            if not (abs(hxo) <= 0.5 * w - hr and abs(hyo) <= 0.5 * l - hr):
                raise ValueError(f"model {self.name!r}: the hole does not lie inside the plate")
            vol = w * h * l - hr * hr * PI * h
            m = self.density * vol
            return rng, vol, m, self.density_factor * m, (0.0, 0.0, 0.0)
        raise ValueError(f"shape type {self.shape} of model {self.name!r} is not supported")


@dataclass
class IactModel:
    master_group: str
    slave_group: str
    equation_type: str
    mechanisms: List[Tuple[str, float]]

    def get(self, name: str) -> float:
        for n, v in self.mechanisms:
            if n == name:
                return v
        raise KeyError(f"IactModel {self.master_group}/{self.slave_group} has no mechanism {name!r}")


@dataclass
class Records:
    """IactRecordTab entries, keyed (first, second) with first < second by construction."""
    first: np.ndarray
    second: np.ndarray
    contact: np.ndarray
    bond: np.ndarray
    kn: np.ndarray
    initial_velocity: np.ndarray
    shear: np.ndarray          # [n,3]
    impact_point: np.ndarray   # [n,3]
    impact_direction: np.ndarray
    impact_to_master: np.ndarray
    angular_impact_to_master: np.ndarray
    overlap: np.ndarray

    @staticmethod
    def empty() -> "Records":
        z1 = np.zeros(0)
        z3 = np.zeros((0, 3))
        zu = np.zeros(0, dtype=np.uint32)
        zb = np.zeros(0, dtype=np.bool_)
        return Records(zu, zu.copy(), zb, zb.copy(), z1, z1.copy(), z3, z3.copy(), z3.copy(), z3.copy(),
                       z3.copy(), z1.copy())

    def __len__(self) -> int:
        return int(self.first.shape[0])


class Scene:
    """In-memory ``DOWorld`` + ``IactRecordTab``.  Object state is SoA float64 [n,3]."""

    def __init__(self, sp: SystemParameter, models: Sequence[DOModel], iact_models: Sequence[IactModel],
                 model_index: np.ndarray, position: np.ndarray, velocity: Optional[np.ndarray] = None,
                 orientation_x: Optional[np.ndarray] = None, orientation_z: Optional[np.ndarray] = None,
                 angular_velocity: Optional[np.ndarray] = None, impact: Optional[np.ndarray] = None,
                 angular_impact: Optional[np.ndarray] = None, ids: Optional[np.ndarray] = None,
                 records: Optional[Records] = None):
        self.sp = sp
        self.models = list(models)
        self.iact_models = list(iact_models)
        n = int(position.shape[0])
        self.model_index = np.ascontiguousarray(model_index, dtype=np.uint32)

        def v3(a, default=None):
            if a is None:
                a = np.zeros((n, 3)) if default is None else np.tile(np.asarray(default, dtype=np.float64), (n, 1))
            return np.ascontiguousarray(a, dtype=np.float64).reshape(n, 3)

        self.position = v3(position)
        self.velocity = v3(velocity)
        self.orientation_x = v3(orientation_x, (1.0, 0.0, 0.0))
        self.orientation_z = v3(orientation_z, (0.0, 0.0, 1.0))
        self.angular_velocity = v3(angular_velocity)
        self.impact = v3(impact)
        self.angular_impact = v3(angular_impact)
        self.ids = np.zeros(n, dtype=np.uint32) if ids is None else np.ascontiguousarray(ids, dtype=np.uint32)
        self.records = Records.empty() if records is None else records

    @property
    def num_objects(self) -> int:
        return int(self.position.shape[0])

    def model_of(self, i: int) -> DOModel:
        return self.models[int(self.model_index[i])]

    def iact_model(self, group_a: str, group_b: str) -> Optional[int]:
        """First IactModel matching the unordered group pair, as DOWorld::GetIactModel
        (DOWorld.cpp:297-302 with IactModel::operator(), IactModel.cpp:16-30)."""
        for k, im in enumerate(self.iact_models):
            if (im.master_group == group_a and im.slave_group == group_b) or \
               (im.master_group == group_b and im.slave_group == group_a):
                return k
        return None

    def copy(self) -> "Scene":
        import copy as _copy
        return _copy.deepcopy(self)

    # ------------------------------------------------------------------ IDO
    def to_ido(self, path: Optional[str] = None) -> bytes:
        out = io.BytesIO()
        w = out.write

        def wstr(s: str):
            b = s.encode("latin-1")
            w(struct.pack("<I", len(b)))
            w(b)

        sp = self.sp
        wstr(RELEASE_DATE)
        w(struct.pack("<IIII", 3, sp.num_udd_do, sp.num_udd_impact, sp.max_id_of_do))
        w(struct.pack("<Id", 1, sp.safety_factor))
        w(struct.pack("<4d", sp.time_start, sp.time_stop, sp.time_current, sp.time_interval))
        w(struct.pack("<3d", *sp.field_acceleration))
        for b in (sp.zoi, sp.pbc):
            w(struct.pack("<3?", *b.switch))
            w(struct.pack("<3d", *b.lower))
            w(struct.pack("<3d", *b.upper))
        w(struct.pack("<I", len(self.models)))
        for m in self.models:
            wstr(m.name)
            wstr(m.group)
            w(struct.pack("<II", m.behavior, m.scope))
            w(struct.pack("<2d", m.density, m.density_factor))
            w(struct.pack("<3d", *m.external_force))
            w(struct.pack("<II", m.color, m.shape))
            attrs = list(m.attrs) + [0.0] * (SHAPE_ATTR_DOUBLES - len(m.attrs))
            w(struct.pack(f"<{SHAPE_ATTR_DOUBLES}d", *attrs))
            w(struct.pack("<I", len(m.materials)))
            for name, val in m.materials:
                wstr(name)
                w(struct.pack("<d", val))
            if m.shape == POLYHEDRA:
                raise ValueError("polyhedra models are not supported")
        w(struct.pack("<I", len(self.iact_models)))
        for im in self.iact_models:
            wstr(im.master_group)
            wstr(im.slave_group)
            wstr(im.equation_type)
            w(struct.pack("<I", len(im.mechanisms)))
            for name, val in im.mechanisms:
                wstr(name)
                w(struct.pack("<d", val))
        n = self.num_objects
        w(struct.pack("<I", n))
        w(self._status_bytes())
        rec = self.records
        w(struct.pack("<I", len(rec)))
        if len(rec):
            if sp.num_udd_impact:
                raise ValueError("user-defined impact values are not supported")
            dt = np.dtype([("a", "<u4"), ("b", "<u4"), ("c", "?"), ("d", "?"), ("kn", "<f8"), ("v0", "<f8"),
                           ("s", "<f8", 3), ("p", "<f8", 3), ("n", "<f8", 3), ("i", "<f8", 3), ("ai", "<f8", 3),
                           ("o", "<f8")])
            arr = np.zeros(len(rec), dtype=dt)
            arr["a"], arr["b"], arr["c"], arr["d"] = rec.first, rec.second, rec.contact, rec.bond
            arr["kn"], arr["v0"] = rec.kn, rec.initial_velocity
            arr["s"], arr["p"], arr["n"] = rec.shear, rec.impact_point, rec.impact_direction
            arr["i"], arr["ai"], arr["o"] = rec.impact_to_master, rec.angular_impact_to_master, rec.overlap
            w(arr.tobytes())
        data = out.getvalue()
        if path is not None:
            with open(path, "wb") as f:
                f.write(data)
        return data

    def _status_bytes(self) -> bytes:
        n = self.num_objects
        names = [m.name.encode("latin-1") for m in self.models]
        lens = np.array([len(b) for b in names], dtype=np.int64)[self.model_index] if n else np.zeros(0, np.int64)
        parts = []
        # Objects are written in order; consecutive runs of equal name length become one record block.
        start = 0
        while start < n:
            L = int(lens[start])
            stop = start
            # extend the run while the name length stays equal
            idx = np.nonzero(lens[start:] != L)[0]
            stop = n if idx.size == 0 else start + int(idx[0])
            dt = np.dtype([("len", "<u4"), ("name", f"S{L}" if L else "V0"), ("id", "<u4"), ("v", "<f8", 21)])
            arr = np.zeros(stop - start, dtype=dt)
            arr["len"] = L
            if L:
                name_table = np.array([b if len(b) == L else b"" for b in names], dtype=f"S{L}")
                arr["name"] = name_table[self.model_index[start:stop]]
            arr["id"] = self.ids[start:stop]
            v = np.concatenate([self.position[start:stop], self.velocity[start:stop],
                                self.orientation_x[start:stop], self.orientation_z[start:stop],
                                self.angular_velocity[start:stop], self.impact[start:stop],
                                self.angular_impact[start:stop]], axis=1)
            arr["v"] = v
            parts.append(arr.tobytes())
            start = stop
        return b"".join(parts)

    @staticmethod
    def from_ido(path_or_bytes) -> "Scene":
        if isinstance(path_or_bytes, (bytes, bytearray)):
            data = bytes(path_or_bytes)
        else:
            with open(path_or_bytes, "rb") as f:
                data = f.read()
        r = _Reader(data)
        r.string()  # release date
        nu = r.u32()
        if nu != 3:
            raise ValueError("IDO: size of integer data is wrong")
        sp = SystemParameter()
        sp.num_udd_do, sp.num_udd_impact, sp.max_id_of_do = r.u32(), r.u32(), r.u32()
        nf = r.u32()
        if nf != 1:
            raise ValueError("IDO: size of float data is wrong")
        sp.safety_factor = r.f64()
        sp.time_start, sp.time_stop, sp.time_current, sp.time_interval = (r.f64() for _ in range(4))
        sp.field_acceleration = tuple(r.f64() for _ in range(3))
        bounds = []
        for _ in range(2):
            sw = tuple(bool(b) for b in r.raw(3))
            lo = tuple(r.f64() for _ in range(3))
            hi = tuple(r.f64() for _ in range(3))
            bounds.append(Boundary(sw, lo, hi))
        sp.zoi, sp.pbc = bounds
        models = []
        for _ in range(r.u32()):
            name, group = r.string(), r.string()
            beh, scope = r.u32(), r.u32()
            dens, dfac = r.f64(), r.f64()
            ext = tuple(r.f64() for _ in range(3))
            color, shape = r.u32(), r.u32()
            attrs = tuple(r.f64() for _ in range(SHAPE_ATTR_DOUBLES))
            mats = [(r.string(), r.f64()) for _ in range(r.u32())]
            if shape == POLYHEDRA:
                raise ValueError("polyhedra models are not supported")
            models.append(DOModel(name, group, beh, scope, dens, dfac, shape, attrs, ext, color, mats))
        iacts = []
        for _ in range(r.u32()):
            mg, sg, eq = r.string(), r.string(), r.string()
            mechs = [(r.string(), r.f64()) for _ in range(r.u32())]
            iacts.append(IactModel(mg, sg, eq, mechs))
        n = r.u32()
        name_to_model = {}
        for k, m in enumerate(models):
            name_to_model.setdefault(m.name, k)
        midx = np.zeros(n, dtype=np.uint32)
        ids = np.zeros(n, dtype=np.uint32)
        vals = np.zeros((n, 21))
        for i in range(n):
            nm = r.string()
            if nm not in name_to_model:
                raise ValueError(f"IDO: unknown model of discrete object {nm!r}")
            midx[i] = name_to_model[nm]
            ids[i] = r.u32()
            vals[i] = np.frombuffer(r.raw(168), dtype="<f8")
        nrec = r.u32()
        if nrec and sp.num_udd_impact:
            raise ValueError("user-defined impact values are not supported")
        dt = np.dtype([("a", "<u4"), ("b", "<u4"), ("c", "?"), ("d", "?"), ("kn", "<f8"), ("v0", "<f8"),
                       ("s", "<f8", 3), ("p", "<f8", 3), ("n", "<f8", 3), ("i", "<f8", 3), ("ai", "<f8", 3),
                       ("o", "<f8")])
        arr = np.frombuffer(r.raw(nrec * dt.itemsize), dtype=dt) if nrec else np.zeros(0, dtype=dt)
        rec = Records(arr["a"].copy(), arr["b"].copy(), arr["c"].copy(), arr["d"].copy(), arr["kn"].copy(),
                      arr["v0"].copy(), arr["s"].copy(), arr["p"].copy(), arr["n"].copy(), arr["i"].copy(),
                      arr["ai"].copy(), arr["o"].copy())
        v = vals
        return Scene(sp, models, iacts, midx, v[:, 0:3], v[:, 3:6], v[:, 6:9], v[:, 9:12], v[:, 12:15],
                     v[:, 15:18], v[:, 18:21], ids=ids, records=rec)


class _Reader:
    def __init__(self, data: bytes):
        self.d = data
        self.p = 0

    def raw(self, k: int) -> bytes:
        if self.p + k > len(self.d):
            raise ValueError("IDO: truncated file")
        b = self.d[self.p:self.p + k]
        self.p += k
        return b

    def u32(self) -> int:
        return struct.unpack("<I", self.raw(4))[0]

    def f64(self) -> float:
        return struct.unpack("<d", self.raw(8))[0]

    def string(self) -> str:
        return self.raw(self.u32()).decode("latin-1")
