"""DOWorldSchema XML scenes (CPU): the engine's reader against XML written by the reference's
own DOWorld::WriteXML, and a lossless .ido -> .xml -> .ido round trip of the engine's writer."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from vedo_gb300 import scenes
from vedo_gb300.scene import Scene


def _vec(node):
    return [float(node.get(k)) for k in ("x", "y", "z")]


def test_reader_maps_the_reference_writers_xml(engine_lib, tmp_path):
    import oracle
    if not os.path.exists(oracle.REF_LIB):
        pytest.skip("the reference CPU build is not present on this host")
    from oracle import RefWorld
    sc = scenes.cluster(n=40, solver="ISwBSDBF", seed=8, steps=500, polydisperse=True, cylinders=2)
    w = RefWorld(sc, up_iact=5)
    w.run(120)                                   # contacts and shear history in the record table
    xml = str(tmp_path / "ref.xml")
    w.write_xml(xml)
    w.close()
    ido = str(tmp_path / "from_xml.ido")
    engine_lib.convert_scene(xml, ido)
    got = Scene.from_ido(ido)
    # the expected values: the same file read with Python's own XML parser, mapped as
    # DOWorld_ReadXML.cpp maps it
    root = ET.parse(xml).getroot()
    tc = root.find("SimParameter/TimeControl")
    assert got.sp.time_current == float(tc.get("Current")) and got.sp.time_stop == float(tc.get("Stop"))
    assert list(got.sp.field_acceleration) == _vec(root.find("SimParameter/FieldAcceleration"))
    models = root.findall("DOModelTab/DOModel")
    assert [m.name for m in got.models] == [m.get("DOName") for m in models]
    for gm, xm in zip(got.models, models):
        assert gm.group == xm.get("DOGroup") and gm.density == float(xm.get("Density"))
        shape = xm.find("Shape")[0]
        if shape.tag == "Sphere":
            assert gm.attrs[0] == float(shape.get("Radius"))
        elif shape.tag == "QuasiPlate":
            assert list(gm.attrs[:3]) == [float(shape.get(k)) for k in ("Width", "Height", "Length")]
        elif shape.tag == "QuasiCylinder":
            assert list(gm.attrs[:2]) == [float(shape.get(k)) for k in ("Radius", "Height")]
    iacts = root.findall("IactModelTab/IactModel")
    assert [(im.equation_type, [v for _, v in im.mechanisms]) for im in got.iact_models] == \
        [(x.get("EquationType"), [float(c.get("Value")) for c in x]) for x in iacts]
    st = root.findall("DOStatusTab/DOStatus")
    assert got.num_objects == len(st)
    for k, tag in (("position", "Position"), ("velocity", "Velocity"), ("orientation_z", "OrientationZ"),
                   ("angular_velocity", "AngularVelocity")):
        assert np.array_equal(getattr(got, k), np.array([_vec(d.find(tag)) for d in st])), k
    rec = root.findall("IactStatusTab/IactStatus")
    assert len(got.records) == len(rec) > 0
    assert list(got.records.first) == [int(r.get("MasterDOStatusSN")) for r in rec]
    assert np.array_equal(got.records.shear, np.array([_vec(r.find("ShearForce")) for r in rec]))


def test_xml_round_trip_is_lossless(engine_lib, tmp_path):
    sc = scenes.cluster(n=30, solver="ISwH", seed=2, orbital=True, cylinders=3)
    a = str(tmp_path / "a.ido")
    sc.to_ido(a)
    x = str(tmp_path / "a.xml")
    b = str(tmp_path / "b.ido")
    engine_lib.convert_scene(a, x)
    engine_lib.convert_scene(x, b)
    s1, s2 = Scene.from_ido(a), Scene.from_ido(b)
    for k in ("position", "velocity", "orientation_x", "orientation_z", "angular_velocity", "impact",
              "angular_impact"):
        assert np.array_equal(getattr(s1, k), getattr(s2, k)), k
    assert [(m.name, m.group, m.behavior, m.scope, m.shape, list(m.attrs)) for m in s1.models] == \
        [(m.name, m.group, m.behavior, m.scope, m.shape, list(m.attrs)) for m in s2.models]
    assert [(i.master_group, i.slave_group, i.equation_type, i.mechanisms) for i in s1.iact_models] == \
        [(i.master_group, i.slave_group, i.equation_type, i.mechanisms) for i in s2.iact_models]
    assert s1.sp.time_stop == s2.sp.time_stop and s1.sp.safety_factor == s2.sp.safety_factor


def test_xml_errors_are_reported(engine_lib, tmp_path):
    bad = tmp_path / "bad.xml"
    bad.write_text("<DOWorld><SimParameter><TimeControl Start='0'/></SimParameter></DOWorld>")
    with pytest.raises(engine_lib.EngineError) as ex:
        engine_lib.convert_scene(str(bad), str(tmp_path / "x.ido"))
    assert ex.value.code == 2
    bad.write_text("<DOWorld><SimParameter>")
    with pytest.raises(engine_lib.EngineError):
        engine_lib.convert_scene(str(bad), str(tmp_path / "x.ido"))
