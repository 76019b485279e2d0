"""CPU tests of the post-processing observables against the reference's own outputs
(tests/golden/observables: CalcCoordinateNum and DOWorld::WriteVTK compiled from the reference):
the oracle's coordination numbers, and the engine library's VTK writer through the scene
conversion, which needs no GPU."""
import glob
import os
import re

import numpy as np
import pytest

from vedo_gb300.scene import Scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "observables", "*.npz")))


def _name(p):
    return os.path.splitext(os.path.basename(p))[0]


def vtk_array(text: str, name: str) -> np.ndarray:
    """The numbers of the DataArray called `name` in a VTK text."""
    i = text.index(f'Name="{name}"')
    body = text[text.index(">", i) + 1:text.index("</DataArray>", i)]
    return np.array([float(x) for x in body.split()])


def mask_granular(text: str) -> str:
    """The reference's statuses read from an IDO file leave the granular temperatures unset
    (DOStatus.cpp:64-67), so their two arrays hold whatever that memory held: blank them."""
    for name in ("GranularTemperatureV", "GranularTemperatureAV"):
        i = text.index(f'Name="{name}"')
        a, b = text.index(">", i) + 1, text.index("</DataArray>", i)
        text = text[:a] + re.sub(r"[^\s]+", "*", text[a:b]) + text[b:]
    return text


@pytest.mark.parametrize("path", FIXTURES, ids=[_name(p) for p in FIXTURES])
def test_oracle_coordination_matches_reference(path, port_lib):
    from oracle import PortWorld
    g = np.load(path)
    sc = Scene.from_ido(g["ido"].tobytes())
    below, touching, avg = PortWorld(sc).coordination(g["box"])
    assert avg == float(g["average"])
    ref = vtk_array(g["coord_vtk"].tobytes().decode(), "CoordinateNumber")
    spheres = np.array([sc.models[m].shape == 1 for m in sc.model_index])
    np.testing.assert_array_equal(below[spheres].astype(float), ref)
    assert np.all(below[~spheres] == 0) and np.all(touching >= below)
    assert np.any(touching > below)          # exact ties: counted by the inclusive test only


@pytest.mark.parametrize("path", FIXTURES, ids=[_name(p) for p in FIXTURES])
def test_vtu_conversion_matches_reference_writer(path, engine_lib, tmp_path):
    g = np.load(path)
    ido = tmp_path / "s.ido"
    ido.write_bytes(g["ido"].tobytes())
    out = tmp_path / "s.vtu"
    engine_lib.convert_scene(str(ido), str(out))
    ours = out.read_text()
    ref = g["world_vtk"].tobytes().decode()
    assert mask_granular(ours) == mask_granular(ref)
    assert np.all(vtk_array(ours, "GranularTemperatureV") == 0.0)


def test_vtu_from_xml_equals_vtu_from_ido(engine_lib, tmp_path):
    """A scene read from DOWorldSchema XML writes the same VTK file as the same scene read from its
    IDO file (the conversion runs on the host)."""
    g = np.load(FIXTURES[0])
    ido = tmp_path / "s.ido"
    ido.write_bytes(g["ido"].tobytes())
    xml = tmp_path / "s.xml"
    engine_lib.convert_scene(str(ido), str(xml))
    a, b = tmp_path / "a.vtu", tmp_path / "b.vtu"
    engine_lib.convert_scene(str(ido), str(a))
    engine_lib.convert_scene(str(xml), str(b))
    assert a.read_text() == b.read_text()
