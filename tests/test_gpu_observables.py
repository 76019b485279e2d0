"""GPU tests of the coordination-number and VTK observables: the device cell-grid count
against the reference's fixtures (exact ties included) and against the oracle's all-pairs count
on larger states, in both forms; the engine's VTK files against the reference's."""
import glob
import os

import numpy as np
import pytest

from vedo_gb300 import scenes
from vedo_gb300.scene import Scene

from test_observables import mask_granular, vtk_array

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "observables", "*.npz")))


def _name(p):
    return os.path.splitext(os.path.basename(p))[0]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("path", FIXTURES, ids=[_name(p) for p in FIXTURES])
def test_device_coordination_matches_reference(path, precision, engine_lib, port_lib, tmp_path):
    from oracle import PortWorld
    g = np.load(path)
    sc = Scene.from_ido(g["ido"].tobytes())
    e = engine_lib.GpuEngine(sc, precision=precision)
    below, touching, avg = e.coordination(g["box"])
    assert avg == float(g["average"])
    ref = vtk_array(g["coord_vtk"].tobytes().decode(), "CoordinateNumber")
    spheres = np.array([sc.models[m].shape == 1 for m in sc.model_index])
    np.testing.assert_array_equal(below[spheres].astype(float), ref)
    pb, pt, _ = PortWorld(sc).coordination(g["box"])
    np.testing.assert_array_equal(below, pb)
    np.testing.assert_array_equal(touching, pt)
    # the engine's files equal the reference's (granular temperatures aside)
    e.write_vtk(str(tmp_path / "c.vtu"), with_coordination=True)
    e.write_vtk(str(tmp_path / "w.vtu"))
    assert mask_granular((tmp_path / "c.vtu").read_text()) == mask_granular(g["coord_vtk"].tobytes().decode())
    assert mask_granular((tmp_path / "w.vtu").read_text()) == mask_granular(g["world_vtk"].tobytes().decode())
    e.close()


def _scene_at(sc, st):
    out = Scene(sc.sp, sc.models, sc.iact_models, sc.model_index, st["position"], st["velocity"],
                sc.orientation_x, sc.orientation_z, st["angular_velocity"])
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_device_coordination_equals_oracle_on_a_settling_box(precision, engine_lib, port_lib):
    """A 5,832-sphere box after 1,500 steps of colliding (hundreds of overlapping pairs, walls
    present): the device counts equal the oracle's all-pairs counts on the same state, and so does
    a box average."""
    from oracle import PortWorld
    sc = scenes.lsd_box(n_side=18, spacing=2.02e-3, vel_sigma=0.3)
    e = engine_lib.GpuEngine(sc, up_iact=20, precision=precision)
    e.run(1500)
    st = e.state(("position", "velocity", "angular_velocity"))
    box = (-0.01, 0.01, -0.01, 0.01, 0.0, 0.02)
    below, touching, avg = e.coordination(box)
    pb, pt, pavg = PortWorld(_scene_at(sc, st)).coordination(box)
    np.testing.assert_array_equal(below, pb)
    np.testing.assert_array_equal(touching, pt)
    assert avg == pavg
    assert below.sum() > 500                                # hundreds of overlapping pairs
    e.close()


def test_device_coordination_of_a_dense_lattice(engine_lib, port_lib):
    """A 27,000-sphere FCC lattice whose neighbours overlap by a hair: 12 contacts per interior
    sphere, counted exactly (equal to the oracle), at the grid's largest cell occupancy."""
    from oracle import PortWorld
    sc = scenes.dense_pack(n=27000)
    e = engine_lib.GpuEngine(sc, precision=1)
    below, touching, _ = e.coordination()
    pb, pt, _ = PortWorld(sc).coordination((0, 0, 0, 0, 0, 0))
    np.testing.assert_array_equal(below, pb)
    np.testing.assert_array_equal(touching, pt)
    assert below.max() == 12
    e.close()


def test_coordination_needs_a_single_scene(engine_lib):
    b = engine_lib.BatchEngine([scenes.cluster(n=27, seed=1), scenes.cluster(n=27, seed=2)])
    with pytest.raises(engine_lib.EngineError) as ex:
        b.coordination()
    assert ex.value.code == 1
    b.close()
