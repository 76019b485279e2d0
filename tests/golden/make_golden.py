"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference DEM CPU path (compiled from the reference sources by
``make -C oracle ref``; needs the reference checkout, default /root/reference or
$VEDO_REFERENCE) on small seeded scenes and stores, per case, the scene as the
reference reads it (.ido bytes), the run parameters and the reference's results:
final object state, candidate list (IactPairTab order), interaction list
(slave/master, active flag, shear history, kn, contact flag) and energies.

    python tests/golden/make_golden.py [case ...]      # all cases, or the named ones

The observables' fixtures (tests/golden/observables/) hold the reference's coordination numbers
(CalcCoordinateNum, compiled with the reference) and its VTK files for scenes with exact ties.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

from vedo_gb300 import scenes  # noqa: E402


LEAP = {"leap_cluster_poly", "leap_box_lsd", "leap_periodic_lsd", "leap_periodic_wide", "leap_wide_y",
        "leap_column_z", "leap_single", "leap_zoi", "leap_zoi_h"}


def cases():
    """(name, scene, steps, up_iact) of every fixture; the leap_* ones run the Leap consultant."""
    yield "box_lsd", scenes.lsd_box(n_side=5, steps=3000, vel_sigma=0.3, seed=11), 2500, 10
    for solver in ("ISwBSDBF", "ISwBtSDBF", "ISwBSDB2F", "ISwHertz", "ISwH"):
        yield f"cluster_{solver}", scenes.cluster(n=48, solver=solver, steps=400, seed=5), 300, 5
    yield "cluster_poly_orbital_cyl", scenes.cluster(n=48, solver="ISwH", polydisperse=True, orbital=True,
                                                     cylinders=3, steps=300, seed=9), 200, 3
    yield "cluster_bsdbf_upiact1", scenes.cluster(n=27, solver="ISwBSDBF", steps=200, seed=2), 150, 1
    yield "cluster_zoi", zoi_scene(), 200, 5
    # the Leap consultant erases the mobile objects that leave the zone at every reset
    # (LeapConsultant.cpp:61-68), re-keying the contact records (IactRecordTab::ModifyPair)
    yield "leap_zoi", leap_zoi_scene(), 1500, 5
    yield "leap_zoi_h", leap_zoi_scene(solver="ISwH", seed=19), 1000, 5
    yield "holed_plate_lsd", scenes.holed_plate_drop(steps=500), 400, 5
    # a lid on the cluster moved by its impulses: a mobile plate (translation and rotation,
    # DOQuasiPlate.cpp:20-41) and a constrained one (along its normal, DOConstrainedQuasiPlate.cpp:18-35)
    yield "piston_mobile_lsd", scenes.piston(behavior="mobile", solver="ISwBSDBF"), 600, 5
    yield "piston_constrained_h", scenes.piston(behavior="constrained", solver="ISwH"), 600, 5
    # periodic boundary: spheres drift across the faces (wrap, minimum image in the detector and
    # in every law's lever arms); ISwH with an orbital floor and side walls that the wrap moves
    yield "periodic_lsd", scenes.periodic_layer(solver="ISwBSDBF"), 400, 5
    yield "periodic_hertz", scenes.periodic_layer(solver="ISwHertz", seed=8), 400, 5
    yield "periodic_btsdbf", scenes.periodic_layer(solver="ISwBtSDBF", seed=15), 300, 5
    yield "periodic_bsdb2f", scenes.periodic_layer(solver="ISwBSDB2F", seed=16), 300, 5
    # the Leap consultant's candidate list: polydisperse (its cell edge takes the largest range),
    # a box, and periodic layers (neighbour zones wrap across the faces)
    yield "leap_cluster_poly", scenes.cluster(n=48, solver="ISwH", polydisperse=True, orbital=True, cylinders=3,
                                              steps=300, seed=9), 200, 3
    yield "leap_box_lsd", scenes.lsd_box(n_side=5, steps=3000, vel_sigma=0.3, seed=11), 600, 10
    yield "leap_periodic_lsd", scenes.periodic_layer(solver="ISwBSDBF"), 400, 5
    yield "leap_periodic_wide", scenes.periodic_layer(nx=8, ny=6, layers=2, solver="ISwBSDBF", seed=22), 400, 5
    # the widest spread along y, then along z: the TrirLeY and TrirLeZ zone orders
    yield "leap_wide_y", scenes.periodic_layer(nx=3, ny=10, layers=2, solver="ISwBSDBF", seed=23), 300, 5
    yield "leap_column_z", scenes.periodic_layer(nx=3, ny=3, layers=12, solver="ISwBSDBF", seed=24,
                                                 drift=(2.0, 1.0)), 300, 5
    # one local sphere in a box: the 98 % quantile's index is negative before truncation
    yield "leap_single", scenes.cluster(n=1, solver="ISwBSDBF", steps=300, seed=3, vel_sigma=2.0), 200, 5
    yield "periodic_far_lsd", scenes.periodic_layer(solver="ISwBSDBF", nx=3, ny=3, layers=2, seed=12,
                                                    outside=True), 200, 4
    yield "periodic_h", scenes.periodic_layer(solver="ISwH", periodic_y=False, floor_spin=40.0, side_walls=True,
                                              seed=9, drift=(0.0, 0.0)), 400, 5


def zoi_scene():
    """A settled LSD cluster (the reference's own .ido after 150 steps, with contact records)
    given a zone of interest in z that leaves about a quarter of the spheres outside: the
    reference erases them before the first step (Consultant::CleanUp) and re-keys the records
    (IactRecordTab::ModifyPair), walls included, since they follow the spheres."""
    import tempfile
    from oracle import RefWorld
    from vedo_gb300.scene import Boundary, Scene
    sc = scenes.cluster(n=48, solver="ISwBSDBF", steps=400, seed=5)
    w = RefWorld(sc, up_iact=5)
    w.run(150)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "w.ido")
        w.write_ido(path)
        w.close()
        out = Scene.from_ido(path)
    mobile = [k for k, m in enumerate(out.model_index) if out.models[m].behavior == 3]
    z = np.sort(out.position[mobile, 2])
    cut = 0.5 * (z[3 * len(z) // 4 - 1] + z[3 * len(z) // 4])
    out.sp.zoi = Boundary(switch=(False, False, True), lower=(0.0, 0.0, float(z[0]) - 1.0), upper=(0.0, 0.0, cut))
    return out


def leap_zoi_scene(solver: str = "ISwBSDBF", seed: int = 13):
    """Colliding spheres (0.5 m/s) in a box of plates with a zone of interest 0.05 mm beyond the
    outermost spheres in x: over the run about half the spheres cross it and are erased at the
    next reset, most erasures with contacts active (records re-keyed)."""
    from vedo_gb300.scene import Boundary
    sc = scenes.cluster(n=48, solver=solver, steps=3000, seed=seed, vel_sigma=0.5)
    mobile = [k for k, m in enumerate(sc.model_index) if sc.models[m].behavior == 3]
    x = sc.position[mobile, 0]
    sc.sp.zoi = Boundary(switch=(True, False, False), lower=(float(x.min()) - 5e-5, 0.0, 0.0),
                         upper=(float(x.max()) + 5e-5, 0.0, 0.0))
    return sc


def observable_cases():
    """(name, scene, box) of the coordination-number / VTK fixtures (tests/golden/observables/)."""
    yield "touching_lattice", scenes.touching_lattice(), (0.0, 0.003, 0.0, 0.003, 0.0, 0.002)
    yield "touching_lattice_whole", scenes.touching_lattice(seed=14, loose=80), (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)


def make_observables(only):
    """The reference's CalcCoordinateNum and DOWorld::WriteVTK on a scene read from its IDO file:
    the box average, the coordination VTK file and the plain world VTK file, as written."""
    import tempfile
    from oracle import ref_coordination
    out_dir = os.path.join(HERE, "observables")
    os.makedirs(out_dir, exist_ok=True)
    for name, sc, box in observable_cases():
        if only and name not in only:
            continue
        with tempfile.TemporaryDirectory() as td:
            cv, wv = os.path.join(td, "c.vtu"), os.path.join(td, "w.vtu")
            avg = ref_coordination(sc, box, cv, wv)
            coord_vtk, world_vtk = open(cv, "rb").read(), open(wv, "rb").read()
        np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), ido=np.frombuffer(sc.to_ido(), np.uint8),
                            box=np.array(box), average=avg, coord_vtk=np.frombuffer(coord_vtk, np.uint8),
                            world_vtk=np.frombuffer(world_vtk, np.uint8))
        print(name, sc.num_objects, "objects, average coordination", avg)


def main():
    import oracle
    oracle.build_ref()
    from oracle import RefWorld
    only = set(sys.argv[1:])
    make_observables(only)
    for name, sc, steps, up in cases():
        if only and name not in only:
            continue
        ido = sc.to_ido()
        consultant = "leap" if name in LEAP else "nbs"
        w = RefWorld(sc, up_iact=up, consultant=consultant)
        cf0, cs0 = w.candidates()
        w.run(steps)
        st = w.state()
        cf, cs = w.candidates()
        it = w.interactions()
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), ido=np.frombuffer(ido, np.uint8), steps=steps,
                            up_iact=up, consultant=consultant, cand0_first=cf0, cand0_second=cs0, cand_first=cf, cand_second=cs,
                            time=w.time(), energy=w.energy(),
                            **{f"state_{k}": v for k, v in st.items()},
                            **{f"iact_{k}": v for k, v in it.items()})
        print(name, sc.num_objects, "objects", len(cf), "candidates", int(it["active"].sum()), "active")
        w.close()


if __name__ == "__main__":
    main()
