"""SystemStatus.csv fixtures written by the reference itself.

Runs the reference DEM CPU path (compiled from its sources by ``make -C oracle ref``; needs the
reference checkout, default /root/reference or $VEDO_REFERENCE) on two seeded scenes with the
candidate list rebuilt every UP_IACT steps, and keeps the SystemStatus.csv its SimMediator
writes (the header and one line at construction and at every reset, SimMediator.cpp:46-123),
with the scene as the reference read it.

    python tests/golden/status/make_status.py     # -> tests/golden/status/<case>.npz
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

from vedo_gb300 import scenes  # noqa: E402


def cases():
    yield "box_lsd", scenes.lsd_box(n_side=5, steps=3000, vel_sigma=0.3, seed=11), 400, 10
    yield "cluster_ISwH", scenes.cluster(n=48, solver="ISwH", steps=400, seed=5), 300, 5


def main():
    import oracle
    oracle.build_ref()
    from oracle import RefWorld
    for name, sc, steps, up in cases():
        w = RefWorld(sc, up_iact=up)
        w.run(steps)
        with open(os.path.join(w.tmp.name, "SystemStatus.csv"), "rb") as f:
            csv = f.read()
        w.close()
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), ido=np.frombuffer(sc.to_ido(), np.uint8),
                            steps=steps, up_iact=up, csv=np.frombuffer(csv, np.uint8))
        print(name, csv.decode().count("\n"), "lines")


if __name__ == "__main__":
    main()
