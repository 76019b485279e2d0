"""anne-gpu, the reference's `anne` command line over the GPU engine: it runs an .ido scene to
t_stop, writes the record and terminate files, and its FP64 result equals the C oracle's."""
import os
import subprocess

import numpy as np
import pytest

from vedo_gb300 import scenes
from vedo_gb300.scene import Scene

pytestmark = pytest.mark.gpu


def test_anne_gpu_runs_to_t_stop_like_the_oracle(engine_lib, port_lib, tmp_path):
    from oracle import PortWorld
    from vedo_gb300 import build
    sc = scenes.cluster(n=64, solver="ISwBSDBF", steps=150, seed=4)
    ido = str(tmp_path / "job.ido")
    sc.to_ido(ido)
    r = subprocess.run([build.CLI, "analysis", ido, "nbs", "50", "5"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert os.path.exists(tmp_path / "terminate.ido")
    # Consultant::RecordIDO naming (Consultant.cpp:217-230): <ido file>_000001.ido, ...
    assert sorted(p for p in os.listdir(tmp_path) if p.startswith("job.ido_")) == \
        ["job.ido_000001.ido", "job.ido_000002.ido", "job.ido_000003.ido"]
    end = Scene.from_ido(str(tmp_path / "terminate.ido"))
    ref = PortWorld(sc, up_iact=5)
    steps = 0
    while ref.time() < sc.sp.time_stop:
        ref.run(1)
        steps += 1
    assert steps == 150
    st = ref.state()
    assert np.array_equal(end.position, st["position"])
    assert np.array_equal(end.velocity, st["velocity"])
    # the mixed form through the same command line
    r = subprocess.run([build.CLI, "analysis", ido, "nbs", "50", "5", "--mixed"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    mx = Scene.from_ido(str(tmp_path / "terminate.ido"))
    # FP32 pair forces: after 150 colliding steps within 5e-5 of the sphere size (1 mm) of the FP64 path
    assert np.abs(mx.position - st["position"]).max() < 5e-8


def test_anne_gpu_usage_and_unsupported_mode(engine_lib, tmp_path):
    from vedo_gb300 import build
    r = subprocess.run([build.CLI], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage: anne-gpu" in r.stdout
    ido = str(tmp_path / "x.ido")
    scenes.cluster(n=8).to_ido(ido)
    r = subprocess.run([build.CLI, "redistribute", ido, "nbs", "10", "1"], capture_output=True, text=True)
    assert r.returncode == 2
