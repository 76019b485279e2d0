import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def port_lib():
    import oracle
    oracle.build_port()
    return oracle


@pytest.fixture(scope="session")
def engine_lib():
    from vedo_gb300 import build
    build.build()
    from vedo_gb300 import engine
    return engine


def _settled(engine, tmp, scene, steps, name, vmax=10.0):
    e = engine.GpuEngine(scene, up_iact=20)
    e.run(steps)
    import numpy as np
    speed = np.linalg.norm(e.state(("velocity",))["velocity"], axis=1).max()
    assert speed < vmax, f"{name}: the settling run is unstable (max speed {speed:.3g} m/s)"
    p = str(tmp / f"{name}.ido")
    e.write_ido(p)
    e.close()
    return p


@pytest.fixture(scope="session")
def box_ido(engine_lib, tmp_path_factory):
    """A 1,728-sphere LSD box after 4,000 FP64 steps: many persistent contacts."""
    from vedo_gb300 import scenes
    sc = scenes.lsd_box(n_side=12, vel_sigma=0.3, spacing=2.05e-3)
    return _settled(engine_lib, tmp_path_factory.mktemp("settled"), sc, 4000, "box")


@pytest.fixture(scope="session")
def drum_ido(engine_lib, tmp_path_factory):
    """A 40,000-sphere Hertz drum after 3,000 FP64 steps (dt 5e-7 s, E 70 GPa)."""
    from vedo_gb300 import scenes
    sc = scenes.hertz_drum(n=40000, seed=3, steps=100, gap=0.002, vel_sigma=0.05, fill="lattice")
    return _settled(engine_lib, tmp_path_factory.mktemp("settled"), sc, 3000, "drum")
