"""Contact-bearing states of the measured workloads, made by running the engine itself.

The configured scenes start loose (a drum filled by random sequential placement, hoppers on a
lattice): for the first thousands of steps nothing touches, and a window timed there measures
free fall.  These helpers advance a scene through its settling with the mixed form and write
the settled state, contact histories included, as an ``.ido`` file, so that a benchmark window
starts where the spheres rest on one another.

Settled states are cached on disk (``$VEDO_CACHE``, default ``/tmp/vedo_gb300_cache``) under a
key made of the scene's parameters, the step count and a digest of the engine library, so that
several processes on one host (the benchmark's two arms) settle a scene once.
"""
from __future__ import annotations

import hashlib
import json
import os
import time
from typing import Callable, Optional

from . import scenes
from .engine import LIB_PATH, GpuEngine

CACHE = os.environ.get("VEDO_CACHE", "/tmp/vedo_gb300_cache")


def _lib_digest() -> str:
    h = hashlib.sha256()
    with open(LIB_PATH, "rb") as f:
        for chunk in iter(lambda: f.read(1 << 20), b""):
            h.update(chunk)
    return h.hexdigest()[:16]


def settle(scene, steps: int, out_path: str, device: int = 0, segment: int = 100_000,
           log: Optional[Callable[[dict], None]] = None) -> dict:
    """Advance `scene` by `steps` time steps in the mixed form (autotuned) and write the state
    with its contact histories to `out_path`.  The run is split into segments of `segment`
    steps, each in a fresh engine read from the previous segment's file, so that the tuning
    (tick shape, skin, cell size) follows the change from free fall to resting contact; the
    segments are ordinary steps (results do not depend on the tuning).  Returns a summary."""
    src = scene
    done = 0
    t0 = time.time()
    info = {}
    while done < steps:
        k = min(segment, steps - done)
        e = GpuEngine(src, precision=1, autotune=True, device=device)
        e.run(k)
        done += k
        o = e.observables()
        info = {"steps": done, "kinetic_energy": float(o[1] + o[2]), "contacts": int(o[9]),
                "z_pp": float(o[9]) / max(1, e.n), "wall_s": round(time.time() - t0, 1), "tuning": e.tuning()}
        if log:
            log(info)
        tmp = out_path + ".part"
        e.write_ido(tmp)
        e.close()
        os.replace(tmp, out_path)
        src = out_path
    info["wall_s"] = round(time.time() - t0, 1)
    return info


def _cached(key: dict, make: Callable[[str], dict]) -> tuple:
    os.makedirs(CACHE, exist_ok=True)
    key = dict(key, lib=_lib_digest())
    name = hashlib.sha256(json.dumps(key, sort_keys=True).encode()).hexdigest()[:20]
    path = os.path.join(CACHE, name + ".ido")
    meta = path + ".json"
    if os.path.exists(path) and os.path.exists(meta):
        with open(meta) as f:
            return path, dict(json.load(f), cached=True)
    info = make(path)
    with open(meta, "w") as f:
        json.dump(dict(info, key=key), f)
    return path, dict(info, cached=False)


def settled_drum(n: int = 1_000_000, seed: int = 2024, settle_steps: int = 300_000, run_steps: int = 10_000,
                 device: int = 0, log=None) -> tuple:
    """The polydisperse Hertz drum (scenes.hertz_drum, random sequential placement) after
    `settle_steps` steps of settling under gravity with its end plates turning: returns the
    ``.ido`` path and a summary (contacts, kinetic energy, wall time, whether cached).  The
    file's time control leaves `run_steps` more steps."""
    def make(path):
        sc = scenes.hertz_drum(n=n, seed=seed, steps=settle_steps + run_steps)
        return settle(sc, settle_steps, path, device=device, log=log)
    return _cached({"kind": "drum", "n": n, "seed": seed, "settle": settle_steps, "run": run_steps}, make)
