"""ctypes binding of the job server (``vedo_srv_*`` in include/vedo_gpu.h) and the serving workload.

:class:`Server` owns one GPU and batches every live job into the same fused launches
(continuous batching); jobs are submitted at any time from any thread.  :func:`job_stream`
draws the seeded Poisson job stream of the serving benchmark and :func:`job_scene` builds a
job's scene.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _abi, scenes
from ._abi import EngineOpts, StateView, dptr, scene_to_desc
from .engine import STATE_FIELDS, EngineError, _opts, lib

JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_CANCELLED, JOB_FAILED = range(5)
STATUS = {0: "queued", 1: "running", 2: "done", 3: "cancelled", 4: "failed"}
# admission charge (include/vedo_gpu.h): per object, and per listed neighbour of a sphere
BYTES_PER_OBJECT = 800
ENTRIES_PER_SPHERE = 18
BYTES_PER_ENTRY = 150
BYTES_PER_ENTRY_PAIR_PASS = 72


def job_charge(num_objects: int, num_spheres: int, pair_pass: bool = False) -> int:
    """Device memory the server's admission counts for a job (`pair_pass`: the server's options
    ask for the pair pass or for autotuning)."""
    per_entry = BYTES_PER_ENTRY + (BYTES_PER_ENTRY_PAIR_PASS if pair_pass else 0)
    return BYTES_PER_OBJECT * num_objects + ENTRIES_PER_SPHERE * per_entry * num_spheres


class JobInfo(C.Structure):
    _fields_ = [("status", C.c_uint32), ("num_objects", C.c_uint32), ("steps", C.c_uint64),
                ("steps_done", C.c_uint64), ("submit_s", C.c_double), ("admit_s", C.c_double),
                ("done_s", C.c_double), ("charged_bytes", C.c_uint64)]


def _srv_lib():
    L = lib()
    if not getattr(L, "_srv_typed", False):
        vp = C.c_void_p
        L.vedo_srv_create.argtypes = [C.POINTER(EngineOpts), C.c_uint64, C.POINTER(vp)]
        L.vedo_srv_submit.argtypes = [vp, C.POINTER(_abi.SceneDesc), C.c_uint64, C.POINTER(C.c_uint64)]
        L.vedo_srv_set_policy.argtypes = [vp, C.c_uint32, C.c_uint64]
        L.vedo_srv_poll.argtypes = [vp, C.c_uint64, C.POINTER(JobInfo)]
        L.vedo_srv_wait.argtypes = [vp, C.c_uint64, C.c_double, C.POINTER(JobInfo)]
        L.vedo_srv_result.argtypes = [vp, C.c_uint64, C.POINTER(StateView)]
        L.vedo_srv_cancel.argtypes = [vp, C.c_uint64]
        L.vedo_srv_stats.argtypes = [vp, C.POINTER(C.c_double)]
        L.vedo_srv_last_error.argtypes = [vp]
        L.vedo_srv_last_error.restype = C.c_char_p
        L.vedo_srv_destroy.argtypes = [vp]
        L._srv_typed = True
    return L


def _info(ji: JobInfo) -> Dict:
    return {"status": STATUS[ji.status], "num_objects": ji.num_objects, "steps": ji.steps,
            "steps_done": ji.steps_done, "submit_s": ji.submit_s, "admit_s": ji.admit_s, "done_s": ji.done_s,
            "charged_bytes": ji.charged_bytes}


class Server:
    """Continuous-batching DEM job server on one GPU (MIXED form).

    `order` = "fifo" (admission in arrival order) or "shortest" (the queued job with the least
    spheres x steps first); `max_live_spheres` caps the spheres of the running jobs (0: no cap
    beyond the HBM budget)."""

    def __init__(self, hbm_budget_bytes: int = 150 * 10**9, device: int = 0, order: str = "fifo",
                 max_live_spheres: int = 0, **engine_opts):
        L = _srv_lib()
        opts = _opts(1, 0, _abi.PRECISION_MIXED, device, None, engine_opts.get("skin"),
                     engine_opts.get("check_interval"), engine_opts.get("tick_block"), engine_opts.get("cell_scale"),
                     engine_opts.get("autotune", False), engine_opts.get("graphs", True),
                     split_tick=engine_opts.get("split_tick", False), pair_pass=engine_opts.get("pair_pass", False),
                     orientations=engine_opts.get("orientations", False),
                     persistent=engine_opts.get("persistent", False))
        h = C.c_void_p()
        rc = L.vedo_srv_create(C.byref(opts), int(hbm_budget_bytes), C.byref(h))
        if rc != 0:
            raise EngineError(rc, L.vedo_srv_last_error(None).decode())
        self.h = h
        self.sizes: Dict[int, int] = {}
        if order not in ("fifo", "shortest"):
            raise ValueError(f"order must be 'fifo' or 'shortest', not {order!r}")
        self._check(L.vedo_srv_set_policy(h, 1 if order == "shortest" else 0, int(max_live_spheres)))

    def _check(self, rc: int):
        if rc != 0:
            raise EngineError(rc, _srv_lib().vedo_srv_last_error(self.h).decode())

    def submit(self, scene, steps: int) -> int:
        desc, keep = scene_to_desc(scene)
        jid = C.c_uint64(0)
        self._check(_srv_lib().vedo_srv_submit(self.h, C.byref(desc), int(steps), C.byref(jid)))
        del keep
        self.sizes[jid.value] = scene.num_objects
        return jid.value

    def poll(self, job: int) -> Dict:
        ji = JobInfo()
        self._check(_srv_lib().vedo_srv_poll(self.h, job, C.byref(ji)))
        return _info(ji)

    def wait(self, job: int, timeout: float = 3600.0) -> Dict:
        ji = JobInfo()
        self._check(_srv_lib().vedo_srv_wait(self.h, job, float(timeout), C.byref(ji)))
        return _info(ji)

    def result(self, job: int, fields=STATE_FIELDS) -> Dict[str, np.ndarray]:
        n = self.sizes[job]
        out = {f: np.zeros((n, 3)) for f in fields}
        v = StateView()
        for f in fields:
            setattr(v, f, dptr(out[f]))
        self._check(_srv_lib().vedo_srv_result(self.h, job, C.byref(v)))
        return out

    def cancel(self, job: int):
        self._check(_srv_lib().vedo_srv_cancel(self.h, job))

    def stats(self) -> Dict:
        o = (C.c_double * 8)()
        self._check(_srv_lib().vedo_srv_stats(self.h, o))
        keys = ("jobs_done", "particle_steps_done", "busy_s", "batches", "batch_objects", "committed_bytes",
                "queued", "running")
        return {k: float(o[i]) for i, k in enumerate(keys)}

    def close(self):
        if getattr(self, "h", None):
            _srv_lib().vedo_srv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---- the serving workload ------------------------------------------------------------------
def job_stream(rate: float = 200.0, duration: float = 60.0, seed: int = 4242, n_lo: int = 2000,
               n_hi: int = 200000, steps_lo: int = 1000, steps_hi: int = 20000) -> List[Tuple]:
    """Seeded Poisson arrivals: (t_arrival_s, kind, n, steps, model, seed) per job; kind
    'settle' or 'projectile' and model 'lsd' or 'hertz' 50/50; n and steps log-uniform."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        kind = "settle" if rng.random() < 0.5 else "projectile"
        model = "lsd" if rng.random() < 0.5 else "hertz"
        n = int(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi))))
        st = int(math.exp(rng.uniform(math.log(steps_lo), math.log(steps_hi))))
        out.append((t, kind, n, st, model, int(rng.integers(0, 2**31 - 1))))
    return out


def job_scene(kind: str, n: int, model: str, seed: int, steps: int = 1000):
    """A serving job's scene (see :func:`vedo_gb300.scenes.serving_job`)."""
    return scenes.serving_job(kind, n, model, seed, steps)


def latency_percentiles(lat: Sequence[float]) -> Dict[str, float]:
    a = np.asarray(lat, dtype=float)
    return {"p50_ms": float(np.percentile(a, 50) * 1e3), "p99_ms": float(np.percentile(a, 99) * 1e3),
            "mean_ms": float(a.mean() * 1e3)}


def serve_stream(server: Server, stream: Sequence[Tuple], scenes_by_job: Optional[List] = None,
                 timeout: float = 3600.0) -> Dict:
    """Submit the jobs at their arrival times (real time, relative to the call), wait for all,
    and report latencies (submission to completion) and throughput.  Scenes are built before
    the clock starts."""
    built = scenes_by_job or [job_scene(k, n, m, sd, st) for (_, k, n, st, m, sd) in stream]
    parts = [int(sum(1 for mi in sc.model_index if sc.models[mi].scope == 2)) for sc in built]
    t0 = time.perf_counter()
    ids = []
    for (ta, *_), sc, (_, _, _, st, _, _) in zip(stream, built, stream):
        d = ta - (time.perf_counter() - t0)
        if d > 0:
            time.sleep(d)
        ids.append(server.submit(sc, st))
    infos = [server.wait(j, timeout) for j in ids]
    wall = time.perf_counter() - t0
    done = [i for i in infos if i["status"] == "done"]
    lat = [i["done_s"] - i["submit_s"] for i in done]
    ps = sum(p * st for p, (_, _, _, st, _, _), i in zip(parts, stream, infos) if i["status"] == "done")
    offered = sum(p * st for p, (_, _, _, st, _, _) in zip(parts, stream)) / max(stream[-1][0], 1e-9)
    return {"jobs": len(stream), "done": len(done), "wall_s": wall, "particle_steps": ps,
            "served_particle_steps_per_s": ps / wall, "offered_particle_steps_per_s": offered,
            **latency_percentiles(lat), "ids": ids, "infos": infos}
