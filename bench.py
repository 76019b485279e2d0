#!/usr/bin/env python3
"""DEM time-step throughput on GB300: particle-steps/s on the 1,000,000-sphere polydisperse
Hertz drum (radii lognormal median 1 mm, sigma_log 0.2, clipped to [0.5, 2] mm, 32 classes;
E = 70 GPa, nu = 0.25, e = 0.7, mu = 0.4 via the frictional Hertz-family law ISwH;
drum R = 0.15 m, L = 0.3 m, polygon shell of 64 fixed plates, end plates at 30 rpm;
dt = 5e-7 s; filled by random sequential placement).  Synthetic seeded scene
(vedo_gb300.scenes.hertz_drum), settled on the GPU before the timed window
(vedo_gb300.workloads.settled_drum: 300,000 steps of settling under gravity, untimed) so that
the window times the contact step of a resting, rotating bed, not free fall.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one DEM time step of the whole scene (SimMediator::Run).  `value` is measured
with CUDA events on the engine's stream around exactly K steps with the scene resident in
HBM; `e2e` goes through the C ABI with host buffers (state uploaded from pinned memory,
stepped, read back, every `--sync` steps).  Under torchrun (N > 1) every rank runs an
independent replica of the scene (no collective on the data path) and `value` is the
particle-steps of all ranks over the slowest rank's time.  `--impl reference` times the
reference algorithm on the host cores (the C restatement of the reference step; the
reference's own build cannot run on this host) on the same settled state.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300 (mixed vs FP64 at stated error); serving p50/p99 ms"
UNIT = "particle-steps/s"
WORKLOAD = "hertz_drum_1M"
TUNE_STEPS = 500


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=1_000_000, help="spheres in the drum")
    ap.add_argument("--up-iact", type=int, default=20, help="candidate-list rebuild interval")
    ap.add_argument("--sync", type=int, default=20, help="e2e: steps between host state round trips")
    ap.add_argument("--e2e-iters", type=int, default=3)
    ap.add_argument("--cpu-sample-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-profile-pass", action="store_true")
    ap.add_argument("--profile-steps", type=int, default=200, help="steps of the per-kernel timing pass")
    ap.add_argument("--batch-scenes", type=int, default=256, help="hopper scenes of the batched workload")
    ap.add_argument("--batch-steps", type=int, default=300, help="timed steps of the batched workload")
    ap.add_argument("--serve-duration", type=float, default=2.0, help="seconds of Poisson arrivals (200/s)")
    ap.add_argument("--serve-steps-scale", type=float, default=1.0, help="job step counts x this factor")
    ap.add_argument("--serve-fp64-jobs", type=int, default=24, help="jobs of the stream run one at a time on FP64")
    ap.add_argument("--serve-cap", type=int, default=2_000_000, help="live-sphere cap of the shortest-first run")
    ap.add_argument("--bed-n", type=int, default=16_000_000, help="spheres of the compressed-bed workload")
    ap.add_argument("--bed-steps", type=int, default=100, help="timed steps of the compressed-bed workload")
    ap.add_argument("--no-bed", action="store_true")
    ap.add_argument("--dense-n", type=int, default=1_000_000, help="spheres of the contact-dense workload")
    ap.add_argument("--no-dense", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-c1", action="store_true")
    ap.add_argument("--settle-steps", type=int, default=300_000, help="drum settling steps before the window")
    ap.add_argument("--c1-cpu-steps", type=int, default=20_000, help="C1 CPU baseline steps (full run: 20000)")
    ap.add_argument("--cpu-job", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-out", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-scene", default=None, help=argparse.SUPPRESS)
    return ap.parse_args()


# ------------------------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend="gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def reduce(self, x: float, op: str) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def gather(self, obj) -> list:
        """Every rank's `obj`, in rank order (the rank's own alone when there is one rank)."""
        if not self.pg:
            return [obj]
        out = [None] * self.world
        self.pg.all_gather_object(out, obj)
        return out

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi samples (clocks, power, throttle reasons) kept for the timed region: the sampler
    runs every 50 ms from before the warm-up, and only samples stamped between the region's start
    and end are used (the nearest ones around it when the region is shorter than one interval)."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            deadline = time.time() + 5.0                  # wait for the sampler's first line
            while time.time() < deadline and os.path.getsize(self.path) == 0:
                time.sleep(0.02)
        except Exception:
            self.proc = None

    def begin(self):
        self.t0 = time.time()

    def end(self):
        self.t1 = time.time()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.1)                                   # one more sample after the region
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 10:
                continue
            try:
                ts = time.mktime(time.strptime(p[0].split(".")[0], "%Y/%m/%d %H:%M:%S")) + float("0." + p[0].split(".")[1])
                rows.append((ts, float(p[2]), float(p[3]), [nm for k, nm in enumerate(names)
                                                            if p[6 + k].lower().startswith("active")]))
            except (ValueError, IndexError):
                continue
        os.unlink(self.path)
        t0, t1 = self.t0 or 0.0, self.t1 or 0.0
        inside = [r for r in rows if t0 <= r[0] <= t1]
        where = "inside the timed region"
        if not inside and rows:                           # region shorter than the interval
            inside = sorted(rows, key=lambda r: min(abs(r[0] - t0), abs(r[0] - t1)))[:2]
            where = "nearest to the timed region"
        sm = [r[1] for r in inside]
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(r[2] for r in inside) if inside else None,
                "reasons": sorted({nm for r in inside for nm in r[3]}), "samples": len(sm), "where": where,
                "region_s": round(t1 - t0, 4)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def emit(d):
    print(json.dumps(d), flush=True)


# ------------------------------------------------------------------------------------------
def cpu_rate(scene, up_iact, steps):
    """The reference step restated in C (oracle/dem_oracle.c), single thread, on this host."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build_port()
    from oracle import PortWorld
    w = PortWorld(scene, up_iact=up_iact)
    t0 = time.perf_counter()
    w.run(steps)
    t1 = time.perf_counter()
    w.close()
    return scene_particles(scene) * steps / (t1 - t0), t1 - t0


def cpu_job(args):
    """A CPU baseline in its own process (so that it runs beside the GPU sections): the C
    restatement of the reference step over `--cpu-scene` (an .ido path, or "c1" for the
    8,000-sphere box) for `--steps` steps; writes its rate to `--cpu-out`."""
    from vedo_gb300 import scenes
    from vedo_gb300.scene import Scene
    if args.cpu_scene == "c1":
        sc = scenes.lsd_box(steps=20000)
    else:
        sc = Scene.from_ido(args.cpu_scene)
    rate, secs = cpu_rate(sc, args.up_iact, args.steps)
    with open(args.cpu_out, "w") as f:
        json.dump({"value": rate, "seconds": secs, "steps": args.steps, "particles": scene_particles(sc)}, f)


class CpuJob:
    """A cpu_job subprocess; result() waits for it and returns its JSON (None if it failed)."""
    def __init__(self, scene_arg, steps, up_iact):
        fd, self.out = tempfile.mkstemp(suffix=".json")
        os.close(fd)
        self.proc = subprocess.Popen([sys.executable, os.path.abspath(__file__), "--cpu-job", "1", "--cpu-scene",
                                      scene_arg, "--steps", str(steps), "--up-iact", str(up_iact), "--cpu-out",
                                      self.out], stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)

    def result(self, timeout=1800):
        try:
            _, err = self.proc.communicate(timeout=timeout)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            return None
        try:
            with open(self.out) as f:
                return json.load(f)
        except (OSError, ValueError):
            sys.stderr.write((err or b"").decode()[-2000:])
            return None
        finally:
            os.unlink(self.out)


def scene_particles(scene):
    from vedo_gb300.scene import SPHERE
    sph = [k for k, m in enumerate(scene.models) if m.shape == SPHERE]
    import numpy as np
    return int(np.isin(scene.model_index, sph).sum())


def settled_drum(args, dist, collective=True):
    """The settled 1M-sphere drum of this rank (built and settled on its GPU once, then cached).
    collective: every rank calls it (the build runs once per host, behind a barrier)."""
    import torch
    from vedo_gb300 import build as vbuild
    from vedo_gb300 import workloads
    if dist.local == 0 or dist.world == 1:
        vbuild.build()
    if collective:
        dist.barrier()
    vbuild.build()
    torch.cuda.set_device(dist.local)
    return workloads.settled_drum(n=args.n, seed=2024 + dist.rank, settle_steps=args.settle_steps,
                                  device=dist.local)


def reference_arm(args, dist):
    """The C restatement of the reference step (single thread: the reference's step is
    sequential) on the same settled drum as the GPU arm.  The settled state is made by the GPU
    engine (untimed input preparation, cached on this host); the timed steps are CPU only."""
    if dist.rank != 0:
        return
    path, info = settled_drum(args, dist, collective=False)
    from vedo_gb300.scene import Scene
    scene = Scene.from_ido(path)
    n = scene_particles(scene)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build_port()
    from oracle import PortWorld
    w = PortWorld(scene, up_iact=args.up_iact)
    w.run(max(0, args.warmup))
    # bound the timed part to about two minutes of CPU work
    t0 = time.perf_counter()
    w.run(1)
    one = time.perf_counter() - t0
    k = max(1, min(args.steps - 1, int(120.0 / max(one, 1e-6))))
    t0 = time.perf_counter()
    w.run(k)
    dt = time.perf_counter() - t0 + one
    k += 1
    value = n * k / dt
    emit({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": k, "warmup": args.warmup,
          "ms_per_step": 1e3 * dt / k, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
          "dtype": "f64", "data": "synthetic (seeded hertz_drum scene, settled)", "impl": "reference",
          "config": {"workload": WORKLOAD, "particles": n, "up_iact": args.up_iact, "steps_timed": k,
                     "steps_requested": args.steps, "settle": info},
          "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                           "sample": f"{k} full time steps of the settled {n}-sphere drum ({info.get('contacts')} "
                                     f"contacts) after {args.warmup} warm-up steps, single thread (the reference "
                                     f"step is sequential)"},
          "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})


# ------------------------------------------------------------------------------------------
def time_form(eng, args, dist, clocks=None):
    """W warm-up steps, then exactly K timed steps (CUDA events on the engine stream, max over
    ranks); returns (ms for K steps, kernel launches in the timed region)."""
    import torch
    if clocks:
        clocks.start()
    eng.run(args.warmup)
    dist.barrier()
    torch.cuda.synchronize()
    if clocks:
        clocks.begin()
    eng.run(args.steps)
    prof = eng.last_run_profile()
    if clocks:
        clocks.end()
    rec = clocks.stop() if clocks else None
    dist.barrier()
    return dist.reduce(prof["total_ms"], "max"), prof["launches"], rec


def ours(args, dist):
    import numpy as np
    import torch
    from vedo_gb300.engine import GpuEngine
    from vedo_gb300.scene import Scene

    dev = dist.local
    # C1's full-run CPU baseline runs beside the GPU sections (single thread, its own process)
    c1_cpu = CpuJob("c1", args.c1_cpu_steps, 20) if (dist.rank == 0 and dist.world == 1 and not args.no_c1
                                                     and not args.no_cpu_baseline) else None
    path, settle_info = settled_drum(args, dist)
    scene = Scene.from_ido(path)
    n = scene_particles(scene)
    cpu_job_c2 = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        cpu_job_c2 = CpuJob(path, args.cpu_sample_steps, args.up_iact)
    total_particles = dist.reduce(float(n), "sum")

    # plain FP64 form (the drop-in): same settled state, same window
    f64 = GpuEngine(path, up_iact=args.up_iact, device=dev)
    t64, l64, _ = time_form(f64, args, dist)
    fp64_value = total_particles * args.steps / (t64 * 1e-3)

    # mixed form (the headline): FP32 pair forces, FP64 integration, compensated sums; the first
    # TUNE_STEPS steps choose the tick shape, skin and cell scale (results do not depend on them)
    eng = GpuEngine(path, up_iact=args.up_iact, device=dev, precision=1, autotune=True)
    eng.run(TUNE_STEPS)
    clocks = Clocks(dev)
    t_ms, launches, clocks_rec = time_form(eng, args, dist, clocks)
    value = total_particles * args.steps / (t_ms * 1e-3)
    o_mx = eng.observables()
    n_active = int(o_mx[9])                       # active contacts at the end of the window

    # error of the mixed form against the FP64 engine on this window: end-of-window energy and
    # the impulses of one step from the FP64 engine's state (restarted through an .ido so both
    # forms start from identical positions, velocities and shear history)
    f64.run(TUNE_STEPS)                          # both forms at the same step
    o64, omx = f64.observables(), eng.observables()
    e64, emx = o64[0] + o64[1] + o64[2], omx[0] + omx[1] + omx[2]
    errors = {"energy_rel": abs(e64 - emx) / max(abs(e64), 1e-300),
              "kinetic_rel": abs(o64[1] - omx[1]) / max(abs(o64[1]), 1e-300),
              "contacts_fp64": int(o64[9]), "contacts_mixed": int(omx[9]),
              "after_steps": TUNE_STEPS + args.warmup + args.steps}
    if args.n <= 2_000_000 and not args.no_profile_pass:
        with tempfile.TemporaryDirectory() as td:
            p2 = os.path.join(td, "w.ido")
            f64.write_ido(p2)
            a = GpuEngine(p2, up_iact=args.up_iact, device=dev)
            b = GpuEngine(p2, up_iact=args.up_iact, device=dev, precision=1)
            a.run(1)
            b.run(1)
            sa, sb = a.state(("impact", "angular_impact")), b.state(("impact", "angular_impact"))
            ia, ib = a.interactions(), b.interactions()
            A = set(zip(ia["first"][ia["active"] == 1].tolist(), ia["second"][ia["active"] == 1].tolist()))
            B = set(zip(ib["first"][ib["active"] == 1].tolist(), ib["second"][ib["active"] == 1].tolist()))
            for k in ("impact", "angular_impact"):
                d = sa[k] - sb[k]
                errors[f"step_{k}_rel_l2"] = float(np.linalg.norm(d) / max(np.linalg.norm(sa[k]), 1e-300))
            errors["contact_set_identical"] = A == B
            errors["contacts"] = len(A)
            a.close()
            b.close()
    f64.close()

    # per-kernel times of the mixed form from one profiled window: every tick launch (the
    # fused detect-force-integrate kernel) is timed alone with CUDA events on the engine stream
    kern = None
    if not args.no_profile_pass:
        eng.set_profiling(True)
        eng.run(args.profile_steps)
        kern = eng.last_run_profile()
        kern["steps"] = args.profile_steps
        eng.set_profiling(False)
    # e2e through the C ABI with pinned host buffers: the state that the step changes (sphere
    # orientations are not integrated in this form)
    fields = ("position", "velocity", "angular_velocity")
    pinned = {f: torch.empty((eng.n, 3), dtype=torch.float64, pin_memory=True) for f in fields}
    host = {f: pinned[f].numpy() for f in fields}
    eng.state(fields, out=host)
    e2e_t = 0.0
    e2e_steps = 0
    for _ in range(args.e2e_iters):
        t0 = time.perf_counter()
        eng.set_state(**host)
        eng.run(args.sync)
        eng.state(fields, out=host)
        t1 = time.perf_counter()
        e2e_t += t1 - t0
        e2e_steps += args.sync
    e2e_t = dist.reduce(e2e_t, "max")
    e2e_value = total_particles * e2e_steps / e2e_t if e2e_t > 0 else None
    xfer = 24 * eng.n * len(fields)

    # algorithmic bytes per particle-step of the mixed form: x, v, w (FP64) read + written
    # (sphere orientation is not integrated in this form), per active contact the FP32 history
    # (shear + kn, 16 B) read + written plus the pair index, plus the per-particle radius
    s_state = 72
    s_hist = 16
    z_pp = n_active / n
    b_alg = 2 * s_state + z_pp * (2 * s_hist + 8) + 8
    peak, peak_kind = peaks()
    roof = None
    if kern and kern["pair_ms"] > 0:
        t_tick = kern["pair_ms"] / kern["steps"]            # average duration of one tick launch
        ach = b_alg * n / (t_tick * 1e-3) / 1e9
        traffic = ncu_traffic("k_tick_drum1M_settled_dram.md") if n == 1_000_000 else None
        tuned = eng.tuning()
        if tuned.get("pair_pass"):
            kname = ("k_tick_pf + k_tick_pairs + k_tick_sum (pair pass: prefilter walk listing the pairs on the "
                     "exact path, one thread per pair for narrow phase + forces, per-sphere ordered sums + "
                     "integration)")
        elif tuned.get("split_tick"):
            kname = ("k_tick_light + k_tick_work (split tick: prefilter walk and integration at high occupancy, the "
                     "per-sphere contact tick over the spheres with a pair on the exact path)")
        else:
            kname = ("k_tick (per-sphere contact tick over the Z-order storage: narrow phase + forces + "
                     "integration, one launch per step)")
        roof = {"kernel": kname,
                "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "traffic": traffic,
                "traffic_source": "profiles/k_tick_drum1M_settled_dram.md (ncu, the same workload at full size)"
                if traffic else None,
                "dram_frac": traffic / (t_tick * 1e-3) / 1e9 / peak if traffic else None,
                "tick_ms": t_tick, "walls_ms": kern["object_ms"] / kern["steps"],
                "profile_pass": {"steps": kern["steps"], "launches": kern["launches"],
                                 "ms_per_step": kern["total_ms"] / kern["steps"], "rebuild_ms": kern["rebuild_ms"],
                                 "note": "graph replay with per-kernel event nodes (they add about 13 us per step)"},
                "share_of_step": t_tick / (t_ms / args.steps), "alg_bytes_per_launch": b_alg * n}
    res = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 forces + f64 state (mixed)",
           "data": "synthetic (seeded hertz_drum scene filled by random sequential placement and settled on the "
                   "GPU, no dataset)",
           "config": {"workload": WORKLOAD, "particles_per_gpu": n, "objects_per_gpu": eng.n,
                      "settle": settle_info,
                      "form": "mixed (FP32 pair-local forces, FP64 overlap numerator and integration, "
                              "Kahan sums; sphere orientations not asked for, so not integrated)",
                      "up_iact_fp64": args.up_iact, "active_contacts": n_active, "z_pp": z_pp,
                      "alg_bytes_per_particle_step": b_alg,
                      "l2": "working set larger than L2 (state + lists > 129 MB)",
                      "parallelism": f"replicas x{dist.world}",
                      "tuning": eng.tuning(),
                      "window": f"steps {TUNE_STEPS + args.warmup}..{TUNE_STEPS + args.warmup + args.steps} after "
                                f"{args.settle_steps} settling steps (FP64 form: steps "
                                f"{args.warmup}..{args.warmup + args.steps} after them); z_pp counted at the "
                                f"window's end"},
           "fp64": {"value": fp64_value, "ms_per_step": t64 / args.steps, "gpu_launches": l64,
                    "form": "plain FP64 drop-in, bit-exact operation order"},
           "mixed_over_fp64": value / fp64_value,
           "errors_mixed_vs_fp64": errors,
           "clocks": clocks_rec, "gpu_launches": launches,
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": xfer / args.sync,
                   "d2h_bytes_per_step": xfer / args.sync,
                   "note": f"vedo_gpu_set_state + vedo_gpu_run({args.sync}) + vedo_gpu_get_state of position, "
                           f"velocity and angular velocity (FP64) of every object per {args.sync} steps, pinned "
                           f"host buffers, mixed form"},
           "roofline": roof, "cpu_baseline": None}
    eng.close()
    if not args.no_batch:
        res["batch"] = batch_workload(args, dist, dev)
    if not args.no_bed:
        res["bed"] = bed_workload(args, dist, dev)
    if not args.no_dense:
        res["dense"] = dense_workload(args, dist, dev)
    if not args.no_c1:
        res["c1"] = c1_workload(args, dist, dev, c1_cpu)
    if not args.no_serve:
        res["serving"] = serving_workload(args, dist, dev)
    if cpu_job_c2:
        r = cpu_job_c2.result()
        if r:
            res["cpu_baseline"] = {"value": r["value"], "unit": UNIT, "cores": 1, "kind": "port",
                                   "sample": f"{r['steps']} time steps of the same settled {n}-sphere drum "
                                             f"(the state the window starts from), single thread, "
                                             f"{r['seconds']:.1f} s, run beside the GPU sections"}
    if dist.rank == 0:
        emit(res)


def c1_workload(args, dist, dev, cpu_job_c1):
    """C1: the 8,000-sphere linear spring-dashpot box, the whole 20,000-step run in the plain
    FP64 form (bit for bit the reference's) and in the mixed form, beside the C restatement of
    the reference's step over the same full run on one host core.  About 2 MB of state: the
    step lives in L2 and is bound by launch latency, so its roofline fraction means nothing."""
    import torch
    from vedo_gb300 import scenes
    from vedo_gb300.engine import GpuEngine
    sc = scenes.lsd_box(steps=20000)
    n = scene_particles(sc)
    out = {"workload": "lsd_box_8k (20,000 steps, dt 1e-6 s, candidate list every 20 steps)", "particles": n}
    for name, prec, pers in (("fp64", 0, False), ("mixed", 1, False), ("mixed_persistent", 1, True)):
        e = GpuEngine(sc, up_iact=20, device=dev, precision=prec, persistent=pers)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e.run(20000)
        wall = time.perf_counter() - t0
        prof = e.last_run_profile()
        o = e.observables()
        out[name] = {"value": n * 20000 / (prof["total_ms"] * 1e-3), "unit": UNIT,
                     "ms_per_step": prof["total_ms"] / 20000, "wall_s": wall, "gpu_launches": prof["launches"],
                     "kinetic_energy_end": float(o[1] + o[2]), "contacts_end": int(o[9])}
        e.close()
    if cpu_job_c1:
        r = cpu_job_c1.result()
        if r:
            out["cpu_baseline"] = {"value": r["value"], "unit": UNIT, "cores": 1, "kind": "port",
                                   "sample": f"{r['steps']} steps of the same scene (the full run), single thread, "
                                             f"{r['seconds']:.1f} s"}
            out["fp64_over_cpu"] = out["fp64"]["value"] / r["value"]
    out["note"] = ("L2-resident (state about 2 MB) and launch/latency-bound: one step is a few microseconds of "
                   "kernels, so the rate measures launch overhead, not HBM; mixed: each check interval of 10 "
                   "steps replayed as a CUDA graph of per-step kernels; mixed_persistent: each interval one "
                   "cooperative launch with grid barriers between the stages (identical results)")
    return out


def ncu_traffic(name):
    """DRAM bytes (read + write) of one step's tick launches from a committed ncu summary of the
    same workload at full size."""
    try:
        for line in open(os.path.join(ROOT, "profiles", name)):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def form_errors(scene, dev, pre_steps, post_steps=200, up_iact=20):
    """The mixed form against the FP64 engine on one scene: the FP64 engine runs `pre_steps`, both
    forms restart from its .ido (identical positions, velocities and contact history), and after
    one step their impulses and active contact sets are compared; after `post_steps` more steps,
    their total energies."""
    import numpy as np
    from vedo_gb300.engine import GpuEngine
    f64 = GpuEngine(scene, up_iact=up_iact, device=dev)
    f64.run(pre_steps)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "w.ido")
        f64.write_ido(path)
        f64.close()
        a = GpuEngine(path, up_iact=up_iact, device=dev)
        b = GpuEngine(path, up_iact=up_iact, device=dev, precision=1)
    a.run(1)
    b.run(1)
    f = ("impact", "angular_impact")
    sa, sb = a.state(f), b.state(f)
    out = {f"step_{k}_rel_l2": float(np.linalg.norm(sa[k] - sb[k]) / max(np.linalg.norm(sa[k]), 1e-300)) for k in f}
    ia, ib = a.interactions(), b.interactions()
    A = set(zip(ia["first"][ia["active"] == 1].tolist(), ia["second"][ia["active"] == 1].tolist()))
    B = set(zip(ib["first"][ib["active"] == 1].tolist(), ib["second"][ib["active"] == 1].tolist()))
    out["contact_set_identical"] = A == B
    out["contacts"] = len(A)
    a.run(post_steps)
    b.run(post_steps)
    oa, ob = a.observables(), b.observables()
    ea, eb = oa[0] + oa[1] + oa[2], ob[0] + ob[1] + ob[2]
    out[f"energy_rel_after_{post_steps}_steps"] = abs(ea - eb) / max(abs(ea), 1e-300)
    out["from_step"] = pre_steps
    a.close()
    b.close()
    return out


def batch_workload(args, dist, dev):
    """The batched workload: hopper scenes of 1e3..5e4 spheres in one autotuned engine whose
    check intervals replay as CUDA graphs (one fused tick launch per step over all scenes).
    On N GPUs the same scenes are placed whole on the GPUs (vedo_gb300.partition.pack_scenes,
    by spheres x steps): a fixed job, so its scaling is strong."""
    import torch
    from vedo_gb300 import partition, scenes
    from vedo_gb300.engine import BatchEngine
    hs = scenes.hopper_batch(args.batch_scenes, seed=2025, steps=5000)
    weights = [scene_particles(h) * 5000 for h in hs]
    mine = partition.pack_scenes(weights, dist.world)[dist.rank]
    hs = [hs[q] for q in mine]
    n = sum(scene_particles(h) for h in hs)
    # errors against the FP64 engine on four of the scenes (a scene's results in the batch are
    # those of the scene alone, bit for bit), from step 1000 of the run
    errs = [] if args.no_profile_pass else [form_errors(hs[q], dev, 1000) for q in range(min(4, len(hs)))]
    b = BatchEngine(hs, device=dev, autotune=True)
    del hs
    b.run(TUNE_STEPS)                # autotuning + warm-up; the tuned settings stay
    dist.barrier()
    torch.cuda.synchronize()
    b.run(args.batch_steps)
    prof = b.last_run_profile()
    t = dist.reduce(prof["total_ms"], "max")
    total = dist.reduce(float(n), "sum")
    contacts = int(b.observables()[9])
    tune = b.tuning()
    # the same window with the check intervals in the other schedule (a replayed graph of per-step
    # kernels, or one persistent cooperative launch): the tuned settings otherwise, fresh engine
    other = None
    if not args.no_profile_pass:
        hs2 = [scenes.hopper_batch(args.batch_scenes, seed=2025, steps=5000)[q] for q in mine]
        b2 = BatchEngine(hs2, device=dev, skin=tune["skin"], cell_scale=tune["cell_scale"],
                         tick_block=tune["tick_block"], stored_splits=tune["stored_splits"],
                         split_tick=tune["split_tick"], pair_pass=tune["pair_pass"],
                         persistent=not tune["persistent"])
        del hs2
        b2.run(TUNE_STEPS)
        torch.cuda.synchronize()
        b2.run(args.batch_steps)
        p2 = b2.last_run_profile()
        other = {"persistent": b2.tuning()["persistent"], "ms_per_step": p2["total_ms"] / args.batch_steps,
                 "gpu_launches": p2["launches"]}
        b2.close()
    out = {"workload": f"hopper_batch_{args.batch_scenes}", "scenes": args.batch_scenes, "particles": int(total),
           "scaling": "strong" if dist.world > 1 else None,
           "placement": {"scenes_per_rank": [len(p) for p in dist.gather(mine)],
                         "particles_per_rank": dist.gather(n), "rule": "longest first to the least-loaded GPU"},
           "active_contacts_end": contacts, "z_pp": contacts / n,
           "value": total * args.batch_steps / (t * 1e-3), "unit": UNIT, "ms_per_step": t / args.batch_steps,
           "steps": args.batch_steps, "gpu_launches": prof["launches"], "tuning": tune,
           "other_schedule": other,
           "errors_mixed_vs_fp64": {"scenes": errs,
                                    "max_step_impact_rel_l2": max((e["step_impact_rel_l2"] for e in errs), default=None),
                                    "all_contact_sets_identical": all(e["contact_set_identical"] for e in errs),
                                    "max_energy_rel": max((e["energy_rel_after_200_steps"] for e in errs),
                                                          default=None)},
           "note": f"steps {TUNE_STEPS}..{TUNE_STEPS + args.batch_steps} of the configured 5000-step run, columns "
                   "resting on touching lattices and draining through the orifice; mixed form, CUDA-graph check "
                   "intervals, autotuned tick block, skin and cell scale; errors on the first four scenes of the GPU's share alone "
                   "(bit-identical to their batch slices)"}
    b.close()
    return out


def bed_workload(args, dist, dev):
    """The large single domain: a compressed Hertz bed (16M spheres by default, 32 rods,
    orbital top plate), mixed form, autotuned; tick-kernel roofline from per-launch events."""
    import torch
    from vedo_gb300 import scenes
    from vedo_gb300.engine import GpuEngine
    errs = None
    if not args.no_profile_pass:
        small = scenes.compressed_bed(n=1_000_000, box=0.1, cylinders=2, seed=5 + dist.rank)
        errs = form_errors(small, dev, 1500)          # the top plate reaches the bed near step 1000
        errs["scene"] = "compressed_bed of 1M spheres (same construction; 0.1 x 0.1 m floor, 2 rods)"
        del small
    sc = scenes.compressed_bed(n=args.bed_n, seed=5 + dist.rank)
    n = scene_particles(sc)
    e = GpuEngine(sc, device=dev, precision=1, autotune=True)
    del sc
    e.run(TUNE_STEPS)                # autotuning + warm-up
    dist.barrier()
    torch.cuda.synchronize()
    e.run(args.bed_steps)
    prof = e.last_run_profile()
    t = dist.reduce(prof["total_ms"], "max")
    e.set_profiling(True)
    e.run(args.profile_steps)
    kp = e.last_run_profile()
    e.set_profiling(False)
    it = e.interactions()
    z = float(it["active"].sum()) / n
    b_alg = 2 * 72 + z * (2 * 16 + 8)              # monodisperse: no per-particle radius
    t_tick = kp["pair_ms"] / args.profile_steps
    peak, _ = peaks()
    ach = b_alg * n / (t_tick * 1e-3) / 1e9
    # a committed capture of the pair-pass tick at this size, when there is one
    traffic = ncu_traffic("k_tick_bed16M_dram.md") if args.bed_n == 16_000_000 else None
    total = dist.reduce(float(n), "sum")
    out = {"workload": f"compressed_bed_{args.bed_n // 1_000_000}M", "particles": n,
           "value": total * args.bed_steps / (t * 1e-3), "unit": UNIT, "ms_per_step": t / args.bed_steps,
           "steps": args.bed_steps, "gpu_launches": prof["launches"], "tuning": e.tuning(), "z_pp": z,
           "errors_mixed_vs_fp64": errs,
           "tick_roofline": {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "tick_ms": t_tick,
                             "alg_bytes_per_particle_step": b_alg, "traffic": traffic,
                             "dram_frac": traffic / (t_tick * 1e-3) / 1e9 / peak if traffic else None,
                             "traffic_source": "profiles/k_tick_bed16M_dram.md" if traffic else None},
           "note": f"steps {TUNE_STEPS}..{TUNE_STEPS + args.bed_steps} of the configured 2000-step run (dt 2e-7 s); "
                   "a simple cubic lattice whose neighbours, floor, walls and top plate touch (solid fraction 0.524, "
                   "standing in for a random loose packing at 0.55); mixed form"}
    e.close()
    return out


def dense_workload(args, dist, dev):
    """Contact-dense stress case (FCC lattice in contact, ~6 contacts per sphere): both forms'
    throughput, the mixed form's per-step impulse error from identical state, its energy after
    200 steps against the FP64 form's, and the tick-kernel roofline with contacts present."""
    import numpy as np
    import torch
    from vedo_gb300 import scenes
    from vedo_gb300.engine import GpuEngine
    sc = scenes.dense_pack(n=args.dense_n, seed=9 + dist.rank)
    n = scene_particles(sc)
    f = "impact", "angular_impact"
    a = GpuEngine(sc, up_iact=20, device=dev)
    b = GpuEngine(sc, device=dev, precision=1)
    a.run(1)
    b.run(1)
    sa, sb = a.state(f), b.state(f)
    err = {k: float(np.linalg.norm(sa[k] - sb[k]) / max(np.linalg.norm(sa[k]), 1e-300)) for k in f}
    ia, ib = a.interactions(), b.interactions()
    A = set(zip(ia["first"][ia["active"] == 1].tolist(), ia["second"][ia["active"] == 1].tolist()))
    B = set(zip(ib["first"][ib["active"] == 1].tolist(), ib["second"][ib["active"] == 1].tolist()))
    z = len(A) / n
    a.run(199)
    b.run(199)
    oa, ob = a.observables(), b.observables()
    ea, eb = oa[0] + oa[1] + oa[2], ob[0] + ob[1] + ob[2]
    # timing: FP64 form over the next steps, mixed form after tuning
    a.run(args.warmup)
    torch.cuda.synchronize()
    a.run(args.steps)
    t64 = dist.reduce(a.last_run_profile()["total_ms"], "max")
    a.close()
    b.close()
    e = GpuEngine(sc, device=dev, precision=1, autotune=True)
    del sc
    e.run(TUNE_STEPS)
    e.run(args.warmup)
    dist.barrier()
    torch.cuda.synchronize()
    e.run(args.steps)
    prof = e.last_run_profile()
    t = dist.reduce(prof["total_ms"], "max")
    e.set_profiling(True)
    e.run(args.profile_steps)
    kp = e.last_run_profile()
    e.set_profiling(False)
    tune = e.tuning()
    e.close()
    total = dist.reduce(float(n), "sum")
    b_alg = 2 * 72 + z * (2 * 16 + 8)                # monodisperse: no per-particle radius
    t_tick = kp["pair_ms"] / args.profile_steps
    peak, _ = peaks()
    ach = b_alg * n / (t_tick * 1e-3) / 1e9
    mixed = total * args.steps / (t * 1e-3)
    fp64 = total * args.steps / (t64 * 1e-3)
    return {"workload": f"dense_fcc_{args.dense_n // 1000}k", "particles": n, "z_pp": z,
            "value": mixed, "unit": UNIT, "ms_per_step": t / args.steps, "fp64_value": fp64,
            "fp64_ms_per_step": t64 / args.steps, "mixed_over_fp64": mixed / fp64, "tuning": tune,
            "errors_mixed_vs_fp64": {"step_impact_rel_l2": err["impact"],
                                     "step_angular_impact_rel_l2": err["angular_impact"],
                                     "contact_set_identical": A == B, "contacts": len(A),
                                     "energy_rel_after_200_steps": abs(ea - eb) / max(abs(ea), 1e-300)},
            "tick_roofline": {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "tick_ms": t_tick,
                              "alg_bytes_per_particle_step": b_alg},
            "note": "FCC lattice with neighbours overlapping by 1e-6 of the diameter (every pair in contact from "
                    "step 0), ISwH E 70 GPa, dt 5e-7; per-step impulse error from identical state after one step"}


def serving_workload(args, dist, dev):
    """The serving stream: Poisson arrivals at 200 jobs/s for `--serve-duration` s, sphere
    counts 2e3..2e5, step counts 1e3..2e4 (x `--serve-steps-scale`).  Served by the
    continuous-batching server (mixed form), latency = completion - submission, over every job
    including the drain after the last arrival.  On N GPUs one server per GPU takes the jobs
    that vedo_gb300.partition.dispatch_stream hands it (in arrival order, to the GPU with the
    least spheres x steps so far); latencies are pooled over all GPUs.  For comparison the
    first `--serve-fp64-jobs` jobs of the stream run one at a time on the plain FP64 engine with
    the same arrival times, on rank 0 (the whole stream would take minutes in that form)."""
    from vedo_gb300 import partition, serve
    from vedo_gb300.engine import GpuEngine
    sl, sh = max(1, int(1000 * args.serve_steps_scale)), max(2, int(20000 * args.serve_steps_scale))
    whole = serve.job_stream(rate=200.0, duration=args.serve_duration, seed=4242, steps_lo=sl, steps_hi=sh)
    if not whole:
        return None
    last_arrival = whole[-1][0]
    ranks = partition.dispatch_stream([n * st for (_, _, n, st, _, _) in whole], dist.world)
    mine = [q for q, r in enumerate(ranks) if r == dist.rank]
    stream = [whole[q] for q in mine]
    built = [serve.job_scene(k, n, m, sd, st) for (_, k, n, st, m, sd) in stream]
    offered = dist.reduce(float(sum(scene_particles(sc) * st for sc, (_, _, _, st, _, _) in zip(built, stream))),
                          "sum") / max(last_arrival, 1e-9)
    dist.barrier()
    with serve.Server(hbm_budget_bytes=150 * 10**9, device=dev) as srv:
        r = serve.serve_stream(srv, stream, built) if stream else None
        batches = srv.stats()["batches"]
    # the same jobs again, shortest work first with the live jobs capped at 2M spheres
    dist.barrier()
    with serve.Server(hbm_budget_bytes=150 * 10**9, device=dev, order="shortest",
                      max_live_spheres=args.serve_cap) as srv:
        r_sf = serve.serve_stream(srv, stream, built) if stream else None
    del built
    lat_sf = {}
    for part in dist.gather({q: i["done_s"] - i["submit_s"] for q, i in zip(mine, r_sf["infos"] if r_sf else [])
                             if i["status"] == "done"}):
        lat_sf.update(part)
    wall_sf = dist.reduce(r_sf["wall_s"] if r_sf else 0.0, "max")
    served_sf = dist.reduce(float(r_sf["particle_steps"]) if r_sf else 0.0, "sum")
    lat = {}
    for part in dist.gather({q: i["done_s"] - i["submit_s"] for q, i in zip(mine, r["infos"] if r else [])
                             if i["status"] == "done"}):
        lat.update(part)
    wall = dist.reduce(r["wall_s"] if r else 0.0, "max")
    served = dist.reduce(float(r["particle_steps"]) if r else 0.0, "sum")
    batches = int(dist.reduce(float(batches), "sum"))
    jobs_per_rank = dist.gather(len(stream))
    if dist.rank != 0:
        return None
    pooled = serve.latency_percentiles(list(lat.values()))
    pooled_sf = serve.latency_percentiles(list(lat_sf.values())) if lat_sf else {}
    # the first jobs of the same stream one at a time on the FP64 engine
    k64 = min(args.serve_fp64_jobs, len(whole))
    t_free, lat64, busy, ps64 = 0.0, [], 0.0, 0
    for ta, k, n, steps, m, sd in whole[:k64]:
        sc = serve.job_scene(k, n, m, sd, steps)
        t0 = time.perf_counter()
        e = GpuEngine(sc, up_iact=20, device=dev)
        e.run(steps)
        e.close()
        d = time.perf_counter() - t0
        busy += d
        start = max(ta, t_free)
        t_free = start + d
        lat64.append(t_free - ta)
        ps64 += scene_particles(sc) * steps
    p64 = serve.latency_percentiles(lat64)
    same = [lat[q] for q in range(k64) if q in lat]
    pm = serve.latency_percentiles(same) if same else {}
    return {"workload": f"serving stream, 200 jobs/s x {args.serve_duration} s ({len(whole)} jobs), "
                        f"steps {sl}..{sh} (x{args.serve_steps_scale:g} of 1e3..2e4), 2e3..2e5 spheres",
            "p50_ms": pooled["p50_ms"], "p99_ms": pooled["p99_ms"], "mean_ms": pooled["mean_ms"],
            "jobs_done": len(lat), "jobs": len(whole), "served_particle_steps_per_s": served / max(wall, 1e-9),
            "offered_particle_steps_per_s": offered, "wall_s": wall,
            "last_arrival_s": last_arrival, "drain_s": wall - last_arrival,
            "batches_built": batches, "hbm_budget_gb_per_gpu": 150, "jobs_per_gpu": jobs_per_rank,
            "policy": "arrival order, admitted against the HBM budget alone",
            "shortest_first": {"p50_ms": pooled_sf.get("p50_ms"), "p99_ms": pooled_sf.get("p99_ms"),
                               "mean_ms": pooled_sf.get("mean_ms"), "jobs_done": len(lat_sf),
                               "served_particle_steps_per_s": served_sf / max(wall_sf, 1e-9), "wall_s": wall_sf,
                               "policy": f"shortest work (spheres x steps) first, live jobs capped at "
                                         f"{args.serve_cap} spheres"},
            "fp64_one_at_a_time": {"jobs": k64, "p50_ms": p64["p50_ms"], "p99_ms": p64["p99_ms"],
                                   "particle_steps_per_s": ps64 / max(busy, 1e-9), "busy_s": busy,
                                   "mixed_server_same_jobs_p50_ms": pm.get("p50_ms"),
                                   "mixed_server_same_jobs_p99_ms": pm.get("p99_ms"),
                                   "note": "the first jobs of the stream, same arrival times, one at a time"}}


def main():
    args = parse()
    if args.cpu_job:
        cpu_job(args)
        return
    dist = Dist()
    try:
        if args.impl == "reference":
            reference_arm(args, dist)
        else:
            ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
