"""Run one workload of the engine, for a profiler or a quick timing.

    python -m vedo_gb300.profile_case <drum|settled|dense|bed|hopper> <spheres> <steps> [--fp64] [--block B]
                                      [--stored] [--split | --pair] [--skin S] [--persistent]

Builds the seeded scene (`settled`: the polydisperse drum after 300,000 steps of settling, made
once per host by vedo_gb300.workloads.settled_drum and cached there), creates the engine (mixed form unless --fp64; fixed settings, no
autotuning, no graph replay, so that every step is one set of plain launches; --persistent: each
check interval one cooperative launch instead), runs 5 warm-up steps and then <steps> steps, and
prints the device time per step.  Under ncu, skip the warm-up
launches with -s and capture the kernel of interest with -k / -c.
"""
from __future__ import annotations

import argparse
import sys

from . import scenes
from .engine import GpuEngine


def make(kind: str, n: int):
    if kind == "drum":
        return scenes.hertz_drum(n=n)
    if kind == "settled":
        from .workloads import settled_drum
        return settled_drum(n=n)[0]
    if kind == "dense":
        return scenes.dense_pack(n=n)
    if kind == "bed":
        side = 0.4 * (n / 16e6) ** 0.5
        return scenes.compressed_bed(n=n, box=max(side, 0.03), cylinders=max(1, int(32 * n / 16e6)))
    if kind == "hopper":
        return scenes.hopper(n=n)
    raise SystemExit(f"unknown workload {kind!r}")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("kind")
    ap.add_argument("n", type=int)
    ap.add_argument("steps", type=int)
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--block", type=int, default=64)
    ap.add_argument("--stored", action="store_true", help="store the hi/lo position splits once per step")
    ap.add_argument("--split", action="store_true", help="light tick + full tick over the deferred spheres")
    ap.add_argument("--pair", action="store_true", help="pair pass: prefilter pass, one evaluation per pair, sums")
    ap.add_argument("--skin", type=float, default=None, help="candidate-list skin (fraction of r_max)")
    ap.add_argument("--persistent", action="store_true", help="one cooperative launch per check interval")
    a = ap.parse_args(argv)
    sc = make(a.kind, a.n)
    if a.fp64:
        e = GpuEngine(sc, up_iact=20)
    else:
        e = GpuEngine(sc, precision=1, tick_block=a.block, graphs=False, stored_splits=a.stored, split_tick=a.split,
                      pair_pass=a.pair, skin=a.skin, persistent=a.persistent)
    e.run(5)
    e.run(a.steps)
    p = e.last_run_profile()
    print(f"{a.kind} n={a.n}: {p['total_ms'] / a.steps:.4f} ms/step over {a.steps} steps, {p['launches']} launches")
    e.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
