"""GPU tests of the job server (vedo_srv_*): continuous batching of DEM jobs.

Bar: a job's result through the server equals the same scene run alone in the MIXED form for
the same steps, bit for bit, although the job joins a batch that is already running, other
jobs join and leave while it runs, and the batch is rebuilt each time."""
import time

import numpy as np
import pytest

from vedo_gb300 import scenes

pytestmark = pytest.mark.gpu

FIELDS = ("position", "velocity", "angular_velocity", "impact", "angular_impact")


def _alone(engine_lib, sc, steps):
    e = engine_lib.GpuEngine(sc, precision=1)
    e.run(steps)
    st = e.state(FIELDS)
    e.close()
    return st


def _wait_running(srv, job, min_steps=1, timeout=60.0):
    t0 = time.time()
    while time.time() - t0 < timeout:
        i = srv.poll(job)
        if i["status"] != "queued" and i["steps_done"] >= min_steps:
            return i
        time.sleep(0.001)
    raise AssertionError("job did not start")


def test_served_jobs_equal_alone(engine_lib):
    from vedo_gb300.serve import Server
    jobs = [(scenes.hopper(n=3000, seed=1, steps=10), 400),
            (scenes.serving_job("projectile", 2500, "lsd", 3), 250),
            (scenes.serving_job("settle", 2000, "hertz", 4), 333),
            (scenes.cluster(n=64, solver="ISwBSDBF", seed=21), 150)]
    with Server(hbm_budget_bytes=8 * 10**9) as srv:
        ids = [srv.submit(*jobs[0])]
        _wait_running(srv, ids[0], 20)            # the others join a running batch
        for sc, st in jobs[1:]:
            ids.append(srv.submit(sc, st))
            time.sleep(0.002)
        infos = [srv.wait(j, 120.0) for j in ids]
        assert all(i["status"] == "done" for i in infos), infos
        assert all(i["steps_done"] == st for i, (_, st) in zip(infos, jobs))
        res = [srv.result(j, FIELDS) for j in ids]
        stats = srv.stats()
    assert stats["jobs_done"] == len(jobs) and stats["batches"] >= 2
    for (sc, st), r in zip(jobs, res):
        ref = _alone(engine_lib, sc, st)
        for k in FIELDS:
            assert np.array_equal(r[k], ref[k]), k


def test_shortest_first_with_a_live_cap(engine_lib):
    """Shortest-work-first admission under a live-sphere cap: with a long job running, a short
    job submitted after a second long one is admitted before it (and finishes first), the cap
    holds the second long job back while the first runs, and every result still equals its scene
    alone."""
    from vedo_gb300.serve import Server
    long1 = (scenes.serving_job("settle", 3000, "lsd", 5), 3000)
    long2 = (scenes.serving_job("settle", 3000, "lsd", 6), 3000)
    short = (scenes.serving_job("projectile", 2000, "lsd", 7), 100)
    n1 = long1[0].num_objects
    with Server(hbm_budget_bytes=8 * 10**9, order="shortest", max_live_spheres=n1 + short[0].num_objects) as srv:
        a = srv.submit(*long1)
        _wait_running(srv, a, 1)
        b = srv.submit(*long2)
        c = srv.submit(*short)
        ib, ic = srv.wait(b, 120.0), srv.wait(c, 120.0)
        ia = srv.wait(a, 120.0)
        res = {j: srv.result(j, FIELDS) for j in (a, b, c)}
    assert all(i["status"] == "done" for i in (ia, ib, ic))
    assert ic["admit_s"] < ib["admit_s"] and ic["done_s"] < ib["done_s"]
    assert ib["admit_s"] >= ia["done_s"] - 1e-6        # the cap: the second long job waits for the first
    for j, (sc, st) in zip((a, b, c), (long1, long2, short)):
        ref = _alone(engine_lib, sc, st)
        for k in FIELDS:
            assert np.array_equal(res[j][k], ref[k]), k


def test_admission_respects_the_hbm_budget(engine_lib):
    from vedo_gb300.serve import Server, job_charge
    scs = [scenes.serving_job("settle", 2000, "lsd", s) for s in range(3)]
    one = max(job_charge(sc.num_objects, 2000) for sc in scs)
    with Server(hbm_budget_bytes=3 * one) as srv:      # half the budget holds one job, not two
        ids = [srv.submit(sc, 200) for sc in scs]
        infos = [srv.wait(j, 120.0) for j in ids]
        res = [srv.result(j, ("position",)) for j in ids]
    assert all(i["status"] == "done" for i in infos)
    for a, b in zip(infos, infos[1:]):
        assert b["admit_s"] >= a["done_s"]            # one at a time
    for sc, r in zip(scs, res):
        assert np.array_equal(r["position"], _alone(engine_lib, sc, 200)["position"])


def test_cancel_and_oversized_jobs(engine_lib):
    from vedo_gb300.serve import Server
    with Server(hbm_budget_bytes=2 * 10**8) as srv:
        big = scenes.serving_job("settle", 60000, "lsd", 1)
        with pytest.raises(engine_lib.EngineError) as ex:
            srv.submit(big, 10)                       # 60k spheres' charge > half of 200 MB
        assert ex.value.code == 4
        j = srv.submit(scenes.serving_job("settle", 3000, "lsd", 2), 10**6)
        _wait_running(srv, j, 1)
        srv.cancel(j)
        assert srv.wait(j, 60.0)["status"] == "cancelled"
        k = srv.submit(scenes.cluster(n=64, seed=3), 50)
        assert srv.wait(k, 60.0)["status"] == "done"


@pytest.mark.parametrize("which", ["projectile", "dense"])
@pytest.mark.parametrize("pair_pass", [False, True])
def test_admission_charge_covers_the_engine_allocations(which, pair_pass, engine_lib):
    """The charge a job is admitted against (objects and expected neighbour-list entries, plus
    the pair pass's per-entry buffers when the server may run it) is at least the device memory
    a MIXED engine of that scene allocates once its list is built and has been rebuilt (two
    lists alive), here measured as the drop in the device's free memory; the dense pack (12
    neighbours per sphere in contact) is the list's worst case."""
    torch = pytest.importorskip("torch")
    from vedo_gb300.scene import SPHERE
    from vedo_gb300.serve import Server, job_charge
    sc = scenes.serving_job("projectile", 40000, "hertz", 3) if which == "projectile" else scenes.dense_pack(n=40000)
    nsph = int(sum(1 for m in sc.model_index if sc.models[m].shape == SPHERE))
    charge = job_charge(sc.num_objects, nsph, pair_pass=pair_pass)
    with Server(hbm_budget_bytes=10**10, pair_pass=pair_pass) as srv:    # the server reports the same charge
        j = srv.submit(sc, 1)
        assert srv.wait(j, 120.0)["charged_bytes"] == charge
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    e = engine_lib.GpuEngine(sc, precision=1, skin=0.4, pair_pass=pair_pass)
    e.run(200)
    e.set_state(position=e.state(("position",))["position"] + 1.0)   # a jump past the skin: a rebuild
    e.run(5)
    torch.cuda.synchronize()
    used = free0 - torch.cuda.mem_get_info()[0]
    e.close()
    assert 0 < used <= charge, (used, charge)
