// serve.cpp - continuous batching of DEM jobs on one GPU (the vedo_srv_* entry points).
//
// One server thread owns the device.  It advances the current batch (a MIXED-form engine
// whose scenes are the live jobs) one check interval at a time, never past the step count of
// the job that finishes first.  A finished job's scene is frozen in place, its final state is
// copied to the host and its memory is released from the budget.  Whenever jobs are admitted
// from the queue, or frozen scenes hold a quarter of the batch, the server builds the next
// batch: the live scenes move over on the device with their contact histories
// (mixed_repack), the admitted jobs are uploaded, and the old batch is freed.  Each scene's
// arithmetic does not depend on the other scenes, on where it sits in the batch, or on when
// the batch is rebuilt, so a job's result is the one it gets when run alone.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/vedo_gpu.h"
#include "engine_base.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    uint64_t id = 0;
    vedo::HScene scene;               // emptied once the scene is on the device
    uint32_t num_objects = 0;
    uint64_t particles = 0;           // spheres (local-scope objects)
    uint64_t steps = 0;
    uint64_t steps_done = 0;
    uint64_t bytes = 0;
    uint32_t status = VEDO_JOB_QUEUED;
    bool cancel = false;
    double t_submit = -1.0, t_admit = -1.0, t_done = -1.0;
    std::vector<double> result[7];
    std::string error;
};

}  // namespace

struct vedo_server {
    vedo_engine_opts opts{};
    uint64_t budget = 0;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::map<uint64_t, std::unique_ptr<Job>> jobs;
    std::deque<uint64_t> queue;
    uint64_t next_id = 1;
    uint64_t committed = 0;
    uint32_t order = VEDO_SRV_FIFO;   // admission order (vedo_srv_set_policy)
    uint64_t max_live = 0;            // cap on the live jobs' spheres (0: none)
    uint64_t live_spheres = 0;        // spheres of the admitted, unfinished jobs
    bool stop = false;
    std::thread th;
    std::string err;
    // owned by the server thread
    vedo::EngineBase* eng = nullptr;
    std::vector<Job*> live;           // the job of each scene of the batch; nullptr = frozen
    uint32_t eng_objects = 0;
    // statistics (under mu)
    double jobs_done = 0, ps_done = 0, busy_s = 0, batches = 0;
    uint32_t running = 0;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    void loop();
    void fail_live(const std::string& msg);
    bool rebatch(std::vector<Job*>& admit);
};

void vedo_server::fail_live(const std::string& msg) {
    std::lock_guard<std::mutex> lk(mu);
    for (Job*& j : live) {
        if (!j) continue;
        j->status = VEDO_JOB_FAILED;
        j->error = msg;
        j->t_done = now();
        committed -= j->bytes;
        live_spheres -= j->particles;
        --running;
        j = nullptr;
    }
    err = msg;
    cv_done.notify_all();
}


// The next batch: live scenes of the current one (moved on the device) + admitted jobs.
bool vedo_server::rebatch(std::vector<Job*>& admit) {
    std::vector<uint32_t> keep;
    std::vector<Job*> next;
    for (uint32_t s = 0; s < live.size(); ++s)
        if (live[s]) {
            keep.push_back(s);
            next.push_back(live[s]);
        }
    std::vector<const vedo::HScene*> add;
    for (Job* j : admit) {
        add.push_back(&j->scene);
        next.push_back(j);
    }
    if (next.empty()) {
        delete eng;
        eng = nullptr;
        live.clear();
        std::lock_guard<std::mutex> lk(mu);
        eng_objects = 0;
        return true;
    }
    int rc = VEDO_OK;
    std::string msg;
    vedo::EngineBase* ne = vedo::mixed_repack(eng, keep, add, opts, &rc, &msg);
    if (!ne) {
        std::lock_guard<std::mutex> lk(mu);
        for (Job* j : admit) {
            j->status = VEDO_JOB_FAILED;
            j->error = "admission failed: " + msg;
            j->t_done = now();
            committed -= j->bytes;
            --running;
        }
        err = msg;
        cv_done.notify_all();
        admit.clear();
        return false;
    }
    delete eng;
    eng = ne;
    live = next;
    for (Job* j : admit) j->scene = vedo::HScene();   // the engine holds its own copy
    std::lock_guard<std::mutex> lk(mu);
    eng_objects = eng->num_objects();
    batches += 1;
    return true;
}

void vedo_server::loop() {
    cudaSetDevice(opts.device);
    for (;;) {
        std::vector<Job*> admit;
        bool compact = false;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return stop || running > 0 || !queue.empty(); });
            if (stop) break;
            // cancelled running jobs leave the batch like finished ones
            for (uint32_t s = 0; s < live.size(); ++s) {
                Job* j = live[s];
                if (!j || !j->cancel) continue;
                lk.unlock();
                vedo::mixed_set_scene_active(eng, s, false);
                lk.lock();
                j->status = VEDO_JOB_CANCELLED;
                j->t_done = now();
                committed -= j->bytes;
                live_spheres -= j->particles;
                --running;
                live[s] = nullptr;
                cv_done.notify_all();
            }
            // admission against half the budget (the next batch is built beside the current one) and
            // the live-sphere cap, in arrival order or shortest work (spheres x steps) first; a job
            // alone larger than the cap is admitted when nothing else runs
            for (;;) {
                while (!queue.empty() && jobs[queue.front()]->status != VEDO_JOB_QUEUED) queue.pop_front();
                if (queue.empty()) break;
                size_t pick = 0;
                if (order == VEDO_SRV_SHORTEST_FIRST) {
                    double best = -1.0;
                    for (size_t q = 0; q < queue.size(); ++q) {
                        const Job* c = jobs[queue[q]].get();
                        if (c->status != VEDO_JOB_QUEUED) continue;
                        const double w = (double)c->particles * (double)c->steps;
                        if (best < 0.0 || w < best) {
                            best = w;
                            pick = q;
                        }
                    }
                }
                Job* j = jobs[queue[pick]].get();
                if (committed + j->bytes > budget / 2) break;
                if (max_live && running > 0 && live_spheres + j->particles > max_live) break;
                committed += j->bytes;
                live_spheres += j->particles;
                j->status = VEDO_JOB_RUNNING;
                j->t_admit = now();
                ++running;
                admit.push_back(j);
                queue.erase(queue.begin() + (std::ptrdiff_t)pick);
            }
        }
        uint64_t frozen = 0;
        for (uint32_t s = 0; s < live.size(); ++s)
            if (!live[s]) {
                uint32_t off = 0, n = 0;
                double t = 0;
                if (vedo::mixed_scene_range(eng, s, &off, &n, &t) == VEDO_OK) frozen += n;
            }
        bool any_live = false;
        for (Job* j : live) any_live = any_live || j;
        compact = frozen > 0 && (4 * frozen > eng_objects || !any_live);
        if (!admit.empty() || compact) rebatch(admit);
        if (!eng) continue;
        // advance to the next check interval, or to the first job's last step
        uint64_t chunk = opts.check_interval ? opts.check_interval : 10;
        for (Job* j : live)
            if (j) chunk = std::min<uint64_t>(chunk, j->steps - j->steps_done);
        if (chunk == 0) chunk = 1;
        const auto c0 = Clock::now();
        int keep = 0;
        const int rc = eng->run((uint32_t)chunk, &keep);
        const double dt_run = std::chrono::duration<double>(Clock::now() - c0).count();
        if (rc != VEDO_OK) {
            fail_live(std::string("batch step failed: ") + eng->error());
            delete eng;
            eng = nullptr;
            live.clear();
            std::lock_guard<std::mutex> lk(mu);
            eng_objects = 0;
            continue;
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            busy_s += dt_run;
        }
        for (uint32_t s = 0; s < live.size(); ++s) {
            Job* j = live[s];
            if (!j) continue;
            const uint64_t done = vedo::mixed_scene_steps(eng, s);
            {
                std::lock_guard<std::mutex> lk(mu);
                j->steps_done = done;
            }
            if (done < j->steps) continue;
            vedo::mixed_set_scene_active(eng, s, false);
            uint32_t off = 0, n = 0;
            double t = 0;
            vedo::mixed_scene_range(eng, s, &off, &n, &t);
            for (auto& r : j->result) r.assign(3 * (size_t)n, 0.0);
            vedo_state_view v{j->result[0].data(), j->result[1].data(), j->result[2].data(), j->result[3].data(),
                              j->result[4].data(), j->result[5].data(), j->result[6].data()};
            const int grc = vedo::mixed_get_state_slice(eng, off, n, v);
            std::lock_guard<std::mutex> lk(mu);
            j->status = grc == VEDO_OK ? VEDO_JOB_DONE : VEDO_JOB_FAILED;
            if (grc != VEDO_OK) j->error = eng->error();
            j->t_done = now();
            committed -= j->bytes;
            live_spheres -= j->particles;
            --running;
            jobs_done += 1;
            ps_done += (double)j->particles * (double)j->steps;
            live[s] = nullptr;
            cv_done.notify_all();
        }
        bool left = false;
        for (Job* j : live) left = left || j;
        if (!left) {                  // idle: free the batch before waiting for work
            std::vector<Job*> none;
            rebatch(none);
        }
    }
    delete eng;
    eng = nullptr;
}

namespace {
thread_local std::string g_srv_error;

void info_of(const Job& j, vedo_job_info* info) {
    info->status = j.status;
    info->num_objects = j.num_objects;
    info->steps = j.steps;
    info->steps_done = j.steps_done;
    info->submit_s = j.t_submit;
    info->admit_s = j.t_admit;
    info->done_s = j.t_done;
    info->charged_bytes = j.bytes;
}
}  // namespace

extern "C" {

int vedo_srv_create(const vedo_engine_opts* opts, uint64_t hbm_budget_bytes, vedo_server** out) {
    if (!out) return VEDO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    vedo_engine_opts o;
    vedo_gpu_default_opts(&o);
    o.precision = VEDO_PRECISION_MIXED;
    if (opts) o = *opts;
    if (o.precision != VEDO_PRECISION_MIXED) {
        g_srv_error = "the server batches jobs in the MIXED form only";
        return VEDO_ERR_INVALID_ARGUMENT;
    }
    if (hbm_budget_bytes == 0) {
        g_srv_error = "zero HBM budget";
        return VEDO_ERR_INVALID_ARGUMENT;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || o.device < 0 || o.device >= ndev) {
        g_srv_error = "no such CUDA device";
        return VEDO_ERR_CUDA;
    }
    vedo_server* s = new (std::nothrow) vedo_server();
    if (!s) return VEDO_ERR_OUT_OF_MEMORY;
    s->opts = o;
    s->opts.output_prefix = nullptr;      // jobs write no files
    s->opts.record = 0;
    s->budget = hbm_budget_bytes;
    s->t0 = Clock::now();
    s->th = std::thread([s] { s->loop(); });
    *out = s;
    return VEDO_OK;
}

int vedo_srv_set_policy(vedo_server* s, uint32_t order, uint64_t max_live_spheres) {
    if (!s || (order != VEDO_SRV_FIFO && order != VEDO_SRV_SHORTEST_FIRST)) return VEDO_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->order = order;
        s->max_live = max_live_spheres;
    }
    s->cv_work.notify_all();
    return VEDO_OK;
}

int vedo_srv_submit(vedo_server* s, const vedo_scene_desc* scene, uint64_t steps, uint64_t* job_id) {
    if (!s || !scene || !job_id || steps == 0) return VEDO_ERR_INVALID_ARGUMENT;
    auto j = std::make_unique<Job>();
    std::string err;
    if (!vedo::scene_from_desc(scene, j->scene, err)) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->err = err;
        return VEDO_ERR_INVALID_SCENE;
    }
    vedo::prepare_scene(j->scene);
    j->num_objects = j->scene.n;
    for (uint32_t i = 0; i < j->scene.n; ++i) {
        const uint32_t m = j->scene.model_of[i];
        if (m < j->scene.models.size() && j->scene.models[m].scope == VEDO_SCOPE_LOCAL) ++j->particles;
    }
    j->steps = steps;
    // an engine that may run the pair pass (asked for, or open to the autotuner) also holds its
    // per-entry worklist, marks and pair records
    const uint64_t per_entry = VEDO_SRV_BYTES_PER_ENTRY +
                               ((s->opts.split_tick == 2 || s->opts.autotune) ? VEDO_SRV_BYTES_PER_ENTRY_PAIR_PASS : 0u);
    j->bytes = (uint64_t)VEDO_SRV_BYTES_PER_OBJECT * j->scene.n +
               (uint64_t)VEDO_SRV_ENTRIES_PER_SPHERE * per_entry * j->particles;
    std::lock_guard<std::mutex> lk(s->mu);
    if (j->bytes > s->budget / 2) {
        s->err = "job needs " + std::to_string(j->bytes) + " bytes, more than half the HBM budget";
        return VEDO_ERR_OUT_OF_MEMORY;
    }
    j->id = s->next_id++;
    j->t_submit = s->now();
    *job_id = j->id;
    s->queue.push_back(j->id);
    s->jobs[j->id] = std::move(j);
    s->cv_work.notify_all();
    return VEDO_OK;
}

int vedo_srv_poll(vedo_server* s, uint64_t job_id, vedo_job_info* info) {
    if (!s || !info) return VEDO_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return VEDO_ERR_INVALID_ARGUMENT;
    info_of(*it->second, info);
    return VEDO_OK;
}

int vedo_srv_wait(vedo_server* s, uint64_t job_id, double timeout_s, vedo_job_info* info) {
    if (!s) return VEDO_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return VEDO_ERR_INVALID_ARGUMENT;
    Job* j = it->second.get();
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
        return j->status == VEDO_JOB_DONE || j->status == VEDO_JOB_CANCELLED || j->status == VEDO_JOB_FAILED;
    });
    if (info) info_of(*j, info);
    return ok ? VEDO_OK : VEDO_ERR_DEVICE_TIMEOUT;
}

int vedo_srv_result(vedo_server* s, uint64_t job_id, const vedo_state_view* out) {
    if (!s || !out) return VEDO_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end() || it->second->status != VEDO_JOB_DONE) return VEDO_ERR_INVALID_ARGUMENT;
    const Job& j = *it->second;
    double* dst[7] = {out->position, out->velocity, out->angular_velocity, out->orientation_x, out->orientation_z,
                      out->impact, out->angular_impact};
    for (int k = 0; k < 7; ++k)
        if (dst[k]) std::memcpy(dst[k], j.result[k].data(), 8 * j.result[k].size());
    return VEDO_OK;
}

int vedo_srv_cancel(vedo_server* s, uint64_t job_id) {
    if (!s) return VEDO_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return VEDO_ERR_INVALID_ARGUMENT;
    Job& j = *it->second;
    if (j.status == VEDO_JOB_QUEUED) {
        j.status = VEDO_JOB_CANCELLED;
        j.t_done = s->now();
        s->cv_done.notify_all();
    } else if (j.status == VEDO_JOB_RUNNING) {
        j.cancel = true;
        s->cv_work.notify_all();
    }
    return VEDO_OK;
}

int vedo_srv_stats(vedo_server* s, double out[8]) {
    if (!s || !out) return VEDO_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    uint32_t queued = 0;
    for (uint64_t id : s->queue)
        if (s->jobs[id]->status == VEDO_JOB_QUEUED) ++queued;
    out[0] = s->jobs_done;
    out[1] = s->ps_done;
    out[2] = s->busy_s;
    out[3] = s->batches;
    out[4] = s->eng_objects;
    out[5] = (double)s->committed;
    out[6] = queued;
    out[7] = s->running;
    return VEDO_OK;
}

const char* vedo_srv_last_error(const vedo_server* s) {
    if (!s) return g_srv_error.c_str();
    std::lock_guard<std::mutex> lk(const_cast<vedo_server*>(s)->mu);
    g_srv_error = s->err;          // a copy: the server thread may replace s->err
    return g_srv_error.c_str();
}

void vedo_srv_destroy(vedo_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->th.joinable()) s->th.join();
    delete s;
}

}  // extern "C"
