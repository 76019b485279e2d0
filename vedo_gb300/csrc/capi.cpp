// capi.cpp - extern "C" entry points of include/vedo_gpu.h over vedo::Engine.
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/vedo_gpu.h"
#include "coordination.h"
#include "engine_base.h"

struct vedo_gpu_engine {
    vedo::EngineBase* p = nullptr;
    ~vedo_gpu_engine() { delete p; }
};

namespace {
thread_local std::string g_create_error;

int create_common(vedo::HScene& s, const vedo_engine_opts* opts, vedo_gpu_engine** out) {
    vedo::prepare_scene(s);
    vedo_engine_opts o;
    vedo_gpu_default_opts(&o);
    if (opts) o = *opts;
    if (o.precision != VEDO_PRECISION_FP64 && o.precision != VEDO_PRECISION_MIXED) {
        g_create_error = "unknown precision form";
        return VEDO_ERR_INVALID_ARGUMENT;
    }
    vedo_gpu_engine* e = new (std::nothrow) vedo_gpu_engine();
    if (!e) return VEDO_ERR_OUT_OF_MEMORY;
    e->p = o.precision == VEDO_PRECISION_MIXED ? vedo::make_mixed_engine() : vedo::make_fp64_engine();
    if (!e->p) {
        delete e;
        return VEDO_ERR_OUT_OF_MEMORY;
    }
    int rc = e->p->init(s, o);
    if (rc != VEDO_OK) {
        g_create_error = e->p->error();
        delete e;
        *out = nullptr;
        return rc;
    }
    *out = e;
    return VEDO_OK;
}
}  // namespace

namespace vedo {
void set_last_error(const std::string& msg) { g_create_error = msg; }
}  // namespace vedo

extern "C" {

void vedo_gpu_default_opts(vedo_engine_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->up_iact = 1;
    o->record = 0;
    o->precision = VEDO_PRECISION_FP64;
    o->device = 0;
    o->output_prefix = nullptr;
    o->skin = 0.15f;
    o->check_interval = 10;
    o->tick_block = 256;
    o->cell_scale = 1.0f;
    o->autotune = 0;
    o->graphs = 1;
    o->stored_splits = 0;
    o->split_tick = 0;
    o->full_walks = 0;
    o->orientations = 0;
    o->persistent = 0;
}

int vedo_gpu_create(const vedo_scene_desc* scene, const vedo_engine_opts* opts, vedo_gpu_engine** out) {
    if (!scene || !out) return VEDO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    vedo::HScene s;
    std::string err;
    if (!vedo::scene_from_desc(scene, s, err)) {
        g_create_error = err;
        return VEDO_ERR_INVALID_SCENE;
    }
    return create_common(s, opts, out);
}

int vedo_gpu_create_from_ido(const char* path, const vedo_engine_opts* opts, vedo_gpu_engine** out) {
    if (!path || !out) return VEDO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    vedo::HScene s;
    std::string err;
    if (!vedo::read_ido(path, s, err)) {
        g_create_error = err;
        return VEDO_ERR_BAD_IDO;
    }
    return create_common(s, opts, out);
}

int vedo_gpu_create_from_xml(const char* path, const vedo_engine_opts* opts, vedo_gpu_engine** out) {
    if (!path || !out) return VEDO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    vedo::HScene s;
    std::string err;
    if (!vedo::read_xml(path, s, err)) {
        g_create_error = err;
        return VEDO_ERR_INVALID_SCENE;
    }
    return create_common(s, opts, out);
}

int vedo_convert_scene(const char* in_path, const char* out_path) {
    if (!in_path || !out_path) return VEDO_ERR_INVALID_ARGUMENT;
    auto ends = [](const std::string& a, const char* b) {
        const size_t n = std::strlen(b);
        return a.size() >= n && a.compare(a.size() - n, n, b) == 0;
    };
    const std::string in(in_path), out(out_path);
    vedo::HScene s;
    std::string err;
    bool ok;
    if (ends(in, ".ido")) ok = vedo::read_ido(in, s, err);
    else if (ends(in, ".xml")) ok = vedo::read_xml(in, s, err);
    else { g_create_error = "input must be .ido or .xml"; return VEDO_ERR_INVALID_ARGUMENT; }
    if (!ok) {
        g_create_error = err;
        return ends(in, ".ido") ? VEDO_ERR_BAD_IDO : VEDO_ERR_INVALID_SCENE;
    }
    if (ends(out, ".ido")) ok = vedo::write_ido(out, s, err);
    else if (ends(out, ".xml")) ok = vedo::write_xml(out, s, err);
    else if (ends(out, ".vtu")) ok = vedo::write_world_vtk(out, s, s.pos.data(), s.vel.data(), s.av.data(), nullptr, err);
    else { g_create_error = "output must be .ido, .xml or .vtu"; return VEDO_ERR_INVALID_ARGUMENT; }
    if (!ok) {
        g_create_error = err;
        return VEDO_ERR_IO;
    }
    return VEDO_OK;
}

int vedo_gpu_run(vedo_gpu_engine* e, uint32_t nsteps, int* keep_running) {
    if (!e) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->run(nsteps, keep_running);
}

int vedo_gpu_step(vedo_gpu_engine* e, uint32_t nsteps, int* keep_running) { return vedo_gpu_run(e, nsteps, keep_running); }

uint32_t vedo_gpu_num_objects(const vedo_gpu_engine* e) { return e ? e->p->num_objects() : 0u; }

int vedo_gpu_get_state(vedo_gpu_engine* e, const vedo_state_view* out) {
    if (!e || !out) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->get_state(*out);
}

int vedo_gpu_set_state(vedo_gpu_engine* e, const vedo_state_view* in) {
    if (!e || !in) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->set_state(*in);
}

int vedo_gpu_num_interactions(vedo_gpu_engine* e, uint32_t* n) {
    if (!e || !n) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->num_interactions(n);
}

int vedo_gpu_get_interactions(vedo_gpu_engine* e, const vedo_contact_view* out) {
    if (!e || !out) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->get_interactions(*out);
}

int vedo_gpu_get_contacts(vedo_gpu_engine* e, const vedo_contact_view* out) { return vedo_gpu_get_interactions(e, out); }

int vedo_gpu_get_observables(vedo_gpu_engine* e, double out[13]) {
    if (!e || !out) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->get_observables(out);
}

double vedo_gpu_time(const vedo_gpu_engine* e) { return e ? e->p->time() : 0.0; }

uint64_t vedo_gpu_step_count(const vedo_gpu_engine* e) { return e ? e->p->steps() : 0u; }

uint64_t vedo_gpu_steps_remaining(const vedo_gpu_engine* e) { return e ? e->p->steps_remaining() : 0u; }

int vedo_gpu_quiet_spheres(vedo_gpu_engine* e, uint64_t* count) {
    if (!e || !count) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->quiet_spheres(count);
}

int vedo_gpu_run_with_impulses(vedo_gpu_engine* e, const double* impulse, const double* angular_impulse,
                               int* keep_running) {
    if (!e) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->run_with_impulses(impulse, angular_impulse, keep_running);
}

int vedo_gpu_list_status(vedo_gpu_engine* e, double out[6]) {
    if (!e || !out) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->list_status(out);
}

int vedo_gpu_coordination(vedo_gpu_engine* e, uint32_t* below, uint32_t* touching, const double* box,
                          double* average) {
    if (!e || (average && !box)) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->coordination(below, touching, box, average);
}

int vedo_gpu_write_vtk(vedo_gpu_engine* e, const char* path, int with_coordination) {
    if (!e || !path) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->write_vtk(path, with_coordination);
}

int vedo_gpu_write_ido(vedo_gpu_engine* e, const char* path) {
    if (!e || !path) return VEDO_ERR_INVALID_ARGUMENT;
    return e->p->write_ido(path);
}

uint64_t vedo_gpu_last_run_profile(const vedo_gpu_engine* e, double out[4]) {
    if (!e || !out) return 0;
    return e->p->last_profile(out);
}

void vedo_gpu_set_profiling(vedo_gpu_engine* e, int on) {
    if (e) e->p->set_profiling(on != 0);
}

const char* vedo_gpu_last_error(const vedo_gpu_engine* e) {
    if (!e) return g_create_error.c_str();
    return e->p->error().c_str();
}

void vedo_gpu_destroy(vedo_gpu_engine* e) { delete e; }

int vedo_gpu_get_tuning(const vedo_gpu_engine* e, float* skin, float* cell_scale, uint32_t* tick_block,
                        uint32_t* stored_splits, uint32_t* split_tick, uint32_t* persistent) {
    if (!e || !skin || !cell_scale || !tick_block) return VEDO_ERR_INVALID_ARGUMENT;
    float t[6];
    const int rc = e->p->tuning(t);
    if (rc != VEDO_OK) return rc;
    *skin = t[0];
    *cell_scale = t[1];
    *tick_block = (uint32_t)t[2];
    if (stored_splits) *stored_splits = (uint32_t)t[3];
    if (split_tick) *split_tick = (uint32_t)t[4];
    if (persistent) *persistent = (uint32_t)t[5];
    return VEDO_OK;
}

const char* vedo_gpu_version(void) { return "vedo-gb300 0.1.0 (sm_103a)"; }

int vedo_gpu_create_batch(const vedo_scene_desc* const* scenes, uint32_t num_scenes, const vedo_engine_opts* opts,
                          vedo_gpu_engine** out) {
    if (!scenes || !out || num_scenes == 0) return VEDO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    vedo_engine_opts o;
    vedo_gpu_default_opts(&o);
    if (opts) o = *opts;
    if (o.precision != VEDO_PRECISION_MIXED) {
        g_create_error = "batches run in the MIXED form only";
        return VEDO_ERR_INVALID_ARGUMENT;
    }
    std::vector<vedo::HScene> hs(num_scenes);
    std::vector<const vedo::HScene*> ptrs(num_scenes);
    for (uint32_t k = 0; k < num_scenes; ++k) {
        std::string err;
        if (!scenes[k] || !vedo::scene_from_desc(scenes[k], hs[k], err)) {
            g_create_error = "scene " + std::to_string(k) + ": " + (scenes[k] ? err : std::string("NULL"));
            return scenes[k] ? VEDO_ERR_INVALID_SCENE : VEDO_ERR_INVALID_ARGUMENT;
        }
        vedo::prepare_scene(hs[k]);
        ptrs[k] = &hs[k];
    }
    vedo_gpu_engine* e = new (std::nothrow) vedo_gpu_engine();
    if (!e) return VEDO_ERR_OUT_OF_MEMORY;
    int rc = VEDO_OK;
    std::string err;
    e->p = vedo::make_mixed_batch(ptrs, o, &rc, &err);
    if (!e->p) {
        g_create_error = err;
        delete e;
        return rc;
    }
    *out = e;
    return VEDO_OK;
}

uint32_t vedo_gpu_num_scenes(const vedo_gpu_engine* e) { return e ? vedo::mixed_num_scenes(e->p) : 0u; }

int vedo_gpu_scene_range(const vedo_gpu_engine* e, uint32_t scene, uint32_t* first_object, uint32_t* num_objects,
                         double* time) {
    if (!e || !first_object || !num_objects) return VEDO_ERR_INVALID_ARGUMENT;
    int rc = vedo::mixed_scene_range(e->p, scene, first_object, num_objects, time);
    if (rc == VEDO_ERR_INVALID_ARGUMENT && scene == 0 && vedo::mixed_num_scenes(e->p) == 1) {
        // a single-scene FP64 engine
        *first_object = 0;
        *num_objects = e->p->num_objects();
        if (time) *time = e->p->time();
        return VEDO_OK;
    }
    return rc;
}

}  // extern "C"
