// engine_base.h - the interface both engine forms implement behind the C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/vedo_gpu.h"
#include "scene_host.h"

namespace vedo {

struct Scratch;

// The device arrays the observables read, objects in the engine's order (single-scene engines).
struct DeviceObjects {
    uint32_t n = 0;
    const uint32_t* model_of = nullptr;
    const ModelDev* models = nullptr;
    const double4_32a* pos = nullptr;
    cudaStream_t stream = nullptr;
    Scratch* scratch = nullptr;
    const HScene* scene = nullptr;       // the models and object order of the scene
    uint64_t* launches = nullptr;        // the engine's kernel launch counter
};

class EngineBase {
public:
    virtual ~EngineBase() = default;
    virtual int init(const HScene& scene, const vedo_engine_opts& opts) = 0;
    virtual int run(uint32_t nsteps, int* keep_running) = 0;
    virtual int get_state(const vedo_state_view& v) = 0;
    virtual int set_state(const vedo_state_view& v) = 0;
    virtual int num_interactions(uint32_t* n) = 0;
    virtual int get_interactions(const vedo_contact_view& v) = 0;
    virtual int get_observables(double out[13]) = 0;
    virtual int write_ido(const char* path) = 0;
    virtual double time() const = 0;
    virtual uint64_t steps() const = 0;
    // SimMediator::Run calls left before t >= t_stop, with the same accumulation t += dt
    virtual uint64_t steps_remaining() const = 0;
    virtual uint32_t num_objects() const = 0;
    virtual uint64_t last_profile(double out[4]) const = 0;
    virtual void set_profiling(bool on) = 0;
    virtual const std::string& error() const = 0;
    // skin fraction, cell scale, tick block size, stored position splits, split tick, persistent
    // tick (MIXED only)
    virtual int tuning(float out[6]) const { (void)out; return VEDO_ERR_INVALID_ARGUMENT; }
    virtual int quiet_spheres(uint64_t* count) {
        *count = 0;
        return VEDO_OK;
    }
    virtual int run_with_impulses(const double* impulse, const double* angular_impulse, int* keep_running) = 0;
    virtual int list_status(double out[6]) {
        for (int k = 0; k < 6; ++k) out[k] = 0.0;
        return VEDO_OK;
    }
    // CalcCoordinateNum over the current state; the world (and coordination numbers) as VTK
    virtual int coordination(uint32_t* below, uint32_t* touching, const double* box, double* average) = 0;
    virtual int write_vtk(const char* path, int with_coordination) = 0;
};

// Shared implementations of the two observables over an engine's DeviceObjects.
int coordination_host(const DeviceObjects& d, uint32_t* below, uint32_t* touching, const double* box,
                      double* average, std::string& err);
int write_vtk_host(EngineBase* e, const DeviceObjects& d, const char* path, int with_coordination, std::string& err);

// count of t += dt steps from t until t >= t_stop (SystemParameter::NextStep, SimMediator.cpp:839-841)
inline uint64_t count_steps(double t, double dt, double t_stop) {
    uint64_t k = 0;
    if (!(dt > 0.0)) return 0;
    while (t < t_stop) {
        t += dt;
        ++k;
    }
    return k;
}

EngineBase* make_fp64_engine();
EngineBase* make_mixed_engine();
// MIXED-form engine over several scenes (vedo_gpu_create_batch); nullptr with *rc / *err on failure.
EngineBase* make_mixed_batch(const std::vector<const HScene*>& scenes, const vedo_engine_opts& opts, int* rc,
                             std::string* err);
// Scene count and per-scene object range / time of a batch engine (1 scene for any other engine).
uint32_t mixed_num_scenes(EngineBase* e);
// Continuous batching: a new MIXED engine from scenes `keep` of `prev` (moved on the device,
// state and contact history) followed by the host scenes `add`; nullptr with *rc / *err.
EngineBase* mixed_repack(EngineBase* prev, const std::vector<uint32_t>& keep, const std::vector<const HScene*>& add,
                         const vedo_engine_opts& opts, int* rc, std::string* err);
int mixed_set_scene_active(EngineBase* e, uint32_t s, bool on);
int mixed_get_state_slice(EngineBase* e, uint32_t off, uint32_t cnt, const vedo_state_view& v);
uint64_t mixed_scene_steps(EngineBase* e, uint32_t s);
int mixed_scene_range(EngineBase* e, uint32_t s, uint32_t* off, uint32_t* n, double* t);

}  // namespace vedo
