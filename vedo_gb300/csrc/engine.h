// engine.h - the GB300 DEM engine object behind the C ABI (include/vedo_gpu.h).
//
// One engine = one scene on one GPU, driven on its own CUDA stream.  Device layout:
//   objects  (n):  pos/vel/av/ox/oz/imp/aimp as double4_32a (x, y, z, pad) - one 32-byte
//                  sector per gathered vector; model index per object.
//   pairs    (P):  candidate list in the reference's NBS order: key (first < second),
//                  oriented (slave, master), parameter index, status (shear + kn as
//                  double4_32a, v0, flag byte), impulse output (J, tA, tB: 9 doubles).
//   CSR     (2P):  for each object, its pair entries (k << 1 | side) in ascending k, so
//                  the per-object impulse sum follows the reference's IactContainer order.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/vedo_gpu.h"
#include "dem_common.cuh"
#include "engine_base.h"
#include "scene_host.h"
#include "sort_scan.h"

namespace vedo {

struct PairList {
    uint32_t np = 0, cap = 0;
    uint32_t* first = nullptr;
    uint32_t* second = nullptr;
    uint2* sm = nullptr;
    uint32_t* param = nullptr;
    double4_32a* hist = nullptr;     // shear (x, y, z), kn
    double* v0 = nullptr;
    uint8_t* flags = nullptr;    // ST_* | PF_* bits (dem_physics.cuh)
    double* out = nullptr;       // [cap][9]: J, tA, tB of the last solve
    uint32_t* csr_ent = nullptr; // [2*cap]
    uint32_t* csr_ptr = nullptr; // [n+1]
    uint32_t* work = nullptr;    // [cap]: the pairs the prefilter left this step (any order)
};

class Engine : public EngineBase {
public:
    Engine() = default;
    ~Engine() override;

    int init(const HScene& scene, const vedo_engine_opts& opts) override;
    int run(uint32_t nsteps, int* keep_running) override;
    int run_with_impulses(const double* impulse, const double* angular_impulse, int* keep_running) override;
    int get_state(const vedo_state_view& v) override;
    int set_state(const vedo_state_view& v) override;
    int num_interactions(uint32_t* n) override;
    int get_interactions(const vedo_contact_view& v) override;
    int get_observables(double out[13]) override;
    int write_ido(const char* path) override;
    int coordination(uint32_t* below, uint32_t* touching, const double* box, double* average) override;
    int write_vtk(const char* path, int with_coordination) override;

    double time() const override { return t_; }
    uint64_t steps() const override { return round_; }
    uint64_t steps_remaining() const override { return count_steps(t_, dt_, t_stop_); }
    uint32_t num_objects() const override { return n_; }
    uint64_t last_profile(double out[4]) const override;
    void set_profiling(bool on) override { profiling_ = on; }
    const std::string& error() const override { return err_; }

private:
    int fail(int code, const std::string& msg) { err_ = msg; return code; }
    int cuda_fail(cudaError_t e, const char* where);
    int rebuild(bool from_records);
    int ensure_list(PairList& L, uint32_t cap);
    void free_list(PairList& L);
    int step_once(bool write_impulses);
    double* d_ext_ = nullptr;                        // [2][n][3] external impulses of run_with_impulses
    const double *ext_imp_ = nullptr, *ext_aimp_ = nullptr;
    int record_ido();
    int status_row(uint64_t records, uint64_t contacts);   // one SystemStatus.csv line
    int status_row_now();
    std::FILE* status_ = nullptr;                    // <output dir>SystemStatus.csv, with an output prefix
    int sync_host_state();
    int ensure_stage();
    int leap_cleanup(bool* erased);                  // LeapConsultant::NextStep's CleanUp at a reset
    int upload_records(const std::vector<uint64_t>& key, const std::vector<double4_32a>& hist,
                       const std::vector<double>& v0, const std::vector<uint8_t>& flags);
    bool zoi_on_ = false;                            // an active zone of interest

    // scene and options
    HScene host_;
    Tables tab_;
    vedo_engine_opts opts_{};
    std::string out_prefix_;
    std::string err_;
    uint32_t n_ = 0, nm_ = 0;
    double dt_ = 0, t_ = 0, t_stop_ = 0, sf_ = 1.1;
    double g_[3] = {0, 0, 0};
    uint64_t round_ = 0;
    uint64_t record_count_ = 0;
    bool backup_pending_ = false;   // ImpactStatus::Backup owed before the next solve
    int device_ = 0;
    cudaStream_t stream_ = nullptr;

    // device: constants
    ModelDev* d_models_ = nullptr;
    PairParam* d_params_ = nullptr;
    double4_32a* d_geom_ = nullptr;     // per (slave model, master model): ra, b0, b1, b2
    double4_32a* d_hole_ = nullptr;     // per (slave model, master model): hole radius, offsets (CD_SHP)
    int* d_group_iact_ = nullptr;
    uint32_t* d_model_of_ = nullptr;
    int* d_err_ = nullptr;
    // device: objects
    double4_32a *d_pos_ = nullptr, *d_vel_ = nullptr, *d_av_ = nullptr, *d_ox_ = nullptr, *d_oz_ = nullptr;
    double4_32a *d_imp_ = nullptr, *d_aimp_ = nullptr;
    // device: pair lists (current and previous)
    PairList cur_, old_;
    std::vector<uint32_t> global_ids_;   // host copy of the scope-global objects
    uint32_t* d_global_ = nullptr;
    // device: broad-phase scratch
    Scratch scratch_;
    double* d_safe_ = nullptr;
    unsigned long long* d_red_ = nullptr;
    uint64_t *d_key_ = nullptr, *d_key_alt_ = nullptr, *d_cell_key_ = nullptr;
    uint32_t *d_sid_ = nullptr, *d_sid_alt_ = nullptr, *d_cell_start_ = nullptr, *d_cellof_ = nullptr;
    uint32_t *d_flag_ = nullptr, *d_task_ = nullptr, *d_total_ = nullptr;
    uint32_t task_cap_ = 0;
    uint32_t *d_ck_ = nullptr, *d_cv_ = nullptr, *d_ck_alt_ = nullptr, *d_cv_alt_ = nullptr;
    uint32_t csr_cap_ = 0;
    uint32_t* d_cnt_ = nullptr;
    // records from the .ido (creation only)
    uint64_t* d_rec_key_ = nullptr;
    uint32_t nrec_ = 0;
    double4_32a* d_rec_hist_ = nullptr;
    double* d_rec_v0_ = nullptr;
    uint8_t* d_rec_flags_ = nullptr;
    // FP32 prefilter copies (prefilter.cuh): position offsets from origin_, unit wall axes,
    // and per (slave model, master model) the contact reach rounded up to float
    float4* d_pos32_ = nullptr;
    // per object: 1 when a pair of this step applied an impulse to it (k_pair_exact sets, k_obj clears)
    uint8_t* d_touched_ = nullptr;
    uint32_t* d_nwork_ = nullptr;   // pairs in the current list's worklist (k_obj empties it)
    unsigned pair_grid_ = 0;        // blocks of k_pair_exact resident at once
    // the candidate list of LeapConsultant (else NBSConsultant), and its cell edge's largest range
    bool leap_ = false;
    double leap_rmax_ = 0.0;
    float4* d_wall32_ = nullptr;
    float* d_reach_ = nullptr;
    double origin_[3] = {0, 0, 0};
    // dense cell -> cell-index map of the broad phase when the grid is small enough
    uint32_t* d_grid_ = nullptr;
    uint64_t grid_cap_ = 0;
    // observables scratch and state I/O staging ([7][n][3] doubles)
    double* d_obs_ = nullptr;
    double* d_stage_ = nullptr;
    // profiling of the last run()
    cudaEvent_t ev_[8] = {};
    bool profiling_ = false;       // per-phase CUDA-event timing (adds a host sync per step)
    double prof_ms_[4] = {0, 0, 0, 0};
    uint64_t launches_ = 0;
};

}  // namespace vedo
