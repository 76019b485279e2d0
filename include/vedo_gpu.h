/*
 * vedo_gpu.h - C ABI of the GB300 DEM time-step engine.
 *
 * The engine replaces, behind one handle, the container-level loops that the
 * reference drives once per time step from SimMediator::Run()
 * (src/vedo/framework/SimMediator.cpp:714-842):
 *   IactContainer::CalculateImpact    (IactContainer.cpp:33-37)  impact solving
 *   DOContainer::AddFieldImpact       (DOContainer.cpp:20-27)    field impulse
 *   DOContainer::AddConstrainedImpact (DOContainer.cpp:47-50)    external force
 *   DOContainer::Response             (DOContainer.cpp:52-55)    integration
 *   IactContainer::CheckContactStatus (IactContainer.cpp:47-50)  narrow phase
 *   Consultant::NextStep / Reset      (NBSConsultant.cpp:35-316) broad phase,
 *   RebuildIactRecordTab + Initiate   (NBSConsultant.cpp:376-395,
 *                                      SimMediator.cpp:640-712)  history carry
 * The reference has no FFI of its own: its plugin surface is the C++ class
 * hierarchy (ContactDetector::Detect, ContactDetector.h:50; ImpactSolver::
 * NextStep, ImpactSolver.h:22-23; DiscreteObject::Response,
 * DiscreteObject.h:107; Consultant, Consultant.h:87-154) selected through the
 * factories registered in CreateNewAssembler (ModuleList.h:42-77).  These entry
 * points are what a SimMediator-level binding calls instead; every argument is
 * a plain pointer or size, and every function returns a status code instead of
 * calling exit() as the reference does on bad input.
 *
 * Units and layouts follow the reference: FP64 everywhere, 3-vectors as
 * [n][3] row-major double arrays, object indices are the DOWorld indices
 * (uint32, the reference's _INT32 build).
 */
#ifndef VEDO_GPU_H
#define VEDO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    VEDO_OK = 0,
    VEDO_ERR_INVALID_ARGUMENT = 1,  /* NULL handle/pointer, size mismatch            */
    VEDO_ERR_INVALID_SCENE = 2,     /* unknown model, bad index, empty world          */
    VEDO_ERR_UNSUPPORTED_MODEL = 3, /* no detector/solver for a shape pair or
                                       equation type (the factories' null result,
                                       Assembler.cpp:72-85), or a feature the chosen
                                       form does not implement (e.g. a periodic
                                       boundary in the mixed form)                    */
    VEDO_ERR_OUT_OF_MEMORY = 4,     /* device allocation failed / admission rejected  */
    VEDO_ERR_CUDA = 5,              /* any other CUDA runtime error                   */
    VEDO_ERR_DEVICE_TIMEOUT = 6,    /* a bounded device wait gave up                  */
    VEDO_ERR_BAD_IDO = 7,           /* unreadable, truncated or inconsistent .ido     */
    VEDO_ERR_IO = 8                 /* output file could not be written               */
};

/* ---- enums mirrored from DOModel.h:25-27 (C++11 build) ------------------ */
enum { VEDO_SHAPE_SPHERE = 1, VEDO_SHAPE_QUASI_CYLINDER = 6, VEDO_SHAPE_QUASI_PLATE = 7,
       VEDO_SHAPE_QUASI_PLATE_WITH_CIRCULAR_HOLE = 8 };
/* No counterpart in the reference (its QuasiCylinder is the outside of a solid rod,
 * CDSphere2QuasiCylinder.cpp:40-50): the inside of a hollow cylinder, a drum shell.  attrs
 * {radius, length} about OrientationZ; global scope; fixed or orbital (a drum turning about its
 * own axis).  A sphere inside touches it where its centre is farther than radius - r from the
 * axis, within the length; beyond either end, the rim circle.  Scenes that use it cannot be
 * read by the reference. */
enum { VEDO_SHAPE_INNER_CYLINDER = 32 };
enum { VEDO_CONSTRAINED = 1, VEDO_FIXED = 2, VEDO_MOBILE = 3, VEDO_ORBITAL = 4 };
enum { VEDO_SCOPE_GLOBAL = 1, VEDO_SCOPE_LOCAL = 2 };

/* ---- scene description (what DOWorld holds, DOWorld.h) ----------------- */
typedef struct vedo_do_model {
    const char* name;          /* DOModel name                                     */
    const char* group;         /* DOGroup; interaction models are found by group   */
    uint32_t behavior;         /* VEDO_CONSTRAINED/FIXED/MOBILE/ORBITAL            */
    uint32_t scope;            /* VEDO_SCOPE_GLOBAL/LOCAL                          */
    uint32_t shape;            /* VEDO_SHAPE_*                                     */
    uint32_t reserved;
    double density;
    double density_factor;
    double external_force[3];
    double attrs[10];          /* DOShapeAttributes union: sphere {radius};
                                  quasicylinder {radius, height};
                                  quasiplate {width, height, length}               */
} vedo_do_model;

typedef struct vedo_iact_model {
    const char* master_group;
    const char* slave_group;
    const char* equation_type;               /* "ISwBSDBF", "ISwHertz", ...       */
    uint32_t num_mechanisms;
    const char* const* mechanism_names;      /* e.g. "NormalStiffness"            */
    const double* mechanism_values;
} vedo_iact_model;

typedef struct vedo_scene_desc {
    /* SystemParameter (SystemParameter.h) */
    double time_start, time_stop, time_interval, time_current;
    double field_acceleration[3];
    double safety_factor;                    /* aries::Constants SafetyFactor     */
    uint8_t zoi_switch[3], pbc_switch[3];
    uint8_t reserved[2];
    double zoi_lower[3], zoi_upper[3];
    double pbc_lower[3], pbc_upper[3];       /* periodic boundary (Boundary.cpp:225-345):
                                                an axis is periodic where its bounds
                                                differ; FP64 form only                 */
    uint32_t max_id_of_do;
    /* models */
    uint32_t num_models;
    const vedo_do_model* models;
    uint32_t num_iact_models;
    const vedo_iact_model* iact_models;
    /* DOStatus, one entry per discrete object, [n][3] doubles each */
    uint32_t num_objects;
    const uint32_t* object_model;            /* index into models                 */
    const uint32_t* object_id;               /* DOStatus ulID (may be NULL)       */
    const double* position;
    const double* velocity;
    const double* orientation_x;
    const double* orientation_z;
    const double* angular_velocity;
    const double* impact;                    /* may be NULL (zeros)               */
    const double* angular_impact;            /* may be NULL (zeros)               */
    /* IactRecordTab (IactRecordTab.cpp:346-530): shear history to re-attach */
    uint32_t num_records;
    const uint32_t* record_first;            /* lower object index                */
    const uint32_t* record_second;           /* higher object index               */
    const uint8_t* record_contact;
    const uint8_t* record_bond;
    const double* record_kn;
    const double* record_initial_velocity;
    const double* record_shear;              /* [n][3]                            */
} vedo_scene_desc;

/* ---- engine options ---------------------------------------------------- */
/* FP64: the drop-in; every FP64 operation in the reference's order, results bit-identical
 *       to the reference for the linear laws (Hertz-family laws and orbital walls within the
 *       last-ulp differences of pow, sin and cos).
 * MIXED: contact forces in FP32 in pair-local coordinates, FP64 positions, velocities and
 *       overlap numerators, FP32 compensated sums per object; contact sets identical to
 *       FP64 at identical positions; sphere orientations are not integrated. */
enum { VEDO_PRECISION_FP64 = 0, VEDO_PRECISION_MIXED = 1 };

typedef struct vedo_engine_opts {
    uint32_t up_iact;         /* candidate-list rebuild interval in steps (anne
                                 <UpIact>, NBSConsultant::ISReset, NBSConsultant.cpp:80-83) */
    uint32_t record;          /* IDO record interval in steps (anne <Record>);
                                 0 = never                                          */
    uint32_t precision;       /* VEDO_PRECISION_FP64 (the drop-in) or _MIXED       */
    int32_t device;           /* CUDA device ordinal                               */
    const char* output_prefix;/* "<prefix>_NNNNNNN.ido" records and terminate.ido are
                                 written when non-NULL, as Consultant::RecordIDO
                                 (Consultant.cpp:217-230) and NBSConsultant::NextStep
                                 (NBSConsultant.cpp:63-76) do; NULL writes nothing  */
    float skin;               /* MIXED only: neighbour-list skin as a fraction of the
                                 largest sphere radius (default 0.15); the list is rebuilt
                                 when any sphere may have moved half of it.  Entries with
                                 orbital walls are gathered with 8 times the skin and the
                                 list is also rebuilt when a sphere's and an orbital wall's
                                 travel together may have used that up                  */
    uint32_t check_interval;  /* MIXED only: steps between displacement checks (10)   */
    uint32_t tick_block;      /* MIXED only: threads per block of the tick kernel, 32..256,
                                 a multiple of 32 (0 = 256)                            */
    float cell_scale;         /* MIXED only: cell edge as a multiple of 2 r_max + skin,
                                 >= 1 (0 = 1)                                          */
    uint32_t autotune;        /* MIXED only: 1 = the first steps of the run choose the tick
                                 block, the skin and the cell scale by timing (results do
                                 not depend on them); read the choice with
                                 vedo_gpu_get_tuning                                    */
    uint32_t graphs;          /* MIXED only: 1 = each check interval of steps is replayed
                                 as one CUDA graph, captured once per neighbour list (default) */
    uint32_t stored_splits;   /* MIXED only: 1 = the hi/lo FP32 splits of the positions used by
                                 the sphere-pair overlap test are stored once per step; 0 = formed
                                 per pair (identical results; the autotuner chooses)       */
    uint32_t split_tick;      /* MIXED only, the form of the tick: 0 = one full tick (each
                                 sphere walks its list and evaluates its pairs); 1 = a light
                                 tick (prefilter only, high occupancy) finishes the spheres
                                 without a pair on the exact path and defers the rest to the
                                 full tick; 2 = the pair pass (a prefilter pass lists the pairs
                                 on the exact path, each is evaluated once, then every sphere
                                 sums its pairs' records in list order).  Identical results;
                                 the autotuner chooses                                     */
    uint32_t full_walks;      /* MIXED only: 1 = every sphere walks its neighbour list every
                                 step; 0 = a sphere whose pairs are all certainly apart since
                                 the rebuild, with clean history, skips the walk (default;
                                 identical results)                                     */
    uint32_t consultant;      /* FP64 only: the candidate list of 0 = NBSConsultant (anne's
                                 "nbs", NBSConsultant.cpp:85-374) or 1 = LeapConsultant
                                 ("leap", LeapConsultant.cpp:108-195, LeapConsultant.h:58-446:
                                 cells ordered along the widest axis, periodic neighbours);
                                 the MIXED form's lists are complete by construction     */
    uint32_t orientations;    /* MIXED only: 1 = integrate the spheres' orientations (Ox, Oz
                                 turned by dt (w + dw/2) each step in FP64, as
                                 DOSphere::Response, DOSphere.cpp:40-44); 0 = leave them as
                                 they are (default: no force or contact depends on a sphere's
                                 orientation, and the turn costs FP64 sines and cosines per
                                 spinning sphere per step).  The FP64 form always turns them */
    uint32_t persistent;      /* MIXED only: 1 = a check interval of steps runs as ONE cooperative
                                 launch (every block resident at once) whose stages are separated
                                 by grid barriers, in place of a replayed graph of per-step
                                 kernels; for the full tick and the pair pass (split_tick 0 or 2)
                                 without mobile or constrained walls, other steps as before.  Each
                                 barrier's wait is bounded (2 s): on expiry the call returns
                                 VEDO_ERR_CUDA and the engine's state is undefined (kernels of
                                 other streams or processes holding SMs for seconds delay its
                                 blocks and can cause that).  Identical results; the autotuner
                                 chooses (default 0)                                      */
} vedo_engine_opts;

typedef struct vedo_gpu_engine vedo_gpu_engine;

/* Default options: up_iact 1, record 0, FP64, device 0, no files; MIXED: skin 0.15,
 * check_interval 10, tick_block 256, cell_scale 1, no autotuning, graphs on. */
void vedo_gpu_default_opts(vedo_engine_opts* opts);

/* Build an engine from a scene.  Replaces DOWorld + NBSConsultant +
 * SimMediator construction (Anne.cpp:83-119, SimMediator.cpp:83-137): the
 * first candidate list is built, interactions are created with the
 * Assembler's slave/master and model-selection rules (Assembler.cpp:15-87,
 * CDFactory.h:66-95, ISFactory.h:45-48) and the IactRecordTab history is
 * re-attached.  The scene's host arrays are copied; the caller keeps them. */
int vedo_gpu_create(const vedo_scene_desc* scene, const vedo_engine_opts* opts, vedo_gpu_engine** out);

/* Same, reading a reference .ido file (DOWorld::ReadIDO, DOWorld_RWIDO.cpp:9-55). */
int vedo_gpu_create_from_ido(const char* path, const vedo_engine_opts* opts, vedo_gpu_engine** out);

/* Same, reading a DOWorldSchema XML scene (DOWorld::ReadXML, DOWorld_ReadXML.cpp:592-660; the
 * reference parses it with boost::property_tree, the engine with its own reader).  As the
 * reference reader does, only a SimConstant named "SafetyFactor" sets the safety factor. */
int vedo_gpu_create_from_xml(const char* path, const vedo_engine_opts* opts, vedo_gpu_engine** out);

/* Convert a scene file between .ido and .xml by the names' extensions, without a GPU (the
 * reference's DOWorld::ReadIDO/WriteIDO and ReadXML/WriteXML; XML values are written with 17
 * significant digits); a .vtu output is the world as the post-processing tool's conversion
 * writes it (DOWorld::WriteVTK<NullExternalFieldVTKWriter>, DOWorld_WriteVTK.h:148-243). */
int vedo_convert_scene(const char* in_path, const char* out_path);

/* Advance nsteps time steps, each one SimMediator::Run() (SimMediator.cpp:714-842).
 * *keep_running (may be NULL) receives the last step's return value,
 * t_current < t_stop (SimMediator.cpp:839-841). */
int vedo_gpu_run(vedo_gpu_engine* e, uint32_t nsteps, int* keep_running);
/* The same under the name of the step contract: `while (sm.Run())` of Anne.cpp:128 becomes
 * `do vedo_gpu_step(e, k, &keep); while (keep);`. */
int vedo_gpu_step(vedo_gpu_engine* e, uint32_t nsteps, int* keep_running);

/* Object state, [n][3] doubles per array; any pointer may be NULL.  impact /
 * angular_impact are the impulses the last Response consumed, as DOStatus
 * holds them after DiscreteObject::ClearImpact (DiscreteObject.cpp:141-147). */
typedef struct vedo_state_view {
    double* position;
    double* velocity;
    double* angular_velocity;
    double* orientation_x;
    double* orientation_z;
    double* impact;
    double* angular_impact;
} vedo_state_view;

/* Objects now (DOWorld's object count).  With the Leap consultant and an active zone of interest
 * the mobile objects that leave the zone are erased at the next reset (LeapConsultant.cpp:61-68,
 * Consultant::CleanUp), so the count, and the length of every state array, can shrink during a
 * vedo_gpu_run call: read it after each call. */
uint32_t vedo_gpu_num_objects(const vedo_gpu_engine* e);
int vedo_gpu_get_state(vedo_gpu_engine* e, const vedo_state_view* out);
/* Overwrite the object state (DOContainer::SetDOStatus, DOContainer.h:55-58). */
int vedo_gpu_set_state(vedo_gpu_engine* e, const vedo_state_view* in);

/* Interaction list in candidate-list order (the reference's IactContainer order).
 * first < second are object indices (the IactRecordTab key); slave/master is
 * the Assembler orientation; active = ContactInfo::bActive of the last
 * narrow-phase pass; shear/kn/contact = the solver's ImpactStatus.  Any
 * pointer may be NULL. */
typedef struct vedo_contact_view {
    uint32_t* first;
    uint32_t* second;
    uint32_t* slave;
    uint32_t* master;
    uint8_t* active;
    double* shear;             /* [n][3] */
    double* kn;
    uint8_t* contact;
} vedo_contact_view;

int vedo_gpu_num_interactions(vedo_gpu_engine* e, uint32_t* n);
int vedo_gpu_get_interactions(vedo_gpu_engine* e, const vedo_contact_view* out);
/* The same under the name of the contacts contract: pairs (first < second), active flag, shear
 * and kn of every interaction, vedo_gpu_num_interactions long. */
int vedo_gpu_get_contacts(vedo_gpu_engine* e, const vedo_contact_view* out);

/* System observables as DOWorld::CalculateSystemEnergy computes them
 * (DOWorld.cpp:481-660) over the current state, mobile objects only:
 * out[0..8] = potential, translational, rotational energy, v min, v max,
 * omega min, omega max, momentum norm, angular-momentum norm;
 * out[9] = number of active contacts, out[10] = mass-weighted centre of mass x,
 * out[11] = y, out[12] = z. */
int vedo_gpu_get_observables(vedo_gpu_engine* e, double out[13]);

/* Simulated time (SystemParameter::GetTimeCurrent) and step counter. */
double vedo_gpu_time(const vedo_gpu_engine* e);
uint64_t vedo_gpu_step_count(const vedo_gpu_engine* e);
/* Steps left until SimMediator::Run would return false (t >= t_stop, with the same FP
 * accumulation t += dt; SimMediator.cpp:839-841), so that a caller can advance to the end in
 * a few vedo_gpu_run calls.  For a batch: scene 0. */
uint64_t vedo_gpu_steps_remaining(const vedo_gpu_engine* e);

/* One time step with an external impulse and angular impulse for every object, as
 * SimMediator::Run(external impacts) (SimMediator.cpp:987-1119, the coupling entry): they are
 * added after the field and constrained impulses (DOContainer::AddImpact), before the response.
 * impulse, angular_impulse: host [n][3] arrays in object order (NULL = zeros).  keep_running as
 * vedo_gpu_run.  In the MIXED form they join the spheres' FP32 compensated sums; fixed and
 * orbital walls do not respond to impulses in either form. */
int vedo_gpu_run_with_impulses(vedo_gpu_engine* e, const double* impulse, const double* angular_impulse,
                               int* keep_running);

/* MIXED form: the number of spheres whose next step skips the neighbour-list walk (every pair
 * certainly apart since the last rebuild and its history clean; results are those of a full
 * walk).  A measure of how much of the list the skin keeps idle.  FP64 form: 0. */
int vedo_gpu_quiet_spheres(vedo_gpu_engine* e, uint64_t* count);

/* MIXED form: the neighbour list's state.  out[0] = steps since its rebuild, out[1] = rebuilds
 * so far, out[2] = bound on any sphere's displacement relative to its scene's drifting frame
 * (free fall from the spheres' velocity midrange at the rebuild), out[3] = bound on any
 * sphere's displacement, out[4] = bound on any orbital wall's approach, out[5] = the share of
 * the list's life used (1 = the next step rebuilds).  FP64 form: zeros. */
int vedo_gpu_list_status(vedo_gpu_engine* e, double out[6]);

/* Write world + active-contact records as a reference .ido
 * (DOWorld::WriteIDO, DOWorld_RWIDO.cpp:149-202). */
int vedo_gpu_write_ido(vedo_gpu_engine* e, const char* path);

/* Coordination numbers of the post-processing tool (CalcCoordinateNum.cpp, replaces
 * CalcCoordinateNum::computeAvgCoordinateNum :8-77 and outputCoordinateNumVTK :79-126), computed
 * on the device from the current state: per object, the number of other spheres whose centre
 * distance is below (`below`) or at most (`touching`) the radius sum, 0 for other shapes (either
 * array may be NULL, else num_objects long).  With `box` = {xmin, xmax, ymin, ymax, zmin, zmax}
 * and `average`, *average = computeAvgCoordinateNum over the box: the `touching` counts of the
 * spheres whose centre lies strictly inside the box widened by their radius, summed as an
 * unsigned 32-bit integer and divided by their number (NaN when there is none).  Single-scene
 * engines (VEDO_ERR_INVALID_ARGUMENT for a batch). */
int vedo_gpu_coordination(vedo_gpu_engine* e, uint32_t* below, uint32_t* touching, const double* box,
                          double* average);

/* The current state as a VTK unstructured-grid file (DOWorld::WriteVTK, DOWorld_WriteVTK.h:148-243):
 * every object a point with position, velocity, angular velocity, their magnitudes, radius (0 for
 * other shapes) and granular temperatures (0); with_coordination != 0 adds the spheres'
 * "CoordinateNumber" field (the `below` counts, spheres in object order) as
 * CalcCoordinateNum::outputCoordinateNumVTK writes it.  Single-scene engines. */
int vedo_gpu_write_vtk(vedo_gpu_engine* e, const char* path, int with_coordination);

/* Device time of the last vedo_gpu_run call in milliseconds, from CUDA events on
 * the engine's stream: out[3] = the whole call; with profiling on (see
 * vedo_gpu_set_profiling) also, FP64 form: out[0] = pair kernel (detect + impact
 * solve), out[1] = object kernels (gather + integrate); MIXED form: out[0] = the
 * fused tick kernel (every launch timed alone), out[1] = the wall kernels; both:
 * out[2] = broad-phase rebuilds.  Returns the number of kernel launches the call
 * issued. */
uint64_t vedo_gpu_last_run_profile(const vedo_gpu_engine* e, double out[4]);

/* Enable per-phase CUDA-event timing for vedo_gpu_last_run_profile (adds one host
 * synchronisation per step; off by default). */
void vedo_gpu_set_profiling(vedo_gpu_engine* e, int on);

/* Message of the last failure of e; with e == NULL, of the last failed create call
 * on this thread. */
const char* vedo_gpu_last_error(const vedo_gpu_engine* e);
void vedo_gpu_destroy(vedo_gpu_engine* e);

/* Skin (fraction of r_max), cell scale, tick block size, split storage, the form of the tick
 * (vedo_engine_opts.split_tick: 0, 1 or 2) and whether a check interval runs as one persistent
 * launch (vedo_engine_opts.persistent; the last three may be NULL) in use by a MIXED-form engine,
 * after autotuning when it was asked for.  No counterpart in the reference. */
int vedo_gpu_get_tuning(const vedo_gpu_engine* e, float* skin, float* cell_scale, uint32_t* tick_block,
                        uint32_t* stored_splits, uint32_t* split_tick, uint32_t* persistent);

/* The persistent tick's grid barrier on its own (no counterpart in the reference): `rounds`
 * barriers over a cooperative grid of every block the device holds at once, where each barrier
 * expects `extra` more arrivals than the grid has (0: a working barrier; > 0: one that nothing
 * completes, whose wait must end after `limit_ns` nanoseconds with the expiry recorded).  out[0]:
 * rounds completed; out[1]: blocks that saw a round's arrivals miscounted; out[2]: 1 = a wait
 * expired; out[3]: the round whose barrier expired first.  The device stays usable either way. */
int vedo_gpu_barrier_check(int32_t device, uint32_t rounds, uint32_t extra, uint64_t limit_ns, uint32_t out[4]);

/* Library version string. */
const char* vedo_gpu_version(void);

/* ---- batches of scenes (MIXED form) -------------------------------------
 * No counterpart in the reference, which runs one DOWorld per anne process
 * (Anne.cpp:83-119).  One engine advances many independent scenes with one
 * fused launch per step: objects are numbered scene after scene (scene s owns
 * objects [first, first + count) of every state and contact array), objects of
 * different scenes never interact, and each scene keeps its own time step, field
 * acceleration, models and interaction models.  A scene's results do not depend
 * on the other scenes of the batch: they are bit-identical to the same scene run
 * alone in the MIXED form.  vedo_gpu_run advances every scene by nsteps steps;
 * *keep_running refers to scene 0.  vedo_gpu_get_observables sums over all
 * scenes with scene 0's field acceleration; vedo_gpu_write_ido needs a
 * single-scene engine. */
int vedo_gpu_create_batch(const vedo_scene_desc* const* scenes, uint32_t num_scenes, const vedo_engine_opts* opts,
                          vedo_gpu_engine** out);
uint32_t vedo_gpu_num_scenes(const vedo_gpu_engine* e);
/* Object range and simulated time of one scene of a batch (scene 0 of a plain engine). */
int vedo_gpu_scene_range(const vedo_gpu_engine* e, uint32_t scene, uint32_t* first_object, uint32_t* num_objects,
                         double* time);

/* ---- serving: continuous batching of DEM jobs (MIXED form) -------------
 * No counterpart in the reference (anne runs one scene per process).  A server owns one
 * GPU and a thread that advances every live job's scene in the same fused launches.  Jobs
 * (a scene and a step count) are submitted from any thread at any time; each waits in a
 * FIFO queue until admission, which counts the job's device memory against the HBM
 * budget: VEDO_SRV_BYTES_PER_OBJECT per object (state, FP32 copies, splits, sort and cell
 * keys, staging) plus, per sphere, VEDO_SRV_ENTRIES_PER_SPHERE neighbour-list entries of
 * VEDO_SRV_BYTES_PER_ENTRY (the current and previous list with their history and flags, the
 * wall-impulse rows, all with the 25 % growth the engine allocates), and
 * VEDO_SRV_BYTES_PER_ENTRY_PAIR_PASS more per entry when the server's options ask for the pair
 * pass or for autotuning (the pair pass's worklist, marks and pair records); a dense packing
 * lists 12-14 neighbours per sphere within its skin.  The live set is kept at
 * or below half the budget, because adding or removing jobs builds the next batch on the
 * device while the current one still exists.  Admitted jobs join the batch at the next
 * check interval, with their state and contact history resident on the device from then
 * on; a job stops after exactly its step count and its final state is copied to the host.
 * A job's result equals the same scene run alone in the MIXED form for the same number
 * of steps, bit for bit. */
/* Admission order: arrival (default), or the queued job with the least work (spheres x steps)
 * first; with a cap on the live jobs' spheres (0: none), a job waits while admitting it would pass
 * the cap (a job larger than the cap alone runs when nothing else does).  Shortest-first with a cap
 * trades the long jobs' latency for the short ones' when the offered work exceeds the GPU's rate.
 * No counterpart in the reference. */
#define VEDO_SRV_FIFO 0u
#define VEDO_SRV_SHORTEST_FIRST 1u
#define VEDO_SRV_BYTES_PER_OBJECT 800u
#define VEDO_SRV_ENTRIES_PER_SPHERE 18u
#define VEDO_SRV_BYTES_PER_ENTRY 150u
#define VEDO_SRV_BYTES_PER_ENTRY_PAIR_PASS 72u
enum { VEDO_JOB_QUEUED = 0, VEDO_JOB_RUNNING = 1, VEDO_JOB_DONE = 2, VEDO_JOB_CANCELLED = 3, VEDO_JOB_FAILED = 4 };

typedef struct vedo_job_info {
    uint32_t status;          /* VEDO_JOB_*                                              */
    uint32_t num_objects;
    uint64_t steps;           /* requested                                               */
    uint64_t steps_done;
    double submit_s;          /* seconds since the server started: submission,          */
    double admit_s;           /*   admission (joined the batch) and completion; -1 = not */
    double done_s;            /*   yet                                                   */
    uint64_t charged_bytes;   /* device memory the admission counts for the job          */
} vedo_job_info;

typedef struct vedo_server vedo_server;

/* opts: engine options of the batch (precision must be MIXED); hbm_budget_bytes: device
 * memory the server may hold. */
int vedo_srv_create(const vedo_engine_opts* opts, uint64_t hbm_budget_bytes, vedo_server** out);
/* Queue a job: the scene is copied; steps >= 1.  Fails (and queues nothing) when the scene is
 * invalid or the job alone would not fit the budget. */
int vedo_srv_set_policy(vedo_server* s, uint32_t order, uint64_t max_live_spheres);
int vedo_srv_submit(vedo_server* s, const vedo_scene_desc* scene, uint64_t steps, uint64_t* job_id);
int vedo_srv_poll(vedo_server* s, uint64_t job_id, vedo_job_info* info);
/* Block until the job is done, cancelled or failed, or timeout_s passes (then
 * VEDO_ERR_DEVICE_TIMEOUT); info may be NULL. */
int vedo_srv_wait(vedo_server* s, uint64_t job_id, double timeout_s, vedo_job_info* info);
/* Final state of a done job ([n][3] host arrays, any pointer may be NULL). */
int vedo_srv_result(vedo_server* s, uint64_t job_id, const vedo_state_view* out);
/* Cancel a queued or running job (a running one stops at the next check interval). */
int vedo_srv_cancel(vedo_server* s, uint64_t job_id);
/* out[0] jobs done, [1] particle-steps of done jobs, [2] seconds the batch was stepping,
 * [3] batches built, [4] objects in the current batch, [5] bytes committed to live jobs,
 * [6] jobs queued, [7] jobs running. */
int vedo_srv_stats(vedo_server* s, double out[8]);
const char* vedo_srv_last_error(const vedo_server* s);
/* Stops the server thread (running jobs are abandoned) and frees the GPU. */
void vedo_srv_destroy(vedo_server* s);

/* ---- allocation-free system energy --------------------------------------
 * No counterpart in the reference.
 * For callers that cannot let a library allocate device memory: a coupled solver or a
 * framework whose own allocator already holds most of HBM (a new cudaMalloc would fail or
 * fragment its pool), or a hook on a time-critical loop (cudaFree, and often cudaMalloc,
 * synchronise the whole device).  The same quantities as vedo_gpu_get_observables, over
 * object state that the caller keeps in its own device buffers:
 *   position, velocity, angular_velocity, inertia: [n][3] doubles (principal moments);
 *   mass: [n] doubles; mobile: [n] bytes, nonzero = counted (NULL counts every object);
 *   field_acceleration: 3 doubles in host memory;
 *   out: 12 doubles in device memory, written when the stream reaches the call:
 *   out[0..8] as vedo_gpu_get_observables out[0..8], out[9..11] the mass-weighted centre.
 * stream is a cudaStream_t (NULL = the legacy default stream); the call does not wait.
 * The reduction's partial sums live in a fixed 1 MiB array that the library declares in
 * device memory, which every GPU that loads the library holds until the process exits.
 * The call allocates nothing.  At most VEDO_NOALLOC_MAX_OBJECTS objects; larger counts
 * return VEDO_ERR_INVALID_ARGUMENT with a message (vedo_gpu_last_error(NULL)), and so do
 * buffers that are not device (or managed) memory of the current device.  The first call on
 * each device, with that device current, looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it for the life of the process; with CUDA's lazy module
 * loading that first call is also where the module is loaded and the array reserved, which
 * can synchronise the device: make one warm-up call at set-up, before any stream capture and
 * outside time-critical loops.  A cudaDeviceReset (or anything else that tears the primary
 * context down) invalidates the kept address: do not call this entry point again in that
 * process after such a reset.  All calls share the one array: calls that overlap on the GPU
 * (on different streams, or from different threads without ordering) race and give wrong
 * results. */
/* ---- scene generation helper -----------------------------------------------
 * No counterpart in the reference (it reads scenes from files; this seeds the synthetic
 * workloads).  Random sequential placement, host only: sphere i (in the given order) is
 * drawn uniformly, up to max_tries times, in the box [lo, hi] shrunk by its radius and, when
 * cyl_radius > 0, inside the cylinder of that radius about the x axis shrunk by its radius;
 * it is kept at the first draw that overlaps no sphere kept before.  out: [n][3] centres
 * (NaN for a sphere not placed); *placed: the count kept.  The same seed gives the same
 * spheres on every host. */
int vedo_place_spheres(uint32_t n, const double* radii, const double lo[3], const double hi[3],
                       double cyl_radius, uint64_t seed, uint32_t max_tries, double* out,
                       uint32_t* placed);

#define VEDO_NOALLOC_MAX_OBJECTS 16777216u
int vedo_gpu_system_energy_noalloc(const double* position, const double* velocity, const double* angular_velocity,
                                   const double* mass, const double* inertia, const uint8_t* mobile,
                                   uint32_t num_objects, const double field_acceleration[3], double* out,
                                   void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VEDO_GPU_H */
