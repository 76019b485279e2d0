/*
 * dem_oracle.h - CPU restatement of the reference DEM time step.
 *
 * TEST INFRASTRUCTURE ONLY.  The GPU engine never links, loads or calls this
 * code; tests, __graft_entry__.smoke() and the CPU-baseline arm of bench.py use
 * it as the checker.  Its results are pinned bit-for-bit against the reference
 * itself (oracle/_ref, built from the reference sources by oracle/Makefile)
 * by tests/test_oracle_vs_ref.py and the committed fixtures in tests/golden/.
 */
#ifndef VEDO_DEM_ORACLE_H
#define VEDO_DEM_ORACLE_H

#include "../include/vedo_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dp_world dp_world;

/* Build the world: NBS candidate list, SimMediator::Initiate, IDO history
 * re-attach.  Returns NULL and fills err on an unsupported/invalid scene. */
/* consultant: 0 NBSConsultant, 1 LeapConsultant (the candidate list each builds) */
dp_world* dp_create(const vedo_scene_desc* scene, unsigned up_iact, int consultant, char* err, size_t errlen);
/* nsteps SimMediator::Run() calls; returns the last t_current < t_stop. */
int dp_run(dp_world* w, unsigned nsteps);
unsigned dp_num_objects(const dp_world* w);
void dp_get_state(const dp_world* w, double* pos, double* vel, double* avel, double* ox, double* oz,
                  double* imp, double* aimp);
void dp_set_state(dp_world* w, const double* pos, const double* vel, const double* avel, const double* ox,
                  const double* oz);
unsigned dp_num_candidates(const dp_world* w);
void dp_get_candidates(const dp_world* w, unsigned* first, unsigned* second);
void dp_get_interactions(const dp_world* w, unsigned* slave, unsigned* master, int* active, double* depth,
                         double* normal, double* shear, double* kn, int* contact);
double dp_time(const dp_world* w);
/* DOWorld::CalculateSystemEnergy over the current state (9 values, same
 * order as vedo_gpu_get_observables out[0..8]). */
void dp_energy(const dp_world* w, double* out9);
/* CalcCoordinateNum (vedo/knight/CalcCoordinateNum.cpp): per object the number of other spheres
   whose centre distance is below (below) / at most (touching) the radius sum, 0 for other shapes;
   returns computeAvgCoordinateNum over box = {xmin, xmax, ymin, ymax, zmin, zmax}. */
double dp_coordination(const dp_world* w, const double* box, unsigned* below, unsigned* touching);
void dp_destroy(dp_world* w);

#ifdef __cplusplus
}
#endif
#endif
