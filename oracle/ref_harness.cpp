/*
 * C entry points around the reference DEM CPU path (test infrastructure only).
 *
 * Linked with the reference sources compiled unmodified from their own tree
 * (recipe: oracle/Makefile), this exposes exactly the step loop of the
 * reference's sequential engine, src/vedo/anne/Anne.cpp:38-128:
 *   DOWorld::ReadIDO (DOWorld_RWIDO.cpp:9-55)
 *   -> NBSConsultant / LeapConsultant / SafeConsultant (Anne.cpp:88-116)
 *   -> SimMediator sm(consultant, CreateNewAssembler())   (SimMediator.cpp:83-137)
 *   -> sm.Run() once per step                             (SimMediator.cpp:714-842)
 * and reads back, after any number of steps, the per-object state held by
 * SimMediator's DOContainer and the candidate / interaction lists held by the
 * consultant and the IactContainer.  Nothing here changes the reference's
 * arithmetic: it only drives it and copies numbers out.
 *
 * The reference writes time_0.csv, SystemStatus.csv and *.ido files into the
 * current directory; vref_open therefore switches into the caller's work
 * directory for the lifetime of the handle.
 */
#include <aries/utility/Constants.h>
#include <vedo/framework/Assembler.h>
#include <vedo/framework/Consultant.h>
#include <vedo/framework/DOWorld.h>
#include <vedo/framework/IactRecordTab.h>
#include <vedo/framework/SimMediator.h>
#include <vedo/common/LeapConsultant.h>
#include <vedo/common/NBSConsultant.h>
#include <vedo/common/SafeConsultant.h>
#include <vedo/ModuleList.h>
#include <vedo/framework/DOWorld_WriteVTK.h>
#include <vedo/knight/CalcCoordinateNum.h>

#include <unistd.h>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <string>

namespace {

struct RefHandle {
    vedo::DOWorld*       world;
    vedo::IactRecordTab* irt;
    vedo::Assembler*     assembler;
    vedo::Consultant*    consultant;
    vedo::SimMediator*   sm;
};

void put3(double* dst, size_t i, const vedo::Vector3df& v) {
    dst[3 * i + 0] = v.x();
    dst[3 * i + 1] = v.y();
    dst[3 * i + 2] = v.z();
}

}  // namespace

extern "C" {

/* Open a scene: consultant is "nbs", "leap" or "safe"; record/upiact as in
 * `anne analysis <ido> <consultant> <record> <upiact>`.  Returns NULL when the
 * IDO file cannot be read. */
void* vref_open(const char* ido_path, const char* consultant, unsigned record, unsigned upiact,
                const char* workdir) {
    if (workdir && workdir[0]) {
        if (chdir(workdir) != 0) return nullptr;
    }
    /* the reference prints "Simulated time" at every reset/record; silence it */
    static std::ofstream devnull("/dev/null");
    std::cout.rdbuf(devnull.rdbuf());
    RefHandle* h = new RefHandle();
    h->world = new vedo::DOWorld;
    h->irt = new vedo::IactRecordTab();
    h->assembler = vedo::CreateNewAssembler();
    if (!h->world->ReadIDO(ido_path, h->irt)) {
        delete h;
        return nullptr;
    }
    std::string t(consultant);
    std::string name(ido_path);
    if (t == "leap") {
        h->consultant = new vedo::LeapConsultant(h->world, h->irt, name, record, upiact);
    } else if (t == "safe") {
        h->consultant = new vedo::SafeConsultant(h->world, h->irt, name, record);
    } else {
        h->consultant = new vedo::NBSConsultant(h->world, h->irt, name, record, upiact);
    }
    h->sm = new vedo::SimMediator(h->consultant, h->assembler);
    return h;
}

/* Run nsteps calls of SimMediator::Run(); returns the last return value
 * (1 while t_current < t_stop). */
int vref_run(void* hp, unsigned nsteps) {
    RefHandle* h = static_cast<RefHandle*>(hp);
    int cont = 1;
    for (unsigned s = 0; s < nsteps; ++s) cont = h->sm->Run() ? 1 : 0;
    return cont;
}

unsigned vref_num_do(void* hp) {
    return static_cast<RefHandle*>(hp)->sm->GetDOContainer()->size();
}

/* Per-object state of SimMediator's DOContainer, each array [n][3]; the impact
 * arrays hold the impulses that the last Response consumed (ClearImpact,
 * DiscreteObject.cpp:141-147).  Any pointer may be NULL. */
void vref_get_state(void* hp, double* pos, double* vel, double* avel, double* ox, double* oz,
                    double* imp, double* aimp) {
    RefHandle* h = static_cast<RefHandle*>(hp);
    const vedo::DOContainer* c = h->sm->GetDOContainer();
    for (unsigned i = 0; i < c->size(); ++i) {
        const vedo::DOStatus* s = c->GetDOStatus(i);
        if (pos) put3(pos, i, s->GetPosition());
        if (vel) put3(vel, i, s->GetVelocity());
        if (avel) put3(avel, i, s->GetAngularVelocity());
        if (ox) put3(ox, i, s->GetOrientationX());
        if (oz) put3(oz, i, s->GetOrientationZ());
        if (imp) put3(imp, i, s->GetImpact());
        if (aimp) put3(aimp, i, s->GetAngularImpact());
    }
}

/* Candidate pair list of the consultant (IactPairTab order). */
unsigned vref_num_candidates(void* hp) {
    return static_cast<RefHandle*>(hp)->consultant->GetIactNum();
}

void vref_get_candidates(void* hp, unsigned* first, unsigned* second) {
    RefHandle* h = static_cast<RefHandle*>(hp);
    unsigned n = h->consultant->GetIactNum();
    for (unsigned k = 0; k < n; ++k) {
        first[k] = h->consultant->GetIactMaster(k);
        second[k] = h->consultant->GetIactSlave(k);
    }
}

unsigned vref_num_interactions(void* hp) {
    return static_cast<RefHandle*>(hp)->sm->GetIactContainer()->size();
}

/* Interaction list of SimMediator, in container order.  slave/master are DO
 * indices in the DOContainer; active = ContactInfo::bActive of the last
 * Detect; shear/kn/contact come from the solver's ImpactStatus; depth and
 * normal from the ContactInfo.  Any pointer may be NULL. */
void vref_get_interactions(void* hp, unsigned* slave, unsigned* master, int* active, double* depth,
                           double* normal, double* shear, double* kn, int* contact) {
    RefHandle* h = static_cast<RefHandle*>(hp);
    vedo::DOContainer* dc = const_cast<vedo::DOContainer*>(h->sm->GetDOContainer());
    std::map<const vedo::DiscreteObject*, unsigned> index;
    for (unsigned i = 0; i < dc->size(); ++i) index[(*dc)[i]] = i;
    vedo::IactContainer* ic = const_cast<vedo::IactContainer*>(h->sm->GetIactContainer());
    for (unsigned k = 0; k < ic->size(); ++k) {
        const vedo::Interaction* it = ic->GetInteraction(k);
        if (slave) slave[k] = index[it->GetSlave()];
        if (master) master[k] = index[it->GetMaster()];
        const vedo::ContactInfo* ci = it->GetContactInfo();
        if (active) active[k] = ci->bActive ? 1 : 0;
        if (depth) depth[k] = ci->dImpactDepth;
        if (normal) put3(normal, k, ci->vImpactDirection);
        const vedo::ImpactStatus* st = it->GetImpactStatus();
        if (shear) put3(shear, k, st->ShearForce());
        if (kn) kn[k] = st->Kn();
        if (contact) contact[k] = st->Contact() ? 1 : 0;
    }
}

double vref_time(void* hp) {
    return static_cast<RefHandle*>(hp)->world->GetSystemParameter()->GetTimeCurrent();
}

/* Energies as last computed by DOWorld::CalculateSystemEnergy (at construction,
 * resets and records): [potential, translation, rotation, vmin, vmax, avmin,
 * avmax, momentum norm, angular momentum norm]. */
void vref_energy(void* hp, double* out9) {
    const vedo::SystemParameter* sp = static_cast<RefHandle*>(hp)->world->GetSystemParameter();
    out9[0] = sp->GetEnergyPotential();
    out9[1] = sp->GetEnergyTranslation();
    out9[2] = sp->GetEnergyRotation();
    out9[3] = sp->GetVelocityMin();
    out9[4] = sp->GetVelocityMax();
    out9[5] = sp->GetAngularVelocityMin();
    out9[6] = sp->GetAngularVelocityMax();
    out9[7] = sp->GetMomentumNorm();
    out9[8] = sp->GetAngularMomentumNorm();
}

/* Write the world and the interaction record table as an IDO file
 * (DOWorld::WriteIDO, DOWorld_RWIDO.cpp:149-202). */
void vref_write_ido(void* hp, const char* path) {
    RefHandle* h = static_cast<RefHandle*>(hp);
    h->world->WriteIDO(path, h->irt);
}

/* The reference's XML writer (DOWorld::WriteXML with the IactRecordTab, DOWorld_WriteXML.cpp). */
void vref_write_xml(void* hp, const char* path) {
    RefHandle* h = static_cast<RefHandle*>(hp);
    h->world->WriteXML(path, h->irt);
}

/* The reference's post-processing observables on a world read from an IDO file (DOWorld::ReadIDO):
 * returns CalcCoordinateNum::computeAvgCoordinateNum over box = {xmin, xmax, ymin, ymax, zmin,
 * zmax} (CalcCoordinateNum.cpp:8-77); with coord_vtk, outputCoordinateNumVTK writes the
 * per-sphere coordination numbers with the world (:79-126); with world_vtk, the world alone as
 * the post-processing tool writes it (DOWorld::WriteVTK<NullExternalFieldVTKWriter>,
 * Knight.cpp:711).  Returns -1 when the file cannot be read. */
double vref_coordination(const char* ido_path, const double* box, const char* coord_vtk, const char* world_vtk) {
    static std::ofstream devnull("/dev/null");
    std::cout.rdbuf(devnull.rdbuf());
    vedo::DOWorld* w = new vedo::DOWorld;
    vedo::IactRecordTab* irt = new vedo::IactRecordTab();
    if (!w->ReadIDO(ido_path, irt)) return -1.0;
    CalcCoordinateNum c;
    const double avg = c.computeAvgCoordinateNum(w, box[0], box[1], box[2], box[3], box[4], box[5]);
    if (coord_vtk && coord_vtk[0]) c.outputCoordinateNumVTK(w, coord_vtk);
    if (world_vtk && world_vtk[0]) w->WriteVTK<vedo::NullExternalFieldVTKWriter>(world_vtk);
    return avg;   /* the world is leaked, as vref_close explains */
}

/* The reference's destructors release memory they do not own (the process aborts with
 * "free(): invalid pointer" when SimMediator, the consultant and DOWorld are deleted in
 * turn), so a closed handle's reference objects are deliberately leaked. */
void vref_close(void* hp) {
    RefHandle* h = static_cast<RefHandle*>(hp);
    delete h;
}

}  // extern "C"
