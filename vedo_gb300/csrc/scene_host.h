// scene_host.h - host-side scene (what the reference's DOWorld holds), the reference
// .ido reader/writer, and the flattening of models into the engine's device tables.
#pragma once

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "../../include/vedo_gpu.h"
#include "dem_common.cuh"

namespace vedo {

struct HModel {
    std::string name, group;
    uint32_t behavior = 0, scope = 0, shape = 0, color = 0;
    double density = 0, density_factor = 0;
    double ext[3] = {0, 0, 0};
    double attrs[10] = {0};
    std::vector<std::pair<std::string, double>> materials;
};

struct HIact {
    std::string master_group, slave_group, equation_type;
    std::vector<std::pair<std::string, double>> mech;
};

struct HRecords {
    std::vector<uint32_t> first, second;
    std::vector<uint8_t> contact, bond;
    std::vector<double> kn, v0, overlap;
    std::vector<double> shear, point, dirn, imp, aimp;   // [n][3]
    size_t size() const { return first.size(); }
};

struct HScene {
    double time_start = 0, time_stop = 0, time_interval = 0, time_current = 0;
    double g[3] = {0, 0, 0};
    double safety_factor = 1.1;
    uint8_t zoi_switch[3] = {0, 0, 0}, pbc_switch[3] = {0, 0, 0};
    double zoi_lower[3] = {0, 0, 0}, zoi_upper[3] = {0, 0, 0}, pbc_lower[3] = {0, 0, 0}, pbc_upper[3] = {0, 0, 0};
    uint32_t num_udd_do = 0, num_udd_impact = 0, max_id_of_do = 0;
    std::vector<HModel> models;
    std::vector<HIact> iacts;
    uint32_t n = 0;
    std::vector<uint32_t> model_of, ids;
    std::vector<double> pos, vel, ox, oz, av, imp, aimp;   // [n][3]
    HRecords rec;
};

// Reference .ido format (DOWorld_RWIDO.cpp:9-202); returns false with a message on error.
bool read_ido(const std::string& path, HScene& s, std::string& err);
bool write_ido(const std::string& path, const HScene& s, std::string& err);
bool scene_from_desc(const vedo_scene_desc* d, HScene& s, std::string& err);
// DOWorldSchema XML (DOWorld_ReadXML.cpp / DOWorld_WriteXML.cpp layout); xml_io.cpp
bool read_xml(const std::string& path, HScene& s, std::string& err);
bool write_xml(const std::string& path, const HScene& s, std::string& err);
// What the reference does to a world before its first step: Boundary::Correct on the zone of
// interest and the periodic boundary (Boundary.cpp:79-128), then Consultant::CleanUp
// (Consultant.cpp:264-319), which SimMediator's constructor runs once (SimMediator.cpp:125-134):
// mobile objects outside an active zone of interest are erased, the others renumbered, and the
// pair records re-keyed as IactRecordTab::ModifyPair does (IactRecordTab.cpp:41-69).  Returns
// the number of erased objects.
uint32_t prepare_scene(HScene& s);
// The three steps of Consultant::CleanUp, for a world whose boundaries are corrected (the Leap
// consultant runs it at every reset, LeapConsultant.cpp:61-68):
//  zoi_outside    the mobile objects outside the zone of interest (ascending), and per object the
//                 ElementMappingJump (minus the erased count up to and including it, unsigned);
//  modify_pair    IactRecordTab::ModifyPair on record keys (later equal keys replace earlier
//                 ones): the surviving (new key, index of its source record) in key order;
//  erase_objects  DOContainer::Erase / DOWorld::EraseDOStatus: the survivors keep their order.
std::vector<uint32_t> zoi_outside(const HScene& s, std::vector<uint32_t>& jump);
std::vector<std::pair<std::pair<uint32_t, uint32_t>, size_t>> modify_pair(
    const std::vector<std::pair<uint32_t, uint32_t>>& keys, const std::vector<uint32_t>& jump);
void erase_objects(HScene& s, const std::vector<uint32_t>& erased);

// Flattened constants for the device.
struct Tables {
    std::vector<ModelDev> models;
    int ngroups = 0;
    std::vector<int> group_iact;          // [ngroups*ngroups] -> interaction model index or -1
    std::vector<PairParam> params;        // [nmodels*nmodels], (slave model, master model)
    std::vector<double> geom;             // [nmodels*nmodels][4]: slave radius, master attrs a0..a2
    std::vector<double> hole;             // [nmodels*nmodels][4]: hole radius, x and y offsets (CD_SHP pairs)
    Periodic pbc{};                       // the periodic boundary (on = 0: none)
};

// DOModel::Analysis + DOcf selection + ImpactSolver constructor constants.  Fails with
// VEDO_ERR_UNSUPPORTED_MODEL / VEDO_ERR_INVALID_SCENE and a message.
int build_tables(const HScene& s, Tables& t, std::string& err);

}  // namespace vedo
