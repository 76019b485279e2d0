// coordination.h - the coordination-number observable and the VTK writer of the world.
#pragma once

#include <cstdint>
#include <string>

#include "dem_common.cuh"
#include "scene_host.h"

namespace vedo {

struct Scratch;

struct Box6 { double v[6]; };   // xmin, xmax, ymin, ymax, zmin, zmax

// CalcCoordinateNum (vedo/knight/CalcCoordinateNum.cpp) over the device state of n objects:
// below[i] / touching[i] (device arrays) = the number of other spheres whose centre distance is
// below / at most the radius sum, 0 for other shapes; with average, *average receives
// computeAvgCoordinateNum over box (host array of 6).  Synchronises the stream.
int coordination_device(uint32_t n, const uint32_t* model_of, const ModelDev* models, const double4_32a* pos,
                        uint32_t* below, uint32_t* touching, const double* box, double* average, Scratch& scratch,
                        cudaStream_t s, std::string& err, uint64_t* launches);

// DOWorld::WriteVTK<ExtFieldWriterT>(filename) (DOWorld_WriteVTK.h:148-243) of the scene's models
// with the given object state (host arrays, [n][3]); with coordination (per object, host), the
// "CoordinateNumber" field of the spheres in object order as outputCoordinateNumVTK adds it.
bool write_world_vtk(const std::string& path, const HScene& s, const double* pos, const double* vel,
                     const double* av, const uint32_t* coordination, std::string& err);

}  // namespace vedo
