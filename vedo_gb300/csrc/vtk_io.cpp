// vtk_io.cpp - the world as a VTK unstructured-grid file, written as DOWorld::WriteVTK writes it.
//
// DOWorld::WriteVTK<ExtFieldWriterT>(filename) (vedo/framework/DOWorld_WriteVTK.h:148-243) puts every
// object in as a point: position, velocity and angular velocity with their magnitudes, the radius
// (0 for shapes other than spheres) and the two granular temperatures, then the extra fields of
// the writer (the coordination number for CalcCoordinateNum::outputCoordinateNumVTK), the points
// again, and an empty cell list.  Numbers go through std::ostream's default formatting (six
// significant digits), as the reference's ofstream writes them, so the files compare byte for byte.
//
// The granular temperatures are those of a default-constructed DOStatus (0): the reference's
// statuses read from an IDO file leave them unset (DOStatus.cpp:64-67), so its own files carry
// whatever that memory held in those two arrays.
#include <cmath>
#include <fstream>
#include <string>
#include <vector>

#include "coordination.h"

namespace vedo {
namespace {

// DataFieldVTKWriter::writeVTKDataArray (DOWorld_WriteVTK.h:79-110)
void data_array(std::ofstream& o, const char* type, const std::string& name, const std::vector<double>& data,
                unsigned ncomp, bool write_ncomp) {
    if (data.empty()) return;
    o << "\t\t\t\t<DataArray type=\"" << type << "\"";
    if (!name.empty()) o << " Name=\"" << name << "\"";
    if (write_ncomp && ncomp != 1) o << " NumberOfComponents=\"" << ncomp << "\"";
    o << " format=\"ascii\">" << std::endl;
    for (size_t i = 0; i < data.size() / ncomp; ++i) {
        o << "\t\t\t\t\t";
        for (unsigned c = 0; c < ncomp; ++c) o << data[ncomp * i + c] << "\t";
        o << std::endl;
    }
    o << "\t\t\t\t</DataArray>" << std::endl;
}

double length3(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

}  // namespace

bool write_world_vtk(const std::string& path, const HScene& s, const double* pos, const double* vel,
                     const double* av, const uint32_t* coordination, std::string& err) {
    std::ofstream o(path.c_str(), std::ios::out);
    if (!o) {
        err = "cannot write " + path;
        return false;
    }
    const size_t n = s.n;
    std::vector<double> P, V, Vs, W, Ws, R, gtv, gtav, cn;
    P.reserve(3 * n); V.reserve(3 * n); W.reserve(3 * n);
    for (size_t i = 0; i < n; ++i) {
        const HModel& m = s.models[s.model_of[i]];
        const bool sphere = m.shape == VEDO_SHAPE_SPHERE;
        R.push_back(sphere ? m.attrs[0] : 0.0);
        for (int k = 0; k < 3; ++k) P.push_back(pos[3 * i + k]);
        for (int k = 0; k < 3; ++k) V.push_back(vel[3 * i + k]);
        Vs.push_back(length3(vel + 3 * i));
        for (int k = 0; k < 3; ++k) W.push_back(av[3 * i + k]);
        Ws.push_back(length3(av + 3 * i));
        gtv.push_back(0.0);
        gtav.push_back(0.0);
        if (coordination && sphere) cn.push_back((double)coordination[i]);
    }
    o << "<?xml version=\"1.0\"?>" << std::endl
      << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">" << std::endl
      << "\t<UnstructuredGrid>" << std::endl
      << "\t\t<Piece NumberOfPoints=\"" << R.size() << "\" NumberOfCells=\"0\">" << std::endl
      << "\t\t\t<PointData Scalars=\"Radius\">" << std::endl;
    data_array(o, "Float64", "Position", P, 3, true);
    data_array(o, "Float64", "Velocity", V, 3, true);
    data_array(o, "Float64", "VelocityScale", Vs, 1, false);
    data_array(o, "Float64", "AngularVelocity", W, 3, true);
    data_array(o, "Float64", "AngularVelocityScale", Ws, 1, false);
    data_array(o, "Float64", "Radius", R, 1, false);
    data_array(o, "Float64", "GranularTemperatureV", gtv, 1, false);
    data_array(o, "Float64", "GranularTemperatureAV", gtav, 1, false);
    if (coordination) data_array(o, "Float64", "CoordinateNumber", cn, 1, true);
    o << "\t\t\t</PointData>" << std::endl
      << "\t\t\t<Points>" << std::endl
      << "\t\t\t\t<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">" << std::endl;
    for (double x : P) o << x << " ";
    o << std::endl
      << "\t\t\t\t</DataArray>" << std::endl
      << "\t\t\t</Points>" << std::endl
      << "\t\t\t<Cells>" << std::endl
      << "\t\t\t\t<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">" << std::endl
      << "\t\t\t\t</DataArray>" << std::endl
      << "\t\t\t</Cells>" << std::endl
      << "\t\t</Piece>" << std::endl
      << "\t</UnstructuredGrid>" << std::endl
      << "</VTKFile>" << std::endl;
    o.close();
    if (!o) {
        err = "write failed: " + path;
        return false;
    }
    return true;
}

}  // namespace vedo
