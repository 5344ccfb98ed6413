// VTK XML output of leaf data (the file output of Mesh::toVTK, src/Mesh.hpp:398-424 and
// src/VTK.hpp:260-440 in the reference): an unstructured grid of quadrilateral cells, one per leaf
// cell, with named cell-data arrays, written as a serial piece plus the parallel wrapper (.pvtu)
// ParaView opens; the quadtree file holds one quadrilateral per leaf patch (level and leaf index as
// cell data) in place of p4est's own VTK writer.  ASCII, VTK XML format version 0.1.
#pragma once

#include <cstdio>
#include <fstream>
#include <iomanip>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

namespace EllipticForest {

struct VTKCellArray {
    std::string name;
    std::vector<double> values;  // one per cell
};

namespace vtk_detail {

inline void dataArray(std::ostream& os, const std::string& type, const std::string& name, int comps,
                      const std::vector<double>& v, const char* indent) {
    double lo = std::numeric_limits<double>::infinity(), hi = -lo;
    for (double x : v) { if (x < lo) lo = x; if (x > hi) hi = x; }
    if (v.empty()) lo = hi = 0.0;
    os << indent << "<DataArray type=\"" << type << "\" Name=\"" << name << "\" NumberOfComponents=\"" << comps
       << "\" format=\"ascii\" RangeMin=\"" << lo << "\" RangeMax=\"" << hi << "\">\n" << indent << "  ";
    for (std::size_t i = 0; i < v.size(); ++i) os << v[i] << ((i + 1) % 12 == 0 ? "\n  " : " ");
    os << "\n" << indent << "</DataArray>\n";
}

}  // namespace vtk_detail

// quads: 4 corners (x, y) per cell, counter-clockwise; data: arrays of ncells values
inline void writeQuadVTU(const std::string& filename, const std::vector<double>& corners,
                         const std::vector<VTKCellArray>& data) {
    const std::size_t ncells = corners.size() / 8;
    std::ofstream os(filename);
    if (!os) throw std::runtime_error("[toVTK] cannot open " + filename);
    os << std::setprecision(17);
    os << "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
       << "  <UnstructuredGrid>\n    <Piece NumberOfPoints=\"" << 4 * ncells << "\" NumberOfCells=\"" << ncells
       << "\">\n      <Points>\n";
    std::vector<double> pts(12 * ncells);
    for (std::size_t c = 0; c < 4 * ncells; ++c) {
        pts[3 * c] = corners[2 * c];
        pts[3 * c + 1] = corners[2 * c + 1];
        pts[3 * c + 2] = 0.0;
    }
    vtk_detail::dataArray(os, "Float64", "Points", 3, pts, "        ");
    os << "      </Points>\n      <Cells>\n";
    std::vector<double> conn(4 * ncells), off(ncells), types(ncells, 9.0);  // 9 = VTK_QUAD
    for (std::size_t c = 0; c < 4 * ncells; ++c) conn[c] = double(c);
    for (std::size_t c = 0; c < ncells; ++c) off[c] = double(4 * (c + 1));
    os << std::setprecision(12);
    vtk_detail::dataArray(os, "Int64", "connectivity", 1, conn, "        ");
    vtk_detail::dataArray(os, "Int64", "offsets", 1, off, "        ");
    vtk_detail::dataArray(os, "UInt8", "types", 1, types, "        ");
    os << std::setprecision(17);
    os << "      </Cells>\n      <CellData>\n";
    for (auto& a : data) {
        if (a.values.size() != ncells) throw std::invalid_argument("[toVTK] cell data '" + a.name + "' has the wrong size");
        vtk_detail::dataArray(os, "Float64", a.name, 1, a.values, "        ");
    }
    os << "      </CellData>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n";
}

inline void writePVTU(const std::string& filename, const std::string& piece, const std::vector<VTKCellArray>& data) {
    std::ofstream os(filename);
    if (!os) throw std::runtime_error("[toVTK] cannot open " + filename);
    os << "<?xml version=\"1.0\"?>\n<VTKFile type=\"PUnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
       << "  <PUnstructuredGrid GhostLevel=\"0\">\n    <PPoints>\n"
       << "      <PDataArray type=\"Float64\" Name=\"Points\" NumberOfComponents=\"3\"/>\n    </PPoints>\n"
       << "    <PCellData>\n";
    for (auto& a : data) os << "      <PDataArray type=\"Float64\" Name=\"" << a.name << "\" NumberOfComponents=\"1\"/>\n";
    os << "    </PCellData>\n    <Piece Source=\"" << piece << "\"/>\n  </PUnstructuredGrid>\n</VTKFile>\n";
}

}  // namespace EllipticForest
