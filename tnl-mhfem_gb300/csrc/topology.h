// Host-side mesh topology and sparsity pattern of the face-trace system.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace mhfem {

struct HostTopology {
    int dim = 0, cell = 0;   // cell: 0 simplices, 1 boxes (rectangles / cuboids)
    int nf = 0, nv = 0, fv = 0;  // faces per cell, vertices per cell, vertices per face
    int64_t V = 0, C = 0, F = 0;
    std::vector<int32_t> cell_faces;   // [C][nf]
    std::vector<int32_t> face_cells;   // [F][2], -1 on the boundary
    std::vector<int32_t> face_verts;   // [F][fv], ascending vertex ids
    std::vector<uint8_t> face_local;   // [F][2], local index in K0, K1
    std::vector<uint8_t> cell_bmask;   // [C], bit e: local face e on the boundary
    std::vector<double> face_measure;  // [F]
    int64_t boundary_faces = 0;
};

// Builds faces from the cells.  Faces are numbered in order of first
// appearance when cells are visited in ascending order and the local faces
// of a cell in order e = 0..nf-1; the adjacent cells of a face are listed in
// ascending order.  Local face e of a simplex is the one opposite local
// vertex e (TNL's subentity order for Triangle / Tetrahedron); the local
// faces of a box follow TNL's Quadrangle (edges 01 12 23 30) and Hexahedron
// (faces 0123 0154 1265 2376 3047 4567) topologies, with the vertices of a
// rectangle counterclockwise from its lowest corner and those of a cuboid
// as that rectangle at the lower z followed by the same at the upper z.
// Returns an empty string on success, else an error message.
std::string build_topology(int dim, int cell, int64_t V, const double* coords, int64_t C,
                           const int32_t* cell_verts, HostTopology& T);

struct HostPattern {
    int n = 0;
    int W = 0;                       // ELL width = max off-diagonal entries per row
    int64_t rows = 0, nnz = 0;       // nnz counts the unit diagonal
    std::vector<uint64_t> qmap;      // [F] 4-bit merged positions of (side, local face)
    std::vector<uint8_t> qdiag;      // [F] merged position of the face itself
    std::vector<int32_t> row_len;    // [rows] full row length (with the diagonal)
    std::vector<int32_t> ell_cols;   // [W][rows], padding = own row
};

// Row structure of the reference's row setters: interior rows list the
// faces of both cells merged in ascending global order (LinearSystem.h:
// 113-245), boundary rows the faces of the single cell in ascending order
// (BoundaryConditions.hpp:155-219) or only the diagonal for FixedValue tags.
void build_pattern(const HostTopology& T, int n, const uint8_t* tags, HostPattern& P);

}  // namespace mhfem
