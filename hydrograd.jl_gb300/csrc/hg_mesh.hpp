// Host-side mesh topology, geometry, boundary tables and cell renumbering.
//
// Restates the reference's mesh construction: edge numbering and boundary
// edges (src/utilities/SRH_2D/SRH_2D_SRHGeom.jl:251-382), ghost cells,
// neighbours and geometry (src/meshes/mesh_2D.jl:75-652) and the static
// boundary tables (src/fvm/boundary_conditions/bc_2D.jl:50-570).  All ids are
// 0-based.  Compiled with -ffp-contract=off so areas, normals and lengths are
// bit-identical to the reference formulas on every host architecture.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "hydrograd_gb.h"

namespace hg {

constexpr int kMaxCellFaces = 8;

struct Boundary {
  int id = 0;                   // NodeString id, or the default wall's id
  int bc = HG_BC_WALL;          // hg_bc
  std::vector<int> faces;       // face ids in NodeString order
  std::vector<signed char> dirs;  // +1 when the face normal points out of the domain
};

struct HostMesh {
  int nCells = 0, nNodes = 0, nFaces = 0, nGhost = 0, maxCellFaces = 0;
  std::vector<double> x, y, z;
  std::vector<int> ncf;               // faces (= nodes) per cell
  std::vector<int> cellNodes;         // [nCells*8]
  std::vector<int> cf;                // [nCells*8] face id of edge slot i (node i -> node i+1)
  std::vector<signed char> cfs;       // [nCells*8] +1 when (node i, node i+1) is the sorted face key
  std::vector<int> faceA, faceB;      // sorted node pair of each face
  std::vector<int> faceC0, faceC1;    // cells of a face in creation order; faceC1 = -1 on a boundary
  std::vector<int> nbr;               // [nCells*8] neighbour cell of slot i, -1 on a boundary
  std::vector<Boundary> bnd;          // boundaries in ascending id order
  std::vector<int> faceBnd;           // [nFaces] index into bnd, -1 for interior faces
  // Geometry
  std::vector<double> area, cx, cy;   // [nCells]
  std::vector<double> snx, sny;       // [nCells*8] outward normal of edge slot i
  std::vector<double> faceLen;        // [nFaces]
  std::vector<double> zbCell;         // [nCells] mean of node z
  // Boundary groups by type, in the order the reference processes them
  // (bc_2D.jl:281-295: inlet-Q, exit-H, wall, symmetry; each by ascending boundary id).
  std::vector<int> inletGroups, exitGroups, wallGroups, symmGroups;   // indices into bnd
};

// Returns HG_OK or an error code with a message in err.
int build_host_mesh(const hg_mesh_desc& d, HostMesh& m, std::string& err);

// Cell permutations perm[new] = old.
std::vector<int> order_cells(const HostMesh& m, int order);
// The same within each cell range [start[r], start[r+1]) (an ensemble's
// members, each a separate component): ranges stay in order, cells stay in
// their range.
std::vector<int> order_cells_ranges(const HostMesh& m, int order, const std::vector<int>& start);

// Disjoint union of meshes (an ensemble): cells, nodes, faces and boundaries of
// part p follow those of parts 0..p-1, with every id offset accordingly;
// boundary ids are renumbered 1, 2, ... in that order, so each type's groups
// are part-major and, within a part, in the part's own order.
void concat_host_meshes(const std::vector<const HostMesh*>& parts, HostMesh& out);

}  // namespace hg

struct hg_mesh {
  hg::HostMesh m;
};
