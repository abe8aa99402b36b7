// Oracle for the 2D shallow-water ODE right-hand side and its time stepping.
//
// TEST INFRASTRUCTURE ONLY.  This header is a CPU (FP64, optionally OpenMP)
// restatement of Hydrograd.jl's hot path.  It exists to check the CUDA product
// path and to time a CPU baseline; nothing in the shipped library includes,
// links or calls it.  Every function cites the reference file:line it follows
// (paths are relative to the Hydrograd.jl project root).
//
// Parity pin: the restatement is checked against the reference's own shipped
// golden data (forward-simulation truth JSON: S0_cells_truth, friction_x/y
// truth, steady-state xi_truth; ManningN sensitivity Jacobians) by the tests
// under tests/, using fixtures generated by tests/golden/make_golden.py.
//
// The scalar type T is templated so that a forward-mode dual number
// (hgo::Dual<N>, see dual.hpp) reproduces what ForwardDiff.jl computes through
// the same code.  Build with -ffp-contract=off so that no a*b+c is fused: Julia
// does not contract either, and the x86 build and the aarch64 build then agree.
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "dual.hpp"

namespace hgo {

// Boundary types (src/fvm/boundary_conditions/bc_2D.jl:154-260).
enum BcType : int { BC_WALL = 0, BC_SYMM = 1, BC_INLETQ = 2, BC_EXITH = 3 };

// eps(Float64): the smooth_* helpers add eps(T) (src/utilities/smooth_functions.jl:4-52).
// For a dual number ForwardDiff's eps(Dual) is eps of the value type, i.e. this constant.
constexpr double kEps = 2.220446049250313e-16;

template <class T> inline T smooth_abs(const T& x) { using std::sqrt; return sqrt(x * x + kEps); }   // smooth_functions.jl:4-12
template <class T> inline T smooth_sqrt(const T& x) { using std::sqrt; return sqrt(x + kEps); }      // smooth_functions.jl:39-44
template <class T> inline T smooth_pow2(const T& x) { T y = x + kEps; return y * y; }               // smooth_functions.jl:47-52 (n = 2)

// ---------------------------------------------------------------------------
// Mesh topology and geometry.
// Restates SRH_2D_SRHGeom.jl:251-382 (edge numbering, boundary edges, default
// wall) and mesh_2D.jl:75-652 (ghost cells, neighbours, areas, centroids,
// outward cell normals, face normals/lengths).  Ids are 0-based here; the
// reference's 1-based ids are kept in the same relative order.
// ---------------------------------------------------------------------------
struct NodeString {
  int id;                 // NodeString id as in the .srhgeom file (1-based in SRH-2D)
  int bc;                 // BcType, or -1 for a NodeString that is not a boundary (monitoring line)
  std::vector<int> nodes; // 0-based node ids, in file order
};

struct Mesh {
  int nCells = 0, nNodes = 0, nFaces = 0, maxNodes = 8;
  std::vector<double> nodeX, nodeY, nodeZ;
  std::vector<int> cellNodesCount;       // [nCells]
  std::vector<int> cellNodes;            // [nCells*8] 0-based node ids
  std::vector<int> cellFaces;            // [nCells*8] 0-based face ids (sign dropped, mesh_2D.jl:161)
  std::vector<int> cellFaceSign;         // [nCells*8] +1 / -1 as elementEdgesList before abs
  std::vector<std::array<int, 2>> faceNodes;   // sorted (min,max) node ids (SRH_2D_SRHGeom.jl:271)
  std::vector<std::vector<int>> faceCells;     // 1 or 2 cells in creation order (SRH_2D_SRHGeom.jl:278,284)
  std::vector<char> faceIsBoundary;            // mesh_2D.jl:265-276
  // Boundaries, keyed by boundary id; faces in NodeString order (SRH_2D_SRHGeom.jl:304-349).
  std::map<int, std::vector<int>> boundaryFaces;
  std::map<int, std::vector<int>> boundaryDirs;  // +1 when the face normal points out (mesh_2D.jl:141-158)
  std::map<int, int> boundaryType;               // BcType per boundary id
  std::vector<int> allBoundaryFaces;             // ghost g <-> allBoundaryFaces[g]
  std::vector<int> faceGhost;                    // [nFaces] ghost id or -1
  std::vector<int> faceBoundaryId;               // [nFaces] boundary id or 0 (internal)
  std::vector<int> cellNeighbors;                // [nCells*8] neighbour cell id, or ghost id for boundary faces
  // Geometry (mesh_2D.jl:456-652)
  std::vector<double> cellAreas, cellCx, cellCy;
  std::vector<double> cellNormals;   // [nCells*8*2] outward normal of cell edge i (node i -> node i+1)
  std::vector<double> cellDist;      // [nCells*8]
  std::vector<double> faceNx, faceNy, faceLengths;
};

// Build the mesh from node coordinates, cell node lists (0-based node ids,
// counter-clockwise) and NodeStrings.
inline Mesh build_mesh(int nNodes, const double* x, const double* y, const double* z, int nCells,
                       const int* cellNodesCount, const int* cellNodes8,
                       const std::vector<NodeString>& strings) {
  Mesh m;
  m.nNodes = nNodes;
  m.nCells = nCells;
  m.nodeX.assign(x, x + nNodes);
  m.nodeY.assign(y, y + nNodes);
  m.nodeZ.assign(z, z + nNodes);
  m.cellNodesCount.assign(cellNodesCount, cellNodesCount + nCells);
  m.cellNodes.assign(cellNodes8, cellNodes8 + (size_t)nCells * 8);

  // Edges: SRH_2D_SRHGeom.jl:251-287.  Edge ids are handed out in the order
  // edges are first met while looping cells and their edges.
  std::unordered_map<uint64_t, int> edges;
  edges.reserve((size_t)nCells * 4);
  auto key = [](int a, int b) -> uint64_t { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; };
  for (int c = 0; c < nCells; ++c) {
    int n = m.cellNodesCount[c];
    for (int i = 0; i < n; ++i) {
      int n1 = m.cellNodes[(size_t)c * 8 + i];
      int n2 = m.cellNodes[(size_t)c * 8 + (i + 1) % n];
      int a = std::min(n1, n2), b = std::max(n1, n2);
      auto it = edges.find(key(a, b));
      if (it == edges.end()) {
        int id = (int)m.faceNodes.size();
        edges.emplace(key(a, b), id);
        m.faceNodes.push_back({a, b});
        m.faceCells.push_back({c});
      } else {
        if (m.faceCells[it->second].size() != 1) throw std::runtime_error("edge shared by more than two cells");
        m.faceCells[it->second].push_back(c);
      }
    }
  }
  m.nFaces = (int)m.faceNodes.size();
  m.faceIsBoundary.assign(m.nFaces, 0);
  for (int f = 0; f < m.nFaces; ++f) m.faceIsBoundary[f] = m.faceCells[f].size() == 1;

  // elementEdgesList with sign: + when (n1,n2) is the sorted key (SRH_2D_SRHGeom.jl:355-377).
  m.cellFaces.assign((size_t)nCells * 8, 0);
  m.cellFaceSign.assign((size_t)nCells * 8, 0);
  for (int c = 0; c < nCells; ++c) {
    int n = m.cellNodesCount[c];
    for (int i = 0; i < n; ++i) {
      int n1 = m.cellNodes[(size_t)c * 8 + i];
      int n2 = m.cellNodes[(size_t)c * 8 + (i + 1) % n];
      int a = std::min(n1, n2), b = std::max(n1, n2);
      int id = edges.at(key(a, b));
      m.cellFaces[(size_t)c * 8 + i] = id;
      m.cellFaceSign[(size_t)c * 8 + i] = (n1 < n2) ? 1 : -1;
    }
  }

  // Boundary edges from NodeStrings (SRH_2D_SRHGeom.jl:303-338); monitoring
  // lines (bc < 0) are skipped; an edge not found is a mesh error.
  std::vector<char> used(m.nFaces, 0);
  int nBoundaryStrings = 0;
  for (const auto& s : strings) {
    if (s.bc < 0) continue;
    ++nBoundaryStrings;
    std::vector<int> list;
    for (size_t i = 0; i + 1 < s.nodes.size(); ++i) {
      int a = std::min(s.nodes[i], s.nodes[i + 1]), b = std::max(s.nodes[i], s.nodes[i + 1]);
      auto it = edges.find(key(a, b));
      if (it == edges.end()) throw std::runtime_error("NodeString edge not found in mesh");
      list.push_back(it->second);
      used[it->second] = 1;
    }
    m.boundaryFaces[s.id] = list;
    m.boundaryType[s.id] = s.bc;
  }
  // Default wall boundary for unused boundary edges (SRH_2D_SRHGeom.jl:344-349; mesh_2D.jl:172-181).
  std::vector<int> unused;
  for (int f = 0; f < m.nFaces; ++f)
    if (m.faceIsBoundary[f] && !used[f]) unused.push_back(f);
  if (!unused.empty()) {
    int defaultId = nBoundaryStrings + 1;
    m.boundaryFaces[defaultId] = unused;
    m.boundaryType[defaultId] = BC_WALL;
  }
  // Directions (mesh_2D.jl:141-158): -1 when the owning cell walks the edge
  // against its sorted node order, i.e. the face normal points inward.
  for (auto& kv : m.boundaryFaces) {
    std::vector<int> dirs(kv.second.size(), 1);
    for (size_t i = 0; i < kv.second.size(); ++i) {
      int f = kv.second[i];
      if (!m.faceIsBoundary[f]) throw std::runtime_error("NodeString edge is not a boundary edge");
      int c = m.faceCells[f][0];
      for (int k = 0; k < m.cellNodesCount[c]; ++k)
        if (m.cellFaces[(size_t)c * 8 + k] == f && m.cellFaceSign[(size_t)c * 8 + k] < 0) dirs[i] = -1;
    }
    m.boundaryDirs[kv.first] = dirs;
  }
  // Ghost cells: one per boundary face.  The reference numbers them in Julia
  // Dict iteration order (SRH_2D_SRHGeom.jl:290); ghost numbering is internal
  // and never changes a result, so ascending face id is used here.
  m.faceGhost.assign(m.nFaces, -1);
  for (int f = 0; f < m.nFaces; ++f)
    if (m.faceIsBoundary[f]) {
      m.faceGhost[f] = (int)m.allBoundaryFaces.size();
      m.allBoundaryFaces.push_back(f);
    }
  m.faceBoundaryId.assign(m.nFaces, 0);
  for (auto& kv : m.boundaryFaces)
    for (int f : kv.second) m.faceBoundaryId[f] = kv.first;
  for (int f = 0; f < m.nFaces; ++f)
    if (m.faceIsBoundary[f] && m.faceBoundaryId[f] == 0) throw std::runtime_error("boundary face without boundary");

  // Neighbours (mesh_2D.jl:229-254).
  m.cellNeighbors.assign((size_t)nCells * 8, -1);
  for (int c = 0; c < nCells; ++c)
    for (int i = 0; i < m.cellNodesCount[c]; ++i) {
      int f = m.cellFaces[(size_t)c * 8 + i];
      const auto& fc = m.faceCells[f];
      if (fc.size() == 2) m.cellNeighbors[(size_t)c * 8 + i] = (fc[0] == c) ? fc[1] : fc[0];
      else m.cellNeighbors[(size_t)c * 8 + i] = m.faceGhost[f];
    }

  // Geometry (mesh_2D.jl:456-547).
  m.cellAreas.assign(nCells, 0.0);
  m.cellCx.assign(nCells, 0.0);
  m.cellCy.assign(nCells, 0.0);
  m.cellNormals.assign((size_t)nCells * 16, 0.0);
  for (int c = 0; c < nCells; ++c) {
    int n = m.cellNodesCount[c];
    double area = 0.0, cx = 0.0, cy = 0.0, asum = 0.0;
    for (int i = 0; i < n; ++i) {   // compute_polygon_area_srhgeom, mesh_2D.jl:600-616
      int a = m.cellNodes[(size_t)c * 8 + i], b = m.cellNodes[(size_t)c * 8 + (i + 1) % n];
      area += m.nodeX[a] * m.nodeY[b] - m.nodeX[b] * m.nodeY[a];
    }
    if (area < 0) throw std::runtime_error("cell nodes are not counter-clockwise");
    m.cellAreas[c] = std::fabs(area) / 2;
    for (int i = 0; i < n; ++i) {   // compute_polygon_centroid_srhgeom, mesh_2D.jl:619-634
      int a = m.cellNodes[(size_t)c * 8 + i], b = m.cellNodes[(size_t)c * 8 + (i + 1) % n];
      double x1 = m.nodeX[a], y1 = m.nodeY[a], x2 = m.nodeX[b], y2 = m.nodeY[b];
      double cross = x1 * y2 - x2 * y1;
      cx += (x1 + x2) * cross;
      cy += (y1 + y2) * cross;
      asum += cross;
    }
    double a2 = std::fabs(asum) / 2;
    m.cellCx[c] = cx / (6 * a2);
    m.cellCy[c] = cy / (6 * a2);
    for (int i = 0; i < n; ++i) {   // compute_face_normals_srhgeom, mesh_2D.jl:550-575
      int a = m.cellNodes[(size_t)c * 8 + i], b = m.cellNodes[(size_t)c * 8 + (i + 1) % n];
      double fx = m.nodeX[b] - m.nodeX[a], fy = m.nodeY[b] - m.nodeY[a];
      double nx = fy, ny = -fx;
      double len = std::sqrt(nx * nx + ny * ny);
      m.cellNormals[(size_t)c * 16 + 2 * i] = nx / len;
      m.cellNormals[(size_t)c * 16 + 2 * i + 1] = ny / len;
    }
  }
  m.faceNx.assign(m.nFaces, 0.0);
  m.faceNy.assign(m.nFaces, 0.0);
  m.faceLengths.assign(m.nFaces, 0.0);
  for (int f = 0; f < m.nFaces; ++f) {   // compute_face_normal_srhgeom, mesh_2D.jl:637-652
    int a = m.faceNodes[f][0], b = m.faceNodes[f][1];
    double nx = m.nodeY[b] - m.nodeY[a], ny = -(m.nodeX[b] - m.nodeX[a]);
    double len = std::sqrt(nx * nx + ny * ny);
    m.faceNx[f] = nx / len;
    m.faceNy[f] = ny / len;
    m.faceLengths[f] = len;
  }
  m.cellDist.assign((size_t)nCells * 8, 0.0);
  for (int c = 0; c < nCells; ++c)   // mesh_2D.jl:494-530
    for (int i = 0; i < m.cellNodesCount[c]; ++i) {
      int f = m.cellFaces[(size_t)c * 8 + i];
      double dx, dy;
      if (m.faceIsBoundary[f]) {
        int a = m.faceNodes[f][0], b = m.faceNodes[f][1];
        dx = m.cellCx[c] - (m.nodeX[a] + m.nodeX[b]) / 2;
        dy = m.cellCy[c] - (m.nodeY[a] + m.nodeY[b]) / 2;
      } else {
        int nb = m.cellNeighbors[(size_t)c * 8 + i];
        dx = m.cellCx[c] - m.cellCx[nb];
        dy = m.cellCy[c] - m.cellCy[nb];
      }
      m.cellDist[(size_t)c * 8 + i] = std::sqrt(dx * dx + dy * dy);
    }
  return m;
}

// Boundary-condition tables (bc_2D.jl:50-570): per boundary of each type, its
// faces, ghosts, internal cells and outward normals (face_direction .* face_normal).
struct BcGroup {
  int boundaryId;
  std::vector<int> faces, ghosts, internals;
  std::vector<double> onx, ony, lengths;
};
struct Bcs {
  std::vector<BcGroup> inletQ, exitH, wall, symm;
};

inline Bcs build_bcs(const Mesh& m) {
  Bcs b;
  for (auto& kv : m.boundaryFaces) {   // boundary ids in ascending order, as compute_boundary_indices_2D! loops 1:numOfBoundaries
    BcGroup g;
    g.boundaryId = kv.first;
    const auto& dirs = m.boundaryDirs.at(kv.first);
    for (size_t i = 0; i < kv.second.size(); ++i) {
      int f = kv.second[i];
      g.faces.push_back(f);
      g.ghosts.push_back(m.faceGhost[f]);
      g.internals.push_back(m.faceCells[f][0]);
      g.onx.push_back(dirs[i] * m.faceNx[f]);
      g.ony.push_back(dirs[i] * m.faceNy[f]);
      g.lengths.push_back(m.faceLengths[f]);
    }
    switch (m.boundaryType.at(kv.first)) {
      case BC_INLETQ: b.inletQ.push_back(g); break;
      case BC_EXITH: b.exitH.push_back(g); break;
      case BC_SYMM: b.symm.push_back(g); break;
      default: b.wall.push_back(g); break;
    }
  }
  return b;
}

// ---------------------------------------------------------------------------
// Bed data (process_bed_2D.jl:46-66; fvm_schemes_2D.jl:111-138,197-213,253-275).
// ---------------------------------------------------------------------------
template <class T>
struct BedData {
  std::vector<T> zbGhost, zbFaces, S0x, S0y;
};

template <class T>
BedData<T> update_bed_data(const Mesh& m, const T* zb) {
  BedData<T> d;
  d.zbGhost.resize(m.allBoundaryFaces.size());
  for (size_t g = 0; g < m.allBoundaryFaces.size(); ++g)          // update_ghost_cells_scalar
    d.zbGhost[g] = zb[m.faceCells[m.allBoundaryFaces[g]][0]];
  d.zbFaces.resize(m.nFaces);
  for (int f = 0; f < m.nFaces; ++f) {                            // cells_to_faces_scalar
    const auto& fc = m.faceCells[f];
    d.zbFaces[f] = fc.size() == 2 ? (zb[fc[0]] + zb[fc[1]]) / 2.0 : zb[fc[0]];
  }
  d.S0x.resize(m.nCells);
  d.S0y.resize(m.nCells);
  for (int c = 0; c < m.nCells; ++c) {                            // compute_cell_gradient_from_faces
    T gx = T(0.0), gy = T(0.0);
    for (int i = 0; i < m.cellNodesCount[c]; ++i) {
      int f = m.cellFaces[(size_t)c * 8 + i];
      double nx = m.cellNormals[(size_t)c * 16 + 2 * i], ny = m.cellNormals[(size_t)c * 16 + 2 * i + 1];
      gx = gx + nx * d.zbFaces[f] * m.faceLengths[f];
      gy = gy + ny * d.zbFaces[f] * m.faceLengths[f];
    }
    d.S0x[c] = -1.0 * (gx / m.cellAreas[c]);                      // S0 = -1.0 * gradient (process_bed_2D.jl:55)
    d.S0y[c] = -1.0 * (gy / m.cellAreas[c]);
  }
  return d;
}

// zb at cells = mean of node z (fvm_schemes_2D.jl:216-224).
inline std::vector<double> nodes_to_cells(const Mesh& m, const std::vector<double>& zn) {
  std::vector<double> zc(m.nCells);
  for (int c = 0; c < m.nCells; ++c) {
    double s = 0.0;
    for (int i = 0; i < m.cellNodesCount[c]; ++i) s += zn[m.cellNodes[(size_t)c * 8 + i]];
    zc[c] = s / m.cellNodesCount[c];
  }
  return zc;
}

// ---------------------------------------------------------------------------
// Roe flux (src/fvm/discretization/Riemman_solvers/swe_2D_solvers.jl:4-164).
// ---------------------------------------------------------------------------
template <class T>
inline void roe_flux(T xiL, T hstillL, T hL, T huL, T hvL, T zbL, T xiR, T hstillR, T hR, T huR, T hvR, T zbR,
                     double g, double nx, double ny, double hmin, T out[3]) {
  using std::sqrt;
  if (value(hL) <= hmin && value(hR) <= hmin) {                          // :16-22 both dry
    out[0] = T(0.0); out[1] = T(0.0); out[2] = T(0.0);
    return;
  } else if (value(hL + zbL) < value(zbR + hmin) && value(hR) <= hmin) {   // :23-38 wall: R <- mirrored L (xiR kept)
    hR = hL; huR = -huL; hvR = -hvL;
  } else if (value(hR + zbR) < value(zbL + hmin) && value(hL) <= hmin) {   // :39-53 wall: L <- mirrored R (xiL kept)
    hL = hR; huL = -huR; hvL = -hvR;
  } else if (value(hL) <= hmin) {                                        // :54-64 left dry: physical flux of R
    T p = 0.5 * g * smooth_pow2(hR);
    out[0] = huR * nx + hvR * ny;
    out[1] = (huR * (huR / hR) + p) * nx + huR * (hvR / hR) * ny;
    out[2] = (hvR * (huR / hR)) * nx + (hvR * (hvR / hR) + p) * ny;
    return;
  } else if (value(hR) <= hmin) {                                        // :65-75 right dry: physical flux of L
    T p = 0.5 * g * smooth_pow2(hL);
    out[0] = huL * nx + hvL * ny;
    out[1] = (huL * (huL / hL) + p) * nx + huL * (hvL / hL) * ny;
    out[2] = (hvL * (huL / hL)) * nx + (hvL * (hvL / hL) + p) * ny;
    return;
  }
  T uL = huL / hL, vL = hvL / hL, uR = huR / hR, vR = hvR / hR;          // :79-82
  T sqrt_hL = smooth_sqrt(hL), sqrt_hR = smooth_sqrt(hR);                // :89-90
  T hRoe = (hL + hR) / 2.0;                                              // :91 arithmetic average
  T uRoe = (sqrt_hL * uL + sqrt_hR * uR) / (sqrt_hL + sqrt_hR);
  T vRoe = (sqrt_hL * vL + sqrt_hR * vR) / (sqrt_hL + sqrt_hR);
  T unRoe = uRoe * nx + vRoe * ny;
  T cRoe = smooth_sqrt(g * hRoe);
  T o2c = 0.5 / cRoe;                                                    // one/2.0/cRoe
  // R, L, |Lambda| (:103-113); absA_dQ = R * (|Lambda| * (L * dQ)) (:118)
  T R10 = T(ny), R11 = uRoe - cRoe * nx, R12 = uRoe + cRoe * nx;
  T R20 = T(-nx), R21 = vRoe - cRoe * ny, R22 = vRoe + cRoe * ny;
  T L00 = -(uRoe * ny - vRoe * nx), L01 = T(ny), L02 = T(-nx);
  T L10 = unRoe * o2c + 0.5, L11 = -nx * o2c, L12 = -ny * o2c;
  T L20 = -unRoe * o2c + 0.5, L21 = nx * o2c, L22 = ny * o2c;
  T a0 = smooth_abs(unRoe), a1 = smooth_abs(unRoe - cRoe), a2 = smooth_abs(unRoe + cRoe);
  T d0 = xiR - xiL, d1 = huR - huL, d2 = hvR - hvL;                      // :115 dQ uses xi
  T w0 = L00 * d0 + L01 * d1 + L02 * d2;
  T w1 = L10 * d0 + L11 * d1 + L12 * d2;
  T w2 = L20 * d0 + L21 * d1 + L22 * d2;
  w0 = a0 * w0; w1 = a1 * w1; w2 = a2 * w2;
  T A0 = w1 + w2;                                                        // row 1 of R is (0 1 1)
  T A1 = R10 * w0 + R11 * w1 + R12 * w2;
  T A2 = R20 * w0 + R21 * w1 + R22 * w2;
  T pL = 0.5 * g * (smooth_pow2(xiL) + 2.0 * xiL * hstillL);           // :122-127 pre-balanced pressure
  T pR = 0.5 * g * (smooth_pow2(xiR) + 2.0 * xiR * hstillR);
  T fL0 = huL * nx + hvL * ny;
  T fL1 = (huL * uL + pL) * nx + huL * vL * ny;
  T fL2 = (hvL * uL) * nx + (hvL * vL + pL) * ny;
  T fR0 = huR * nx + hvR * ny;
  T fR1 = (huR * uR + pR) * nx + huR * vR * ny;
  T fR2 = (hvR * uR) * nx + (hvR * vR + pR) * ny;
  out[0] = (fL0 + fR0 - A0) / 2.0;                                       // :131-133
  out[1] = (fL1 + fR1 - A1) / 2.0;
  out[2] = (fL2 + fR2 - A2) / 2.0;
}

// ---------------------------------------------------------------------------
// HLL flux -- new: the reference's RiemannSolver "HLL" raises an error
// (semi_discretize_swe_2D.jl:356-357), so this follows the published scheme:
// Harten, Lax & van Leer (1983), with Einfeldt's (1988) wave-speed estimates
// S_L = min(un_L - c_L, un_Roe - c_Roe), S_R = max(un_R + c_R, un_Roe + c_Roe).
// It works on the same variables as roe_flux -- the pre-balanced pressure
// 0.5 g (xi^2 + 2 xi hstill) and the xi jump in the continuity component, so a
// lake at rest (xi = 0, q = 0) has zero flux -- and takes roe_flux's dry, wall
// and one-side-dry branches unchanged; only the wet-wet flux differs:
//   F = F_L (S_L >= 0),  F_R (S_R <= 0),
//   else (S_R F_L - S_L F_R + S_L S_R (U_R - U_L)) / (S_R - S_L).
// ---------------------------------------------------------------------------
template <class T>
inline void hll_flux(T xiL, T hstillL, T hL, T huL, T hvL, T zbL, T xiR, T hstillR, T hR, T huR, T hvR, T zbR,
                     double g, double nx, double ny, double hmin, T out[3]) {
  if (value(hL) <= hmin && value(hR) <= hmin) {                          // roe_flux's branches
    out[0] = T(0.0); out[1] = T(0.0); out[2] = T(0.0);
    return;
  } else if (value(hL + zbL) < value(zbR + hmin) && value(hR) <= hmin) {
    hR = hL; huR = -huL; hvR = -hvL;
  } else if (value(hR + zbR) < value(zbL + hmin) && value(hL) <= hmin) {
    hL = hR; huL = -huR; hvL = -hvR;
  } else if (value(hL) <= hmin) {
    T p = 0.5 * g * smooth_pow2(hR);
    out[0] = huR * nx + hvR * ny;
    out[1] = (huR * (huR / hR) + p) * nx + huR * (hvR / hR) * ny;
    out[2] = (hvR * (huR / hR)) * nx + (hvR * (hvR / hR) + p) * ny;
    return;
  } else if (value(hR) <= hmin) {
    T p = 0.5 * g * smooth_pow2(hL);
    out[0] = huL * nx + hvL * ny;
    out[1] = (huL * (huL / hL) + p) * nx + huL * (hvL / hL) * ny;
    out[2] = (hvL * (huL / hL)) * nx + (hvL * (hvL / hL) + p) * ny;
    return;
  }
  T uL = huL / hL, vL = hvL / hL, uR = huR / hR, vR = hvR / hR;
  T sqrt_hL = smooth_sqrt(hL), sqrt_hR = smooth_sqrt(hR);
  T hRoe = (hL + hR) / 2.0;
  T uRoe = (sqrt_hL * uL + sqrt_hR * uR) / (sqrt_hL + sqrt_hR);
  T vRoe = (sqrt_hL * vL + sqrt_hR * vR) / (sqrt_hL + sqrt_hR);
  T unRoe = uRoe * nx + vRoe * ny;
  T cRoe = smooth_sqrt(g * hRoe);
  T unL = uL * nx + vL * ny, unR = uR * nx + vR * ny;
  T cL = smooth_sqrt(g * hL), cR = smooth_sqrt(g * hR);
  T sL1 = unL - cL, sL2 = unRoe - cRoe, sR1 = unR + cR, sR2 = unRoe + cRoe;
  T sL = value(sL1) <= value(sL2) ? sL1 : sL2;
  T sR = value(sR1) >= value(sR2) ? sR1 : sR2;
  T pL = 0.5 * g * (smooth_pow2(xiL) + 2.0 * xiL * hstillL);
  T pR = 0.5 * g * (smooth_pow2(xiR) + 2.0 * xiR * hstillR);
  T fL[3] = {huL * nx + hvL * ny, (huL * uL + pL) * nx + huL * vL * ny, (hvL * uL) * nx + (hvL * vL + pL) * ny};
  T fR[3] = {huR * nx + hvR * ny, (huR * uR + pR) * nx + huR * vR * ny, (hvR * uR) * nx + (hvR * vR + pR) * ny};
  if (value(sL) >= 0.0) {
    for (int k = 0; k < 3; ++k) out[k] = fL[k];
  } else if (value(sR) <= 0.0) {
    for (int k = 0; k < 3; ++k) out[k] = fR[k];
  } else {
    T d[3] = {xiR - xiL, huR - huL, hvR - hvL};
    T den = sR - sL;
    for (int k = 0; k < 3; ++k) out[k] = (sR * fL[k] - sL * fR[k] + sL * sR * d[k]) / den;
  }
}

// ---------------------------------------------------------------------------
// The RHS (src/fvm/discretization/semi_discretize_swe_2D.jl:18-277).
// ---------------------------------------------------------------------------
enum Riemann : int { RIEMANN_ROE = 0, RIEMANN_HLL = 1 };
struct Consts {
  double g = 9.81, k_n = 1.0, h_small = 1.0e-3;   // solve_swe_2D.jl:51-107
  int riemann = RIEMANN_ROE;                      // swe_2D_constants.jl:16 RiemannSolver ("Roe"; "HLL" new)
};

// ---------------------------------------------------------------------------
// State-dependent flow resistance.
// ---------------------------------------------------------------------------
// Kinds: Manning's n as a function of the state (ManningN_option "variable",
// process_ManningN_2D.jl:102-213, applied at semi_discretize_swe_2D.jl:141-149),
// and the UDE closures (process_ManningN_2D.jl:216-273 for n; the flow
// resistance magnitude of process_FlowResistance_UDE.jl:3-45, applied at
// semi_discretize_swe_2D.jl:516-533).
enum ResKind : int {
  RES_CONSTANT = 0, RES_POWER_LAW = 1, RES_SIGMOID = 2, RES_INVERSE = 3, RES_H_UMAG_KS = 4,
  RES_UDE_MANNING_H = 5, RES_UDE_MANNING_H_UMAG_KS = 6, RES_UDE_FLOW_RESISTANCE = 7
};
enum Act : int { ACT_RELU = 0, ACT_LEAKYRELU = 1, ACT_SIGMOID = 2, ACT_TANH = 3, ACT_SOFTPLUS = 4 };

// NNlib's activations (relu, leakyrelu with a = 0.01, sigmoid, tanh, softplus).
inline double sigmoid_nn(double x) {
  const double t = std::exp(-std::fabs(x));
  return x >= 0 ? 1.0 / (1.0 + t) : t / (1.0 + t);
}
inline double activation(int a, double x) {
  switch (a) {
    case ACT_RELU: return x > 0 ? x : 0.0;
    case ACT_LEAKYRELU: return x > 0 ? x : 0.01 * x;
    case ACT_SIGMOID: return sigmoid_nn(x);
    case ACT_TANH: return std::tanh(x);
    default: return std::log1p(std::exp(-std::fabs(x))) + (x > 0 ? x : 0.0);   // softplus
  }
}

// The UDE network (process_UDE.jl:3-56): a Lux Chain of [Dense(in, w_l, act_l),
// LayerNorm(w_l)] per hidden layer, a linear Dense(w_L, 1), and the output
// bound lo + (hi - lo) sigmoid(y).  params: Lux's flattened order -- per layer,
// Dense weight (out x in, column-major) then bias; LayerNorm scale then bias.
// LayerNorm: y = (x - mu) / sqrt(var + eps) * scale + bias with eps = 1f-5 and
// the uncorrected variance; with overBatch its statistics are taken over the
// whole (width x cells) array, as Lux's LayerNorm does with its default
// dims = Colon(), otherwise over each cell's features.
struct Mlp {
  int inDim = 1;
  std::vector<int> hidden, act;
  std::vector<double> params;
  double outLo = 0.0, outHi = 1.0;
  bool overBatch = true;
  double lnEps = (double)1e-5f;
  size_t n_params() const {
    size_t n = 0;
    int in = inDim;
    for (int w : hidden) { n += (size_t)w * in + w + 2 * w; in = w; }
    return n + (size_t)in + 1;
  }
};

struct Resistance {
  int kind = RES_CONSTANT;
  double nLower = 0.0, nUpper = 0.0, k = 0.0, hMid = 0.0;   // function parameters
  std::vector<double> ks;                                  // roughness height per cell
  Mlp mlp;
  double hB[2] = {0, 1}, uB[2] = {0, 1}, ksB[2] = {0, 1};  // input normalisation bounds
};

// Manning's n functions of process_ManningN_2D.jl:140-213 at one cell; for
// h_Umag_ks also h/ks, the friction factor and Re (Cheng 2008, Eq. 17).
inline double manning_fn(const Resistance& r, double h, double umag, double ks, double* hks = nullptr,
                         double* ff = nullptr, double* re = nullptr) {
  switch (r.kind) {
    case RES_POWER_LAW: return r.nLower + (r.nUpper - r.nLower) * std::pow(h + kEps, -r.k);            // :164-175
    case RES_SIGMOID: return r.nLower + (r.nUpper - r.nLower) / (1.0 + std::exp(r.k * (h - r.hMid)));  // :180-193
    case RES_INVERSE: return r.nLower + (r.nUpper - r.nLower) / (1.0 + r.k * h);                        // :149-160
    default: {                                                                                          // :197-213
      const double nu = 1.0e-6;
      const double Re = umag * h / nu;
      const double h_ks = h / ks;
      const double alpha = 1.0 / (1.0 + std::pow(Re / 850.0, 9.0));
      const double rb = Re / (h_ks * 160.0);
      const double beta = 1.0 / (1.0 + rb * rb);
      const double part1 = std::pow(Re / 24.0, alpha);
      const double part2 = std::pow(1.8 * std::log10(Re / 2.1), 2.0 * (1.0 - alpha) * beta);
      const double part3 = std::pow(2.0 * std::log10(11.8 * h_ks), 2.0 * (1.0 - alpha) * (1.0 - beta));
      const double f = 1.0 / (part1 * part2 * part3);
      if (hks) *hks = h_ks;
      if (ff) *ff = f;
      if (re) *re = Re;
      return std::sqrt(f / 8.0) * std::pow(h, 1.0 / 6.0) / std::sqrt(9.81);
    }
  }
}

// Forward pass of the network over all cells: in[c * inDim + j] are the
// normalised inputs, out[c] the bounded outputs.
inline void mlp_forward(const Mlp& M, const std::vector<double>& in, size_t nCells, std::vector<double>& out) {
  std::vector<double> a(in), z;
  int din = M.inDim;
  size_t off = 0;
  const double* P = M.params.data();
  for (size_t l = 0; l < M.hidden.size(); ++l) {
    const int w = M.hidden[l];
    const double *W = P + off, *b = W + (size_t)w * din, *sc = b + w, *bi = sc + w;
    off += (size_t)w * din + 3 * (size_t)w;
    z.assign(nCells * w, 0.0);
    for (size_t c = 0; c < nCells; ++c)
      for (int o = 0; o < w; ++o) {
        double s = 0.0;
        for (int i = 0; i < din; ++i) s += W[o + (size_t)i * w] * a[c * din + i];
        z[c * w + o] = activation(M.act[l], s + b[o]);
      }
    std::vector<double> mu(nCells), var(nCells);
    if (M.overBatch) {
      double s = 0.0;
      for (double v : z) s += v;
      const double m = s / (double)z.size();
      double q = 0.0;
      for (double v : z) q += (v - m) * (v - m);
      std::fill(mu.begin(), mu.end(), m);
      std::fill(var.begin(), var.end(), q / (double)z.size());
    } else {
      for (size_t c = 0; c < nCells; ++c) {
        double s = 0.0, q = 0.0;
        for (int o = 0; o < w; ++o) s += z[c * w + o];
        mu[c] = s / w;
        for (int o = 0; o < w; ++o) q += (z[c * w + o] - mu[c]) * (z[c * w + o] - mu[c]);
        var[c] = q / w;
      }
    }
    a.assign(nCells * w, 0.0);
    for (size_t c = 0; c < nCells; ++c)
      for (int o = 0; o < w; ++o)
        a[c * w + o] = (z[c * w + o] - mu[c]) / std::sqrt(var[c] + M.lnEps) * sc[o] + bi[o];
    din = w;
  }
  const double *W = P + off, *b = W + din;
  out.assign(nCells, 0.0);
  for (size_t c = 0; c < nCells; ++c) {
    double s = 0.0;
    for (int i = 0; i < din; ++i) s += W[i] * a[c * din + i];
    out[c] = M.outLo + (M.outHi - M.outLo) * sigmoid_nn(s + b[0]);
  }
}

inline double normalise(double x, const double* b) { return 2.0 * (x - b[0]) / (b[1] - b[0]) - 1.0; }

// Per-cell resistance of the clamped state: Manning's n (kinds 1-6) or the
// flow resistance magnitude (kind 7).  Umag = |q| / h (semi_discretize_swe_2D.jl:143-145).
inline void resistance_cells(const Resistance& r, const std::vector<double>& h, const std::vector<double>& qx,
                             const std::vector<double>& qy, std::vector<double>& out) {
  const size_t N = h.size();
  out.assign(N, 0.0);
  if (r.kind >= RES_POWER_LAW && r.kind <= RES_H_UMAG_KS) {
    for (size_t c = 0; c < N; ++c) {
      const double u = qx[c] / h[c], v = qy[c] / h[c];
      out[c] = manning_fn(r, h[c], std::sqrt(u * u + v * v), r.ks.empty() ? 0.0 : r.ks[c]);
    }
    return;
  }
  const int nin = r.mlp.inDim;
  std::vector<double> in(N * nin);
  for (size_t c = 0; c < N; ++c) {
    in[c * nin] = normalise(h[c], r.hB);
    if (r.kind == RES_UDE_MANNING_H_UMAG_KS) {
      const double u = qx[c] / h[c], v = qy[c] / h[c];
      in[c * nin + 1] = normalise(std::sqrt(u * u + v * v), r.uB);
      in[c * nin + 2] = normalise(r.ks[c], r.ksB);
    } else if (r.kind == RES_UDE_FLOW_RESISTANCE) {   // process_FlowResistance_UDE.jl:13-20
      const double qb[2] = {r.hB[0] * r.uB[0], r.hB[1] * r.uB[1]};
      in[c * nin + 1] = normalise(smooth_sqrt(qx[c] * qx[c] + qy[c] * qy[c]), qb);
    }
  }
  mlp_forward(r.mlp, in, N, out);
}

// Inlet-Q hydrograph of one group: points (t, q), t increasing; Q(t) is the
// linear interpolation, held at the end values outside the points.  The
// reference's inlet discharges are constant (bc_2D.jl:192); this is the
// time-varying inlet of the long-horizon workload, checked here as the device
// evaluates it.
inline double hydro_at(const std::vector<double>& tq, double t) {
  const size_t n = tq.size() / 2;
  const double* T = tq.data();
  const double* Qv = tq.data() + n;
  if (t <= T[0]) return Qv[0];
  if (t >= T[n - 1]) return Qv[n - 1];
  size_t k = 0;
  while (k + 1 < n - 1 && T[k + 1] <= t) ++k;
  const double w = (t - T[k]) / (T[k + 1] - T[k]);
  return Qv[k] + w * (Qv[k + 1] - Qv[k]);
}

template <class T>
struct Params {
  Resistance res;                // state-dependent n / UDE closure (kind RES_CONSTANT: manningCells)
  std::vector<std::vector<double>> hydro;   // per inlet-Q group: times then discharges (empty: constant)
  std::vector<T> manningCells;   // ManningN_cells (process_ManningN_2D.jl:242-269 for zones)
  std::vector<T> zbCells;        // zb_cells (active parameter replaces it, semi_discretize_swe_2D.jl:114-126)
  std::vector<T> inletQ;         // inletQ_TotalQ per inlet-Q boundary (:190-199)
  std::vector<T> exitWSE;        // exitH_WSE per exit-H boundary
  BedData<T> bed;                // derived from zbCells
};

struct Case {
  Mesh mesh;
  Bcs bcs;
  Consts k;
  std::vector<double> hstill;        // wstill - zb (process_ICs_2D.jl:55,84); not recomputed when zb changes
  std::vector<double> hstillGhost;   // setup_ghost_cells_initial_condition (process_ICs_2D.jl:145-155)
};

template <class T>
void set_zb(const Case& cs, Params<T>& p, const std::vector<T>& zb) {
  p.zbCells = zb;
  p.bed = update_bed_data<T>(cs.mesh, zb.data());
}

// Ghost states (bc_2D.jl:575-875).  h, qx, qy are the clamped cell states.
template <class T>
void ghost_states(const Case& cs, const Params<T>& p, const std::vector<T>& manning, const std::vector<T>& h,
                  const std::vector<T>& qx, const std::vector<T>& qy, std::vector<T>& hg, std::vector<T>& qxg,
                  std::vector<T>& qyg) {
  const Mesh& m = cs.mesh;
  size_t nG = m.allBoundaryFaces.size();
  hg.assign(nG, T(0.0)); qxg.assign(nG, T(0.0)); qyg.assign(nG, T(0.0));
  const double hs = cs.k.h_small;
  for (size_t b = 0; b < cs.bcs.inletQ.size(); ++b) {                    // :640-730 inlet-Q
    const BcGroup& G = cs.bcs.inletQ[b];
    T totalA = T(0.0);
    std::vector<double> wet(G.faces.size());
    for (size_t i = 0; i < G.faces.size(); ++i) {
      int c = G.internals[i];
      wet[i] = value(h[c]) > hs ? 1.0 : 0.0;
      totalA = totalA + std::pow(G.lengths[i], 5.0 / 3.0) * h[c] / manning[c] * wet[i];
    }
    if (!(value(totalA) > 1e-10)) throw std::runtime_error("inlet-Q conveyance is not positive (bc_2D.jl:679)");
    for (size_t i = 0; i < G.faces.size(); ++i) {
      int c = G.internals[i], gh = G.ghosts[i];
      T vn = p.inletQ[b] / totalA * std::pow(G.lengths[i], 2.0 / 3.0) / manning[c];
      hg[gh] = h[c];
      qxg[gh] = -h[c] * vn * G.onx[i] * wet[i];
      qyg[gh] = -h[c] * vn * G.ony[i] * wet[i];
    }
  }
  for (size_t b = 0; b < cs.bcs.exitH.size(); ++b) {                     // :748-773 exit-H
    const BcGroup& G = cs.bcs.exitH[b];
    for (size_t i = 0; i < G.faces.size(); ++i) {
      int c = G.internals[i], gh = G.ghosts[i];
      T hn = p.exitWSE[b] - p.zbCells[c];
      hg[gh] = value(hn) > hs ? hn : T(hs);                               // max(h_small, WSE - zb_cell)
      qxg[gh] = qx[c];
      qyg[gh] = qy[c];
    }
  }
  for (const BcGroup& G : cs.bcs.wall)                                   // :777-799 wall
    for (size_t i = 0; i < G.faces.size(); ++i) {
      int c = G.internals[i], gh = G.ghosts[i];
      hg[gh] = h[c]; qxg[gh] = -qx[c]; qyg[gh] = -qy[c];
    }
  for (const BcGroup& G : cs.bcs.symm)                                   // :803-834 symmetry
    for (size_t i = 0; i < G.faces.size(); ++i) {
      int c = G.internals[i], gh = G.ghosts[i];
      T vdn = qx[c] * G.onx[i] + qy[c] * G.ony[i];
      hg[gh] = h[c];
      qxg[gh] = qx[c] - 2.0 * vdn * G.onx[i];
      qyg[gh] = qy[c] - 2.0 * vdn * G.ony[i];
    }
}

// Manning friction (semi_discretize_swe_2D.jl:544-547).
template <class T>
inline T friction_factor(double g, double k_n, double h_small, const T& n, const T& h, const T& qx, const T& qy) {
  using std::pow;
  return g * (n * n) / (k_n * k_n) / pow(h + h_small, 7.0 / 3.0) * smooth_sqrt(qx * qx + qy * qy);
}

// dQ = swe_2d_rhs(Q) with Q = [xi; qx; qy] (semi_discretize_swe_2D.jl:18-277).
template <class T>
void rhs(const Case& cs, const Params<T>& p, const T* Q, T* dQ, int nthreads = 1) {
  const Mesh& m = cs.mesh;
  const int N = m.nCells;
  const double hs = cs.k.h_small, g = cs.k.g;
  std::vector<T> h(N), qx(N), qy(N);
  for (int i = 0; i < N; ++i) {                                         // :101-106 clamp
    T hh = Q[i] + cs.hstill[i];
    bool dry = value(hh) <= hs;
    h[i] = dry ? T(hs) : hh;
    qx[i] = dry ? T(0.0) : Q[N + i];
    qy[i] = dry ? T(0.0) : Q[2 * N + i];
  }
  // State-dependent resistance (:141-149, :167-181, :516-533): n replaces
  // ManningN_cells everywhere it is read (friction and the inlet-Q
  // conveyance); the flow-resistance closure replaces the friction only.
  const std::vector<T>* manning = &p.manningCells;
  std::vector<T> resCells;
  if (p.res.kind != RES_CONSTANT) {
    if constexpr (std::is_same_v<T, double>) {
      resistance_cells(p.res, h, qx, qy, resCells);
      if (p.res.kind != RES_UDE_FLOW_RESISTANCE) manning = &resCells;
    } else {
      throw std::runtime_error("state-dependent resistance: FP64 values only");
    }
  }
  std::vector<T> hg, qxg, qyg;
  ghost_states(cs, p, *manning, h, qx, qy, hg, qxg, qyg);               // :215-217
  std::vector<T> xig(hg.size());
  for (size_t k = 0; k < hg.size(); ++k) xig[k] = hg[k] - cs.hstillGhost[k];   // :220
  (void)nthreads;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1) if (nthreads > 1)
  for (int c = 0; c < N; ++c) {                                          // compute_inviscid_fluxes :286-419
    T fs0 = T(0.0), fs1 = T(0.0), fs2 = T(0.0);
    for (int i = 0; i < m.cellNodesCount[c]; ++i) {
      int f = m.cellFaces[(size_t)c * 8 + i];
      int r = m.cellNeighbors[(size_t)c * 8 + i];
      double nx = m.cellNormals[(size_t)c * 16 + 2 * i], ny = m.cellNormals[(size_t)c * 16 + 2 * i + 1];
      T xiR, hstR, hR, huR, hvR, zbR;
      if (!m.faceIsBoundary[f]) {
        xiR = Q[r]; hstR = T(cs.hstill[r]); hR = h[r]; huR = qx[r]; hvR = qy[r]; zbR = p.zbCells[r];
      } else {
        xiR = xig[r]; hstR = T(cs.hstillGhost[r]); hR = hg[r]; huR = qxg[r]; hvR = qyg[r]; zbR = p.bed.zbGhost[r];
      }
      T F[3];
      if (cs.k.riemann == RIEMANN_HLL)
        hll_flux<T>(Q[c], T(cs.hstill[c]), h[c], qx[c], qy[c], p.zbCells[c], xiR, hstR, hR, huR, hvR, zbR, g, nx,
                    ny, hs, F);
      else
        roe_flux<T>(Q[c], T(cs.hstill[c]), h[c], qx[c], qy[c], p.zbCells[c], xiR, hstR, hR, huR, hvR, zbR, g, nx,
                    ny, hs, F);
      double L = m.faceLengths[f];
      fs0 = fs0 + F[0] * L;                                              // :387
      fs1 = fs1 + F[1] * L;
      fs2 = fs2 + F[2] * L;
    }
    double A = m.cellAreas[c];
    T inv0 = -fs0 / A, inv1 = -fs1 / A, inv2 = -fs2 / A;                // :415
    // compute_source_terms (:449-505) + compute_friction_terms (:508-559)
    T frx, fry;
    if (p.res.kind == RES_UDE_FLOW_RESISTANCE) {                          // :517-529
      const T mag = smooth_sqrt(qx[c] * qx[c] + qy[c] * qy[c]);
      frx = resCells[c] * qx[c] / mag;
      fry = resCells[c] * qy[c] / mag;
    } else {
      T fr = friction_factor<T>(g, cs.k.k_n, hs, (*manning)[c], h[c], qx[c], qy[c]);
      frx = fr * qx[c];
      fry = fr * qy[c];
    }
    bool above = value(h[c]) > hs;
    T sx = above ? (g * Q[c] * p.bed.S0x[c] - frx) : T(0.0);
    T sy = above ? (g * Q[c] * p.bed.S0y[c] - fry) : T(0.0);
    dQ[c] = inv0 + 0.0;                                                  // continuity source is zero (:478)
    dQ[N + c] = inv1 + sx;                                               // :264
    dQ[2 * N + c] = inv2 + sy;
  }
}

// Wet/dry diagnostic flags (src/fvm/discretization/process_dry_wet.jl:2-35).
// Recomputed by the reference each RHS call but never consumed by fluxes or
// sources; kept here as a diagnostic only.
inline void dry_wet_flags(const Mesh& m, const std::vector<double>& h, const std::vector<double>& zb, double h_small,
                          std::vector<char>& wet, std::vector<char>& adjDry, std::vector<char>& adjHighDry) {
  int N = m.nCells;
  wet.assign(N, 0); adjDry.assign(N, 0); adjHighDry.assign(N, 0);
  for (int c = 0; c < N; ++c) wet[c] = h[c] > h_small;
  for (int c = 0; c < N; ++c)
    for (int i = 0; i < m.cellNodesCount[c]; ++i) {
      int f = m.cellFaces[(size_t)c * 8 + i], nb = m.cellNeighbors[(size_t)c * 8 + i];
      bool bnd = m.faceIsBoundary[f];
      if (bnd || !wet[nb]) adjDry[c] = 1;
      if (bnd || (!wet[nb] && (h[c] + zb[c]) < zb[nb])) adjHighDry[c] = 1;
    }
}

// ---------------------------------------------------------------------------
// Time stepping.
// ---------------------------------------------------------------------------
// Forward Euler with the reference's clamp (custom_ODE_solvers.jl:5-33): the
// first state block is compared with h_small as if it were h.
template <class T>
void euler_step_reference(const Case& cs, const Params<T>& p, std::vector<T>& Q, double dt, int nthreads = 1) {
  const int N = cs.mesh.nCells;
  std::vector<T> dQ(3 * (size_t)N);
  rhs<T>(cs, p, Q.data(), dQ.data(), nthreads);
  for (size_t k = 0; k < Q.size(); ++k) Q[k] = Q[k] + dt * dQ[k];
  for (int i = 0; i < N; ++i)
    if (value(Q[i]) < cs.k.h_small) { Q[i] = T(cs.k.h_small); Q[N + i] = T(0.0); Q[2 * N + i] = T(0.0); }
}

// xi of a dry cell: the largest xi with xi + hstill <= h_small in FP64, so
// that the RHS sees the cell as dry (h <= h_small).  h_small - hstill alone can
// round to a depth one ulp above h_small: a wet film whose Manning friction
// (h + h_small)^(-7/3) breaks any explicit step.
inline double dry_xi(double h_small, double hstill) {
  double x = h_small - hstill;
  while (x + hstill > h_small) x = std::nextafter(x, -INFINITY);
  return x;
}

// Depth-positivity clamp applied after each explicit stage: where
// h = xi + hstill <= h_small the cell is dry: xi = dry_xi (h = h_small) and
// q = 0.  With hstill = 0 this is custom_ODE_update_cells' clamp
// (custom_ODE_solvers.jl:18-26), except that it also resets a cell sitting
// exactly at h_small, whose momentum the RHS ignores (it clamps h <= h_small,
// semi_discretize_swe_2D.jl:104-106) but which would otherwise accumulate.
template <class T>
inline void clamp_stage(const Case& cs, T* Q) {
  const int N = cs.mesh.nCells;
  for (int i = 0; i < N; ++i)
    if (value(Q[i]) + cs.hstill[i] <= cs.k.h_small) {
      Q[i] = T(dry_xi(cs.k.h_small, cs.hstill[i]));
      Q[N + i] = T(0.0);
      Q[2 * N + i] = T(0.0);
    }
}

// CFL time step from the state Q: dt = CFL * min_c A_c / sum_f L_f (|u.n_f| + sqrt(g h)),
// with the clamped h, u = qx/h, v = qy/h of cell c and its outward normals.
// (The reference stores CFL = 0.4 but never uses it, solve_swe_2D.jl:86.)
inline double cfl_dt(const Case& cs, const double* Q, double cfl) {
  const Mesh& m = cs.mesh;
  const int N = m.nCells;
  double best = INFINITY;
  for (int c = 0; c < N; ++c) {
    double h = Q[c] + cs.hstill[c];
    double qx = Q[N + c], qy = Q[2 * N + c];
    if (h <= cs.k.h_small) { h = cs.k.h_small; qx = 0.0; qy = 0.0; }
    double u = qx / h, v = qy / h, a = std::sqrt(cs.k.g * h);
    double s = 0.0;
    for (int i = 0; i < m.cellNodesCount[c]; ++i) {
      double nx = m.cellNormals[(size_t)c * 16 + 2 * i], ny = m.cellNormals[(size_t)c * 16 + 2 * i + 1];
      s += m.faceLengths[m.cellFaces[(size_t)c * 8 + i]] * (std::fabs(u * nx + v * ny) + a);
    }
    double r = m.cellAreas[c] / s;
    if (r < best) best = r;
  }
  return cfl * best;
}

// One SSP-RK2 (Heun) step: Q1 = C(Q0 + dt R(Q0)); Q2 = C(0.5*(Q0 + (Q1 + dt R(Q1)))).
// The parameters at time t: inlet discharges from their hydrographs, if any.
template <class T>
const Params<T>& params_at(const Params<T>& p, Params<T>& scratch, double t) {
  bool any = false;
  for (const auto& h : p.hydro) any = any || !h.empty();
  if (!any) return p;
  if (scratch.inletQ.size() != p.inletQ.size()) scratch = p;
  for (size_t g = 0; g < p.hydro.size() && g < scratch.inletQ.size(); ++g)
    if (!p.hydro[g].empty()) scratch.inletQ[g] = T(hydro_at(p.hydro[g], t));
  return scratch;
}

// One SSP-RK2 step from time t (stage 1 at t, stage 2 at t + dt).
template <class T>
void rk2_step(const Case& cs, const Params<T>& p, std::vector<T>& Q, double dt, int nthreads = 1, double t = 0.0) {
  const size_t n3 = Q.size();
  std::vector<T> R(n3), Q1(n3);
  Params<T> scratch;
  rhs<T>(cs, params_at(p, scratch, t), Q.data(), R.data(), nthreads);
  for (size_t k = 0; k < n3; ++k) Q1[k] = Q[k] + dt * R[k];
  clamp_stage<T>(cs, Q1.data());
  rhs<T>(cs, params_at(p, scratch, t + dt), Q1.data(), R.data(), nthreads);
  for (size_t k = 0; k < n3; ++k) Q[k] = 0.5 * (Q[k] + (Q1[k] + dt * R[k]));
  clamp_stage<T>(cs, Q.data());
}

// Tsitouras 5(4) pair (Ch. Tsitouras, Comput. Math. Appl. 62 (2011)
// 770-775), restated from the published tableau, with the step control of
// Hairer, Norsett & Wanner, Solving ODEs I, II.4: weighted RMS norm of the
// embedded error (scale abstol + reltol max(|Q|, |Qnew|)), PI controller with
// gains 0.14 / 0.08, safety 0.9, factor in [0.2, 10], the starting step of
// II.4 when dt0 <= 0, and steps clamped onto t1; adaptive == false takes fixed
// steps of dt0.  The CPU check of the device integrator (same algorithm);
// stats: accepted, rejected, RHS evaluations.  Returns false after maxSteps
// steps.
struct Tsit5Stats {
  int accepted = 0, rejected = 0, evals = 0;
};

// The Tsit5 tableau: nodes c, coefficients a (row 6: the 5th-order weights b,
// the seventh stage being the new state), and b - bhat.
struct Tsit5Tab {
  double C[7];
  double A[7][6];
  double BT[7];
};
inline const Tsit5Tab& tsit5_tab() {
  static const Tsit5Tab t = {
      {0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0},
      {{0, 0, 0, 0, 0, 0},
       {0.161, 0, 0, 0, 0, 0},
       {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
       {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
       {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
       {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
       {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}},
      {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995, -0.1447110071732629,
       0.5823571654525552, -0.45808210592918697, 0.015151515151515152}};
  return t;
}

// One fixed Tsit5 step of size h from time t, on any scalar type (dual numbers
// give forward-mode derivatives): the stages and the new state exactly as
// tsit5() forms them with adaptive == false (the same operations in the same
// order), with no clamp of the state (the RHS clamps its own copy of h).
template <class T>
void tsit5_fixed_step(const Case& cs, const Params<T>& p, std::vector<T>& Q, double h, int nthreads = 1,
                      double t = 0.0) {
  const Tsit5Tab& tb = tsit5_tab();
  const size_t n3 = Q.size();
  std::vector<std::vector<T>> K(6, std::vector<T>(n3));
  std::vector<T> Y(n3);
  Params<T> scratch;
  rhs<T>(cs, params_at(p, scratch, t), Q.data(), K[0].data(), nthreads);
  for (int i = 1; i < 7; ++i) {
    for (size_t k = 0; k < n3; ++k) {
      T s(0.0);
      for (int j = 0; j < i; ++j) s = s + tb.A[i][j] * K[j][k];
      Y[k] = Q[k] + h * s;
    }
    if (i < 6) rhs<T>(cs, params_at(p, scratch, t + tb.C[i] * h), Y.data(), K[i].data(), nthreads);
  }
  Q.swap(Y);
}

inline bool tsit5(const Case& cs, const Params<double>& p, std::vector<double>& Q, double t0, double t1, double abstol,
                  double reltol, double dt0, bool adaptive, int maxSteps, Tsit5Stats& st, int nthreads = 1) {
  const double(&C)[7] = tsit5_tab().C;
  const double(&A)[7][6] = tsit5_tab().A;
  const double(&BT)[7] = tsit5_tab().BT;
  const size_t n3 = Q.size();
  std::vector<std::vector<double>> K(7, std::vector<double>(n3));
  std::vector<double> Y(n3), Qn(n3);
  auto norm = [&](const std::vector<double>& ua, const std::vector<double>& ub, const std::vector<double>& e) {
    double s = 0.0;
    for (size_t i = 0; i < n3; ++i) {
      const double r = e[i] / (abstol + reltol * std::max(std::fabs(ua[i]), std::fabs(ub[i])));
      s += r * r;
    }
    return std::sqrt(s / (double)n3);
  };
  Params<double> scratch;
  rhs<double>(cs, params_at(p, scratch, t0), Q.data(), K[0].data(), nthreads);
  st.evals = 1;
  double dt = dt0;
  if (adaptive && !(dt > 0)) {
    const double d0 = norm(Q, Q, Q), d1 = norm(Q, Q, K[0]);
    const double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
    for (size_t i = 0; i < n3; ++i) Y[i] = Q[i] + h0 * K[0][i];
    rhs<double>(cs, params_at(p, scratch, t0 + h0), Y.data(), K[1].data(), nthreads);
    ++st.evals;
    std::vector<double> df(n3);
    for (size_t i = 0; i < n3; ++i) df[i] = (K[1][i] - K[0][i]) / h0;
    const double d2 = norm(Q, Q, df);
    const double m = std::max(d1, d2);
    const double h1 = m <= 1e-15 ? std::max(1e-6, h0 * 1e-3) : std::pow(0.01 / m, 1.0 / 5.0);
    dt = std::min(100.0 * h0, h1);
  }
  if (adaptive) dt = std::min(dt, t1 - t0);
  const double beta1 = 7.0 / 50.0, beta2 = 2.0 / 25.0, gamma = 0.9, qmin = 0.2, qmax = 10.0;
  double errOld = 1e-4, t = t0;
  std::vector<double> E(n3);
  while (t1 - t > 1e-14 * std::max(1.0, std::fabs(t1))) {
    if (st.accepted + st.rejected >= maxSteps) return false;
    double h = dt;
    bool hit = false;
    if (t + h >= t1 - 1e-14 * std::max(1.0, std::fabs(t1))) {
      h = t1 - t;
      hit = true;
    }
    for (int i = 1; i < 7; ++i) {
      std::vector<double>& dst = (i == 6) ? Qn : Y;
      for (size_t k = 0; k < n3; ++k) {
        double s = 0.0;
        for (int j = 0; j < i; ++j) s += A[i][j] * K[j][k];
        dst[k] = Q[k] + h * s;
      }
      rhs<double>(cs, params_at(p, scratch, t + C[i] * h), dst.data(), K[i].data(), nthreads);
    }
    st.evals += 6;
    double eest = 0.0;
    if (adaptive) {
      for (size_t k = 0; k < n3; ++k) {
        double s = 0.0;
        for (int j = 0; j < 7; ++j) s += BT[j] * K[j][k];
        E[k] = h * s;
      }
      eest = norm(Q, Qn, E);
    }
    if (eest <= 1.0) {
      t = hit ? t1 : t + h;
      Q.swap(Qn);
      K[0].swap(K[6]);
      ++st.accepted;
      if (!adaptive) continue;
      const double fac = std::min(qmax, std::max(qmin, gamma * std::pow(std::max(eest, 1e-12), -beta1) *
                                                            std::pow(errOld, beta2)));
      errOld = std::max(eest, 1e-4);
      dt = h * fac;
    } else {
      ++st.rejected;
      dt = h * (std::isfinite(eest) ? std::max(qmin, gamma * std::pow(eest, -beta1)) : qmin);
      if (dt < 1e-14 * std::max(1.0, std::fabs(t))) return false;
    }
  }
  return true;
}

}  // namespace hgo
