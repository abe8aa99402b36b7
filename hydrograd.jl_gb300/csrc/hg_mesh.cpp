// Host mesh construction and cell renumbering (see hg_mesh.hpp).
#include "hg_mesh.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <deque>
#include <numeric>
#include <utility>

namespace hg {

namespace {

inline uint64_t edge_key(int a, int b) {
  int lo = a < b ? a : b, hi = a < b ? b : a;
  return ((uint64_t)(uint32_t)lo << 32) | (uint32_t)hi;
}

// Locate the face of edge (a,b) with a binary search over the sorted key table.
struct EdgeIndex {
  std::vector<uint64_t> keys;   // sorted
  std::vector<int> face;        // face id of keys[i]
  int find(int a, int b) const {
    uint64_t k = edge_key(a, b);
    auto it = std::lower_bound(keys.begin(), keys.end(), k);
    if (it == keys.end() || *it != k) return -1;
    return face[it - keys.begin()];
  }
};

}  // namespace

int build_host_mesh(const hg_mesh_desc& d, HostMesh& m, std::string& err) {
  if (d.n_nodes <= 0 || d.n_cells <= 0 || !d.node_x || !d.node_y || !d.node_z || !d.cell_node_count ||
      !d.cell_nodes) {
    err = "mesh: empty mesh or null array";
    return HG_ERR_ARG;
  }
  if (d.n_strings < 0 || (d.n_strings > 0 && (!d.string_ids || !d.string_offsets || !d.string_nodes || !d.string_bc))) {
    err = "mesh: bad NodeString arrays";
    return HG_ERR_ARG;
  }
  const int N = d.n_cells;
  m.nCells = N;
  m.nNodes = d.n_nodes;
  m.x.assign(d.node_x, d.node_x + d.n_nodes);
  m.y.assign(d.node_y, d.node_y + d.n_nodes);
  m.z.assign(d.node_z, d.node_z + d.n_nodes);
  m.ncf.assign(d.cell_node_count, d.cell_node_count + N);
  m.cellNodes.assign(d.cell_nodes, d.cell_nodes + (size_t)N * 8);
  m.maxCellFaces = 0;
  for (int c = 0; c < N; ++c) {
    int n = m.ncf[c];
    if (n < 3 || n > kMaxCellFaces) {
      err = "mesh: cell " + std::to_string(c) + " has " + std::to_string(n) + " nodes (3..8 allowed)";
      return HG_ERR_MESH;
    }
    m.maxCellFaces = std::max(m.maxCellFaces, n);
    for (int i = 0; i < n; ++i) {
      int v = m.cellNodes[(size_t)c * 8 + i];
      if (v < 0 || v >= d.n_nodes) {
        err = "mesh: cell " + std::to_string(c) + " references node " + std::to_string(v);
        return HG_ERR_ARG;
      }
    }
  }

  // --- Edges.  Face ids follow the order in which a loop over cells and their
  // edges first meets each edge (SRH_2D_SRHGeom.jl:251-287).
  std::vector<std::pair<uint64_t, int64_t>> occ;   // (key, c*8+i)
  occ.reserve((size_t)N * 4);
  for (int c = 0; c < N; ++c)
    for (int i = 0; i < m.ncf[c]; ++i) {
      int a = m.cellNodes[(size_t)c * 8 + i], b = m.cellNodes[(size_t)c * 8 + (i + 1) % m.ncf[c]];
      if (a == b) {
        err = "mesh: degenerate edge in cell " + std::to_string(c);
        return HG_ERR_MESH;
      }
      occ.emplace_back(edge_key(a, b), (int64_t)c * 8 + i);
    }
  std::sort(occ.begin(), occ.end());
  // Groups of equal keys; each group is one face.  First occurrence = min slot.
  std::vector<std::pair<int64_t, size_t>> groups;   // (first slot, start index)
  for (size_t s = 0; s < occ.size();) {
    size_t e = s;
    while (e < occ.size() && occ[e].first == occ[s].first) ++e;
    if (e - s > 2) {
      err = "mesh: an edge is shared by more than two cells";
      return HG_ERR_MESH;
    }
    groups.emplace_back(occ[s].second, s);
    s = e;
  }
  std::vector<size_t> gorder(groups.size());
  std::iota(gorder.begin(), gorder.end(), 0);
  std::sort(gorder.begin(), gorder.end(), [&](size_t a, size_t b) { return groups[a].first < groups[b].first; });
  m.nFaces = (int)groups.size();
  m.faceA.resize(m.nFaces); m.faceB.resize(m.nFaces);
  m.faceC0.resize(m.nFaces); m.faceC1.resize(m.nFaces);
  m.cf.assign((size_t)N * 8, -1);
  m.cfs.assign((size_t)N * 8, 0);
  EdgeIndex eidx;
  eidx.keys.resize(groups.size());
  eidx.face.resize(groups.size());
  for (int f = 0; f < m.nFaces; ++f) {
    size_t gi = gorder[f];
    size_t s = groups[gi].second;
    uint64_t k = occ[s].first;
    m.faceA[f] = (int)(k >> 32);
    m.faceB[f] = (int)(k & 0xffffffffu);
    bool two = (s + 1 < occ.size() && occ[s + 1].first == k);
    int64_t s0 = occ[s].second, s1 = two ? occ[s + 1].second : -1;   // slots sorted ascending
    m.faceC0[f] = (int)(s0 / 8);
    m.faceC1[f] = two ? (int)(s1 / 8) : -1;
    if (two && m.faceC0[f] == m.faceC1[f]) {
      err = "mesh: a cell uses the same edge twice";
      return HG_ERR_MESH;
    }
    m.cf[s0] = f;
    if (two) m.cf[s1] = f;
    eidx.keys[gi] = k;
    eidx.face[gi] = f;
  }
  // occ is sorted by key and groups were built in that order, so eidx.keys is sorted.
  for (int c = 0; c < N; ++c)
    for (int i = 0; i < m.ncf[c]; ++i) {
      int a = m.cellNodes[(size_t)c * 8 + i], b = m.cellNodes[(size_t)c * 8 + (i + 1) % m.ncf[c]];
      m.cfs[(size_t)c * 8 + i] = (a < b) ? 1 : -1;
    }

  // --- Neighbours (mesh_2D.jl:229-254).
  m.nbr.assign((size_t)N * 8, -1);
  for (int c = 0; c < N; ++c)
    for (int i = 0; i < m.ncf[c]; ++i) {
      int f = m.cf[(size_t)c * 8 + i];
      if (m.faceC1[f] >= 0) m.nbr[(size_t)c * 8 + i] = (m.faceC0[f] == c) ? m.faceC1[f] : m.faceC0[f];
    }

  // --- Boundaries from NodeStrings (SRH_2D_SRHGeom.jl:303-349).
  std::vector<char> used(m.nFaces, 0);
  std::vector<Boundary> bl;
  int nBoundaryStrings = 0;
  for (int s = 0; s < d.n_strings; ++s) {
    int bc = d.string_bc[s];
    if (bc == HG_BC_NONE) continue;
    if (bc < HG_BC_WALL || bc > HG_BC_EXITH) {
      err = "mesh: NodeString " + std::to_string(d.string_ids[s]) + " has an unknown boundary type";
      return HG_ERR_ARG;
    }
    ++nBoundaryStrings;
    Boundary b;
    b.id = d.string_ids[s];
    b.bc = bc;
    int o0 = d.string_offsets[s], o1 = d.string_offsets[s + 1];
    for (int k = o0; k + 1 < o1; ++k) {
      int a = d.string_nodes[k], bb = d.string_nodes[k + 1];
      int f = (a >= 0 && bb >= 0 && a < m.nNodes && bb < m.nNodes) ? eidx.find(a, bb) : -1;
      if (f < 0) {
        err = "mesh: edge (" + std::to_string(a) + "," + std::to_string(bb) + ") of NodeString " +
              std::to_string(b.id) + " is not a mesh edge";
        return HG_ERR_MESH;
      }
      if (m.faceC1[f] >= 0) {
        err = "mesh: NodeString " + std::to_string(b.id) + " runs along an interior edge";
        return HG_ERR_MESH;
      }
      b.faces.push_back(f);
      used[f] = 1;
    }
    bl.push_back(std::move(b));
  }
  {
    Boundary def;
    def.id = nBoundaryStrings + 1;   // defaultWallBoundaryID (SRH_2D_SRHGeom.jl:347)
    def.bc = HG_BC_WALL;
    for (int f = 0; f < m.nFaces; ++f)
      if (m.faceC1[f] < 0 && !used[f]) def.faces.push_back(f);
    if (!def.faces.empty()) bl.push_back(std::move(def));
  }
  std::sort(bl.begin(), bl.end(), [](const Boundary& a, const Boundary& b) { return a.id < b.id; });
  for (size_t i = 1; i < bl.size(); ++i)
    if (bl[i].id == bl[i - 1].id) {
      err = "mesh: duplicate boundary id " + std::to_string(bl[i].id);
      return HG_ERR_ARG;
    }
  m.faceBnd.assign(m.nFaces, -1);
  for (size_t bi = 0; bi < bl.size(); ++bi) {
    Boundary& b = bl[bi];
    b.dirs.resize(b.faces.size());
    for (size_t k = 0; k < b.faces.size(); ++k) {
      int f = b.faces[k];
      int c = m.faceC0[f];
      signed char dir = 1;   // mesh_2D.jl:141-158
      for (int i = 0; i < m.ncf[c]; ++i)
        if (m.cf[(size_t)c * 8 + i] == f && m.cfs[(size_t)c * 8 + i] < 0) dir = -1;
      b.dirs[k] = dir;
      if (m.faceBnd[f] < 0) m.faceBnd[f] = (int)bi;   // first boundary holding the face (mesh_2D.jl:391-396)
    }
  }
  m.bnd = std::move(bl);
  m.nGhost = 0;
  for (int f = 0; f < m.nFaces; ++f)
    if (m.faceC1[f] < 0) ++m.nGhost;
  for (size_t bi = 0; bi < m.bnd.size(); ++bi) {
    switch (m.bnd[bi].bc) {
      case HG_BC_INLETQ: m.inletGroups.push_back((int)bi); break;
      case HG_BC_EXITH: m.exitGroups.push_back((int)bi); break;
      case HG_BC_SYMM: m.symmGroups.push_back((int)bi); break;
      default: m.wallGroups.push_back((int)bi); break;
    }
  }

  // --- Geometry (mesh_2D.jl:456-652), same operation order as the reference.
  m.area.assign(N, 0.0); m.cx.assign(N, 0.0); m.cy.assign(N, 0.0);
  m.snx.assign((size_t)N * 8, 0.0); m.sny.assign((size_t)N * 8, 0.0);
  m.zbCell.assign(N, 0.0);
  for (int c = 0; c < N; ++c) {
    const int n = m.ncf[c];
    const int* nodes = &m.cellNodes[(size_t)c * 8];
    double a2 = 0.0;
    for (int i = 0; i < n; ++i) {
      int p = nodes[i], q = nodes[(i + 1) % n];
      a2 += m.x[p] * m.y[q] - m.x[q] * m.y[p];
    }
    if (a2 < 0) {
      err = "mesh: cell " + std::to_string(c) + " is not counter-clockwise (mesh_2D.jl:577-597)";
      return HG_ERR_MESH;
    }
    m.area[c] = std::fabs(a2) / 2;
    double sx = 0.0, sy = 0.0, ss = 0.0;
    for (int i = 0; i < n; ++i) {
      int p = nodes[i], q = nodes[(i + 1) % n];
      double x1 = m.x[p], y1 = m.y[p], x2 = m.x[q], y2 = m.y[q];
      double cr = x1 * y2 - x2 * y1;
      sx += (x1 + x2) * cr;
      sy += (y1 + y2) * cr;
      ss += cr;
    }
    double aa = std::fabs(ss) / 2;
    m.cx[c] = sx / (6 * aa);
    m.cy[c] = sy / (6 * aa);
    double zs = 0.0;
    for (int i = 0; i < n; ++i) {
      int p = nodes[i], q = nodes[(i + 1) % n];
      double ex = m.x[q] - m.x[p], ey = m.y[q] - m.y[p];
      double nx = ey, ny = -ex;
      double len = std::sqrt(nx * nx + ny * ny);
      if (!(len > 0)) {
        err = "mesh: zero-length edge in cell " + std::to_string(c);
        return HG_ERR_MESH;
      }
      m.snx[(size_t)c * 8 + i] = nx / len;
      m.sny[(size_t)c * 8 + i] = ny / len;
      zs += m.z[nodes[i]];
    }
    m.zbCell[c] = zs / n;   // nodes_to_cells_scalar (fvm_schemes_2D.jl:216-224)
  }
  m.faceLen.assign(m.nFaces, 0.0);
  for (int f = 0; f < m.nFaces; ++f) {
    int p = m.faceA[f], q = m.faceB[f];
    double nx = m.y[q] - m.y[p], ny = -(m.x[q] - m.x[p]);
    m.faceLen[f] = std::sqrt(nx * nx + ny * ny);
  }
  return HG_OK;
}

namespace {

// Reverse Cuthill-McKee over the cell adjacency graph.  Each connected
// component starts from a pseudo-peripheral cell (repeated BFS to the farthest
// cell of least degree); neighbours are visited by ascending degree.
std::vector<int> order_rcm(const HostMesh& m) {
  const int N = m.nCells;
  std::vector<int> deg(N, 0);
  for (int c = 0; c < N; ++c)
    for (int i = 0; i < m.ncf[c]; ++i)
      if (m.nbr[(size_t)c * 8 + i] >= 0) ++deg[c];
  std::vector<int> order;
  order.reserve(N);
  std::vector<char> seen(N, 0);
  std::vector<int> level(N, -1);
  auto bfs_far = [&](int s, std::vector<int>& comp) {
    comp.clear();
    std::deque<int> q{s};
    level[s] = 0;
    comp.push_back(s);
    int far = s;
    while (!q.empty()) {
      int c = q.front();
      q.pop_front();
      if (level[c] > level[far] || (level[c] == level[far] && deg[c] < deg[far])) far = c;
      for (int i = 0; i < m.ncf[c]; ++i) {
        int nb = m.nbr[(size_t)c * 8 + i];
        if (nb >= 0 && level[nb] < 0) {
          level[nb] = level[c] + 1;
          comp.push_back(nb);
          q.push_back(nb);
        }
      }
    }
    for (int c : comp) level[c] = -1;
    return far;
  };
  std::vector<int> comp;
  for (int s0 = 0; s0 < N; ++s0) {
    if (seen[s0]) continue;
    int start = s0;
    for (int it = 0; it < 3; ++it) start = bfs_far(start, comp);
    std::vector<int> cm;
    cm.reserve(comp.size());
    std::deque<int> q{start};
    seen[start] = 1;
    std::vector<int> nbs;
    while (!q.empty()) {
      int c = q.front();
      q.pop_front();
      cm.push_back(c);
      nbs.clear();
      for (int i = 0; i < m.ncf[c]; ++i) {
        int nb = m.nbr[(size_t)c * 8 + i];
        if (nb >= 0 && !seen[nb]) {
          seen[nb] = 1;
          nbs.push_back(nb);
        }
      }
      std::sort(nbs.begin(), nbs.end(), [&](int a, int b) { return deg[a] != deg[b] ? deg[a] < deg[b] : a < b; });
      for (int nb : nbs) q.push_back(nb);
    }
    order.insert(order.end(), cm.rbegin(), cm.rend());
  }
  return order;
}

// Hilbert-curve index of (x, y) on a 2^16 x 2^16 grid.
uint64_t hilbert_index(uint32_t x, uint32_t y) {
  uint64_t d = 0;
  for (uint32_t s = 1u << 15; s > 0; s >>= 1) {
    uint32_t rx = (x & s) > 0, ry = (y & s) > 0;
    d += (uint64_t)s * s * ((3 * rx) ^ ry);
    if (ry == 0) {
      if (rx == 1) {
        x = s - 1 - x;
        y = s - 1 - y;
      }
      std::swap(x, y);
    }
  }
  return d;
}

// Hilbert order of the cells [a, b), appended to order.
void hilbert_range(const HostMesh& m, int a, int b, std::vector<int>& order) {
  double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
  for (int c = a; c < b; ++c) {
    x0 = std::min(x0, m.cx[c]); x1 = std::max(x1, m.cx[c]);
    y0 = std::min(y0, m.cy[c]); y1 = std::max(y1, m.cy[c]);
  }
  double sc = 65535.0 / std::max(std::max(x1 - x0, y1 - y0), 1e-300);
  std::vector<std::pair<uint64_t, int>> key(b - a);
  for (int c = a; c < b; ++c) {
    uint32_t ix = (uint32_t)std::min(65535.0, std::max(0.0, (m.cx[c] - x0) * sc));
    uint32_t iy = (uint32_t)std::min(65535.0, std::max(0.0, (m.cy[c] - y0) * sc));
    key[c - a] = {hilbert_index(ix, iy), c};
  }
  std::sort(key.begin(), key.end());
  for (const auto& k : key) order.push_back(k.second);
}

std::vector<int> order_hilbert(const HostMesh& m) {
  std::vector<int> order;
  order.reserve(m.nCells);
  hilbert_range(m, 0, m.nCells, order);
  return order;
}

}  // namespace

std::vector<int> order_cells(const HostMesh& m, int order) {
  if (order == HG_ORDER_RCM) return order_rcm(m);
  if (order == HG_ORDER_HILBERT) return order_hilbert(m);
  std::vector<int> id(m.nCells);
  std::iota(id.begin(), id.end(), 0);
  return id;
}

std::vector<int> order_cells_ranges(const HostMesh& m, int order, const std::vector<int>& start) {
  if (order != HG_ORDER_HILBERT) return order_cells(m, order);   // RCM visits components in cell order
  std::vector<int> out;
  out.reserve(m.nCells);
  for (size_t r = 0; r + 1 < start.size(); ++r) hilbert_range(m, start[r], start[r + 1], out);
  return out;
}

void concat_host_meshes(const std::vector<const HostMesh*>& parts, HostMesh& o) {
  o = HostMesh();
  size_t C = 0, V = 0, F = 0;
  for (const HostMesh* p : parts) {
    C += p->nCells;
    V += p->nNodes;
    F += p->nFaces;
  }
  for (auto* v : {&o.x, &o.y, &o.z}) v->reserve(V);
  o.cellNodes.reserve(C * 8);
  o.cf.reserve(C * 8);
  o.nbr.reserve(C * 8);
  o.faceC0.reserve(F);
  o.faceC1.reserve(F);
  int cOff = 0, vOff = 0, fOff = 0, bOff = 0;
  auto shift = [](int v, int off) { return v >= 0 ? v + off : v; };
  for (const HostMesh* p : parts) {
    const HostMesh& m = *p;
    o.maxCellFaces = std::max(o.maxCellFaces, m.maxCellFaces);
    o.nGhost += m.nGhost;
    o.x.insert(o.x.end(), m.x.begin(), m.x.end());
    o.y.insert(o.y.end(), m.y.begin(), m.y.end());
    o.z.insert(o.z.end(), m.z.begin(), m.z.end());
    o.ncf.insert(o.ncf.end(), m.ncf.begin(), m.ncf.end());
    for (int v : m.cellNodes) o.cellNodes.push_back(shift(v, vOff));
    for (int c = 0; c < m.nCells; ++c)
      for (int i = 0; i < kMaxCellFaces; ++i) {
        const size_t k = (size_t)c * 8 + i;
        o.cf.push_back(i < m.ncf[c] ? m.cf[k] + fOff : m.cf[k]);
        o.nbr.push_back(shift(m.nbr[k], cOff));
      }
    o.cfs.insert(o.cfs.end(), m.cfs.begin(), m.cfs.end());
    for (int v : m.faceA) o.faceA.push_back(v + vOff);
    for (int v : m.faceB) o.faceB.push_back(v + vOff);
    for (int v : m.faceC0) o.faceC0.push_back(v + cOff);
    for (int v : m.faceC1) o.faceC1.push_back(shift(v, cOff));
    for (const Boundary& b : m.bnd) {
      Boundary nb = b;
      nb.id = (int)o.bnd.size() + 1;
      for (int& f : nb.faces) f += fOff;
      o.bnd.push_back(std::move(nb));
    }
    for (int v : m.faceBnd) o.faceBnd.push_back(shift(v, bOff));
    for (auto pr : {std::make_pair(&o.area, &m.area), std::make_pair(&o.cx, &m.cx), std::make_pair(&o.cy, &m.cy),
                    std::make_pair(&o.snx, &m.snx), std::make_pair(&o.sny, &m.sny),
                    std::make_pair(&o.faceLen, &m.faceLen), std::make_pair(&o.zbCell, &m.zbCell)})
      pr.first->insert(pr.first->end(), pr.second->begin(), pr.second->end());
    for (int g : m.inletGroups) o.inletGroups.push_back(g + bOff);
    for (int g : m.exitGroups) o.exitGroups.push_back(g + bOff);
    for (int g : m.wallGroups) o.wallGroups.push_back(g + bOff);
    for (int g : m.symmGroups) o.symmGroups.push_back(g + bOff);
    cOff += m.nCells;
    vOff += m.nNodes;
    fOff += m.nFaces;
    bOff += (int)m.bnd.size();
  }
  o.nCells = cOff;
  o.nNodes = vOff;
  o.nFaces = fOff;
}

}  // namespace hg
