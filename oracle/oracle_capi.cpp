// C entry points of the oracle, for ctypes.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/ and by bench.py's CPU-baseline
// and reference legs, never by the library.  All ids at this interface are
// 0-based; the state layout is the reference's Q = [xi; q_x; q_y]
// (semi_discretize_swe_2D.jl:93-95).
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "hg_oracle.hpp"

using namespace hgo;

namespace {

struct OracleCase {
  Case cs;
  Params<double> p;
  std::vector<int> zoneOfCell;   // matID_cells (0-based zone index)
  std::string err;
};

thread_local std::string g_err;

template <int ND>
using D = Dual<ND>;

template <int ND>
Params<D<ND>> lift_params(const OracleCase& oc, int nDir, const double* dManning, const double* dZb,
                          const double* dInletQ) {
  const int N = oc.cs.mesh.nCells;
  Params<D<ND>> q;
  q.manningCells.resize(N);
  std::vector<D<ND>> zb(N);
  for (int c = 0; c < N; ++c) {
    q.manningCells[c] = D<ND>(oc.p.manningCells[c]);
    zb[c] = D<ND>(oc.p.zbCells[c]);
    for (int k = 0; k < nDir; ++k) {
      if (dManning) q.manningCells[c].d[k] = dManning[(size_t)k * N + c];
      if (dZb) zb[c].d[k] = dZb[(size_t)k * N + c];
    }
  }
  set_zb<D<ND>>(oc.cs, q, zb);
  int nQ = (int)oc.p.inletQ.size();
  q.inletQ.resize(nQ);
  for (int b = 0; b < nQ; ++b) {
    q.inletQ[b] = D<ND>(oc.p.inletQ[b]);
    for (int k = 0; k < nDir; ++k)
      if (dInletQ) q.inletQ[b].d[k] = dInletQ[(size_t)k * nQ + b];
  }
  q.exitWSE.resize(oc.p.exitWSE.size());
  for (size_t b = 0; b < oc.p.exitWSE.size(); ++b) q.exitWSE[b] = D<ND>(oc.p.exitWSE[b]);
  q.hydro = oc.p.hydro;
  return q;
}

// Forward run with tangents.  Loss (optional) = mean over steps k=1..K and
// probes p of (h_p^k - obs[k][p])^2 with h = xi + hstill after each step.
template <int ND>
int run_tangent(OracleCase& oc, const double* Q0, int nsteps, double dt, int nDir, const double* dManning,
                const double* dZb, const double* dInletQ, int nProbe, const int* probes, const double* obs,
                double* Qout, double* dQout, double* loss, double* dloss, int nthreads, int method = 0) {
  const int N = oc.cs.mesh.nCells;
  Params<D<ND>> q = lift_params<ND>(oc, nDir, dManning, dZb, dInletQ);
  std::vector<D<ND>> Q(3 * (size_t)N);
  for (size_t k = 0; k < Q.size(); ++k) Q[k] = D<ND>(Q0[k]);
  D<ND> L(0.0);
  for (int s = 0; s < nsteps; ++s) {
    if (method == 1) tsit5_fixed_step<D<ND>>(oc.cs, q, Q, dt, nthreads, s * dt);
    else rk2_step<D<ND>>(oc.cs, q, Q, dt, nthreads, s * dt);
    for (int pi = 0; pi < nProbe; ++pi) {
      int c = probes[pi];
      D<ND> e = (Q[c] + oc.cs.hstill[c]) - obs[(size_t)s * nProbe + pi];
      L = L + e * e;
    }
  }
  if (nProbe > 0) L = L / (double(nsteps) * nProbe);
  if (Qout)
    for (size_t k = 0; k < Q.size(); ++k) Qout[k] = Q[k].v;
  if (dQout)
    for (int d = 0; d < nDir; ++d)
      for (size_t k = 0; k < Q.size(); ++k) dQout[(size_t)d * Q.size() + k] = Q[k].d[d];
  if (loss) *loss = L.v;
  if (dloss)
    for (int d = 0; d < nDir; ++d) dloss[d] = L.d[d];
  return 0;
}

}  // namespace

extern "C" {

const char* ho_last_error() { return g_err.c_str(); }

// bcTypes per NodeString: 0 wall, 1 symm, 2 inlet-Q, 3 exit-H, -1 not a boundary.
void* ho_create(int nNodes, const double* x, const double* y, const double* z, int nCells, const int* cellNodesCount,
                const int* cellNodes8, int nStrings, const int* stringIds, const int* stringOffsets,
                const int* stringNodes, const int* bcTypes, double g, double k_n, double h_small) {
  try {
    std::vector<NodeString> strings;
    for (int s = 0; s < nStrings; ++s) {
      NodeString ns;
      ns.id = stringIds[s];
      ns.bc = bcTypes[s];
      ns.nodes.assign(stringNodes + stringOffsets[s], stringNodes + stringOffsets[s + 1]);
      strings.push_back(ns);
    }
    auto oc = std::make_unique<OracleCase>();
    oc->cs.mesh = build_mesh(nNodes, x, y, z, nCells, cellNodesCount, cellNodes8, strings);
    oc->cs.bcs = build_bcs(oc->cs.mesh);
    oc->cs.k.g = g;
    oc->cs.k.k_n = k_n;
    oc->cs.k.h_small = h_small;
    const Mesh& m = oc->cs.mesh;
    std::vector<double> zc = nodes_to_cells(m, m.nodeZ);   // setup_bed (process_bed_2D.jl:9-43)
    set_zb<double>(oc->cs, oc->p, zc);
    oc->p.manningCells.assign(m.nCells, 0.03);
    oc->p.inletQ.assign(oc->cs.bcs.inletQ.size(), 0.0);
    oc->p.exitWSE.assign(oc->cs.bcs.exitH.size(), 0.0);
    oc->cs.hstill.assign(m.nCells, 0.0);
    oc->cs.hstillGhost.assign(m.allBoundaryFaces.size(), 0.0);
    return oc.release();
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

void ho_destroy(void* h) { delete static_cast<OracleCase*>(h); }

// Sizes: [nCells, nFaces, nGhosts, nInletQ, nExitH, nWall, nSymm]
void ho_sizes(void* h, int* out) {
  auto* oc = static_cast<OracleCase*>(h);
  const Mesh& m = oc->cs.mesh;
  out[0] = m.nCells; out[1] = m.nFaces; out[2] = (int)m.allBoundaryFaces.size();
  out[3] = (int)oc->cs.bcs.inletQ.size(); out[4] = (int)oc->cs.bcs.exitH.size();
  out[5] = (int)oc->cs.bcs.wall.size(); out[6] = (int)oc->cs.bcs.symm.size();
}

// Mesh arrays: cellFaces [N*8], cellNeighbors [N*8] (ghost id for boundary faces),
// faceIsBoundary [F], areas [N], normals [N*16], faceLengths [F], faceNodes [F*2].
void ho_mesh_arrays(void* h, int* cellFaces, int* cellNeighbors, int* faceIsBoundary, double* areas,
                    double* normals, double* faceLengths, int* faceNodes, double* cellCentroids) {
  auto* oc = static_cast<OracleCase*>(h);
  const Mesh& m = oc->cs.mesh;
  if (cellFaces) std::memcpy(cellFaces, m.cellFaces.data(), m.cellFaces.size() * sizeof(int));
  if (cellNeighbors) std::memcpy(cellNeighbors, m.cellNeighbors.data(), m.cellNeighbors.size() * sizeof(int));
  if (faceIsBoundary)
    for (int f = 0; f < m.nFaces; ++f) faceIsBoundary[f] = m.faceIsBoundary[f];
  if (areas) std::memcpy(areas, m.cellAreas.data(), m.nCells * sizeof(double));
  if (normals) std::memcpy(normals, m.cellNormals.data(), m.cellNormals.size() * sizeof(double));
  if (faceLengths) std::memcpy(faceLengths, m.faceLengths.data(), m.nFaces * sizeof(double));
  if (faceNodes)
    for (int f = 0; f < m.nFaces; ++f) { faceNodes[2 * f] = m.faceNodes[f][0]; faceNodes[2 * f + 1] = m.faceNodes[f][1]; }
  if (cellCentroids)
    for (int c = 0; c < m.nCells; ++c) { cellCentroids[2 * c] = m.cellCx[c]; cellCentroids[2 * c + 1] = m.cellCy[c]; }
}

// Bed: zb cells [N], S0 [N*2] (x,y interleaved), zb faces [F].
void ho_bed(void* h, double* zbCells, double* S0, double* zbFaces) {
  auto* oc = static_cast<OracleCase*>(h);
  const int N = oc->cs.mesh.nCells;
  if (zbCells) std::memcpy(zbCells, oc->p.zbCells.data(), N * sizeof(double));
  if (S0)
    for (int c = 0; c < N; ++c) { S0[2 * c] = oc->p.bed.S0x[c]; S0[2 * c + 1] = oc->p.bed.S0y[c]; }
  if (zbFaces) std::memcpy(zbFaces, oc->p.bed.zbFaces.data(), oc->cs.mesh.nFaces * sizeof(double));
}

// hstill = wstill - zb_cells for cells; ghost hstill = hstill of the internal cell.
void ho_set_wstill(void* h, const double* wstill) {
  auto* oc = static_cast<OracleCase*>(h);
  const Mesh& m = oc->cs.mesh;
  for (int c = 0; c < m.nCells; ++c) oc->cs.hstill[c] = wstill[c] - oc->p.zbCells[c];
  for (size_t g = 0; g < m.allBoundaryFaces.size(); ++g)
    oc->cs.hstillGhost[g] = oc->cs.hstill[m.faceCells[m.allBoundaryFaces[g]][0]];
}
void ho_set_hstill(void* h, const double* hstill) {
  auto* oc = static_cast<OracleCase*>(h);
  const Mesh& m = oc->cs.mesh;
  std::memcpy(oc->cs.hstill.data(), hstill, m.nCells * sizeof(double));
  for (size_t g = 0; g < m.allBoundaryFaces.size(); ++g)
    oc->cs.hstillGhost[g] = oc->cs.hstill[m.faceCells[m.allBoundaryFaces[g]][0]];
}
void ho_get_hstill(void* h, double* hstill) {
  auto* oc = static_cast<OracleCase*>(h);
  std::memcpy(hstill, oc->cs.hstill.data(), oc->cs.mesh.nCells * sizeof(double));
}

void ho_set_manning_cells(void* h, const double* n) {
  auto* oc = static_cast<OracleCase*>(h);
  oc->p.manningCells.assign(n, n + oc->cs.mesh.nCells);
}
// The zb parameter path (semi_discretize_swe_2D.jl:114-126): replaces zb_cells and
// recomputes ghost/face/S0 values; hstill is left unchanged.
void ho_set_zb_cells(void* h, const double* zb) {
  auto* oc = static_cast<OracleCase*>(h);
  std::vector<double> z(zb, zb + oc->cs.mesh.nCells);
  set_zb<double>(oc->cs, oc->p, z);
}
void ho_set_inletq(void* h, const double* q, int n) {
  auto* oc = static_cast<OracleCase*>(h);
  oc->p.inletQ.assign(q, q + n);
}
void ho_set_exith(void* h, const double* wse, int n) {
  auto* oc = static_cast<OracleCase*>(h);
  oc->p.exitWSE.assign(wse, wse + n);
}

int ho_rhs(void* h, const double* Q, double* dQ, int nthreads) {
  auto* oc = static_cast<OracleCase*>(h);
  try {
    rhs<double>(oc->cs, oc->p, Q, dQ, nthreads);
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// Riemann solver of the faces: 0 Roe (swe_2D_solvers.jl:4-164), 1 HLL (hgo::hll_flux).
int ho_set_riemann(void* h, int kind) {
  auto* oc = static_cast<OracleCase*>(h);
  if (kind != RIEMANN_ROE && kind != RIEMANN_HLL) {
    g_err = "ho_set_riemann: 0 (Roe) or 1 (HLL)";
    return 1;
  }
  oc->cs.k.riemann = kind;
  return 0;
}

// Inlet-Q hydrograph of group g (hgo::hydro_at); n = 0 removes it.
int ho_set_hydrograph(void* h, int g, int n, const double* t, const double* q) {
  auto* oc = static_cast<OracleCase*>(h);
  if (g < 0 || g >= (int)oc->p.inletQ.size()) {
    g_err = "ho_set_hydrograph: bad group";
    return 1;
  }
  oc->p.hydro.resize(oc->p.inletQ.size());
  oc->p.hydro[g].assign(t, t + n);
  oc->p.hydro[g].insert(oc->p.hydro[g].end(), q, q + n);
  return 0;
}

// Manning's n as a function of the state (process_ManningN_2D.jl:102-213):
// kind RES_POWER_LAW..RES_H_UMAG_KS, params {n_lower, n_upper, k, h_mid}, ks per
// cell (h_Umag_ks); kind RES_CONSTANT switches back to the cells' n.
int ho_set_resistance_fn(void* h, int kind, const double* params, const double* ks) {
  auto* oc = static_cast<OracleCase*>(h);
  if (kind < RES_CONSTANT || kind > RES_H_UMAG_KS) {
    g_err = "ho_set_resistance_fn: bad kind";
    return 1;
  }
  Resistance r;
  r.kind = kind;
  if (params) { r.nLower = params[0]; r.nUpper = params[1]; r.k = params[2]; r.hMid = params[3]; }
  if (ks) r.ks.assign(ks, ks + oc->cs.mesh.nCells);
  oc->p.res = r;
  return 0;
}
// UDE closures (process_ManningN_2D.jl:216-273, process_FlowResistance_UDE.jl:3-45)
// with the network of process_UDE.jl:3-56 (hgo::Mlp).
int ho_set_ude(void* h, int kind, int inDim, int nHidden, const int* hidden, const int* act, const double* params,
               int nParams, double outLo, double outHi, const double* hB, const double* uB, const double* ksB,
               const double* ks, int overBatch) {
  auto* oc = static_cast<OracleCase*>(h);
  Resistance r;
  r.kind = kind;
  r.mlp.inDim = inDim;
  r.mlp.hidden.assign(hidden, hidden + nHidden);
  r.mlp.act.assign(act, act + nHidden);
  r.mlp.params.assign(params, params + nParams);
  r.mlp.outLo = outLo;
  r.mlp.outHi = outHi;
  r.mlp.overBatch = overBatch != 0;
  if ((size_t)nParams != r.mlp.n_params()) {
    g_err = "ho_set_ude: parameter count does not match the layer sizes";
    return 1;
  }
  for (int i = 0; i < 2; ++i) {
    r.hB[i] = hB ? hB[i] : 0.0;
    r.uB[i] = uB ? uB[i] : 0.0;
    r.ksB[i] = ksB ? ksB[i] : 0.0;
  }
  if (ks) r.ks.assign(ks, ks + oc->cs.mesh.nCells);
  oc->p.res = r;
  return 0;
}
// The resistance field of the state Q (after the RHS's clamp): n per cell, or
// the flow-resistance magnitude for the flow-resistance closure.
int ho_resistance_cells(void* h, const double* Q, double* out) {
  auto* oc = static_cast<OracleCase*>(h);
  const int N = oc->cs.mesh.nCells;
  const double hs = oc->cs.k.h_small;
  std::vector<double> hh(N), qx(N), qy(N), r;
  for (int i = 0; i < N; ++i) {
    const double d = Q[i] + oc->cs.hstill[i];
    const bool dry = d <= hs;
    hh[i] = dry ? hs : d;
    qx[i] = dry ? 0.0 : Q[N + i];
    qy[i] = dry ? 0.0 : Q[2 * N + i];
  }
  if (oc->p.res.kind == RES_CONSTANT) r = oc->p.manningCells;
  else resistance_cells(oc->p.res, hh, qx, qy, r);
  std::memcpy(out, r.data(), sizeof(double) * N);
  return 0;
}
// The n functions alone at given (h, Umag, ks), with h/ks, f and Re of h_Umag_ks.
int ho_manning_fn(int kind, const double* params, int n, const double* hh, const double* umag, const double* ks,
                  double* nOut, double* hks, double* ff, double* re) {
  Resistance r;
  r.kind = kind;
  r.nLower = params[0]; r.nUpper = params[1]; r.k = params[2]; r.hMid = params[3];
  for (int i = 0; i < n; ++i) {
    double a = 0, b = 0, c = 0;
    nOut[i] = manning_fn(r, hh[i], umag ? umag[i] : 0.0, ks ? ks[i] : 0.0, &a, &b, &c);
    if (hks) hks[i] = a;
    if (ff) ff[i] = b;
    if (re) re[i] = c;
  }
  return 0;
}

void ho_friction(void* h, const double* hh, const double* qx, const double* qy, double* fx, double* fy) {
  auto* oc = static_cast<OracleCase*>(h);
  const auto& k = oc->cs.k;
  for (int c = 0; c < oc->cs.mesh.nCells; ++c) {
    double fr = friction_factor<double>(k.g, k.k_n, k.h_small, oc->p.manningCells[c], hh[c], qx[c], qy[c]);
    fx[c] = fr * qx[c];
    fy[c] = fr * qy[c];
  }
}

double ho_cfl_dt(void* h, const double* Q, double cfl) {
  return cfl_dt(static_cast<OracleCase*>(h)->cs, Q, cfl);
}

// nsteps SSP-RK2 steps in place.  dt > 0: fixed step; dt <= 0: CFL step recomputed
// from the state before every step.  dtOut (optional) receives the steps used.
int ho_rk2(void* h, double* Q, int nsteps, double dt, double cfl, int nthreads, double* dtOut) {
  auto* oc = static_cast<OracleCase*>(h);
  try {
    std::vector<double> q(Q, Q + 3 * (size_t)oc->cs.mesh.nCells);
    double t = 0.0;   // hydrographs: the run starts at t = 0
    for (int s = 0; s < nsteps; ++s) {
      double d = dt > 0 ? dt : cfl_dt(oc->cs, q.data(), cfl);
      if (dtOut) dtOut[s] = d;
      rk2_step<double>(oc->cs, oc->p, q, d, nthreads, t);
      t += d;
    }
    std::memcpy(Q, q.data(), q.size() * sizeof(double));
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// Tsit5 from t0 to t1 (hgo::tsit5); stats[3] = accepted, rejected, RHS evaluations.
int ho_tsit5(void* h, double* Q, double t0, double t1, double abstol, double reltol, double dt0, int adaptive,
             int maxSteps, int nthreads, int* stats) {
  auto* oc = static_cast<OracleCase*>(h);
  try {
    std::vector<double> q(Q, Q + 3 * (size_t)oc->cs.mesh.nCells);
    Tsit5Stats st;
    if (!adaptive && !(dt0 > 0)) {
      g_err = "tsit5: fixed steps need dt0 > 0";
      return 1;
    }
    if (!tsit5(oc->cs, oc->p, q, t0, t1, abstol, reltol, dt0, adaptive != 0, maxSteps > 0 ? maxSteps : 10000000, st,
               nthreads)) {
      g_err = "tsit5: step limit or step-size underflow";
      return 1;
    }
    std::memcpy(Q, q.data(), q.size() * sizeof(double));
    if (stats) {
      stats[0] = st.accepted;
      stats[1] = st.rejected;
      stats[2] = st.evals;
    }
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// Reference forward-Euler loop with its clamp (custom_ODE_solvers.jl:5-33).
int ho_euler_reference(void* h, double* Q, int nsteps, double dt, int nthreads) {
  auto* oc = static_cast<OracleCase*>(h);
  try {
    std::vector<double> q(Q, Q + 3 * (size_t)oc->cs.mesh.nCells);
    for (int s = 0; s < nsteps; ++s) euler_step_reference<double>(oc->cs, oc->p, q, dt, nthreads);
    std::memcpy(Q, q.data(), q.size() * sizeof(double));
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// Forward-mode tangent run of nsteps fixed-dt SSP-RK2 (method 0) or Tsit5
// (method 1) steps (nDir <= 8 directions).
// Tangent seeds: dManning [nDir*N] (per-cell n), dZb [nDir*N] (per-cell zb, the
// active zb parameter path), dInletQ [nDir*nInlet]; any may be NULL.
static int tangent_entry(void* h, const double* Q0, int nsteps, double dt, int nDir, const double* dManning,
                         const double* dZb, const double* dInletQ, int nProbe, const int* probes, const double* obs,
                         double* Qout, double* dQout, double* loss, double* dloss, int nthreads, int method) {
  auto* oc = static_cast<OracleCase*>(h);
  try {
    if (nDir <= 1)
      return run_tangent<1>(*oc, Q0, nsteps, dt, nDir, dManning, dZb, dInletQ, nProbe, probes, obs, Qout, dQout, loss,
                            dloss, nthreads, method);
    if (nDir <= 3)
      return run_tangent<3>(*oc, Q0, nsteps, dt, nDir, dManning, dZb, dInletQ, nProbe, probes, obs, Qout, dQout, loss,
                            dloss, nthreads, method);
    if (nDir <= 8)
      return run_tangent<8>(*oc, Q0, nsteps, dt, nDir, dManning, dZb, dInletQ, nProbe, probes, obs, Qout, dQout, loss,
                            dloss, nthreads, method);
    g_err = "nDir > 8";
    return 2;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

int ho_rk2_tangent(void* h, const double* Q0, int nsteps, double dt, int nDir, const double* dManning,
                   const double* dZb, const double* dInletQ, int nProbe, const int* probes, const double* obs,
                   double* Qout, double* dQout, double* loss, double* dloss, int nthreads) {
  return tangent_entry(h, Q0, nsteps, dt, nDir, dManning, dZb, dInletQ, nProbe, probes, obs, Qout, dQout, loss, dloss,
                       nthreads, 0);
}

int ho_tsit5_tangent(void* h, const double* Q0, int nsteps, double dt, int nDir, const double* dManning,
                     const double* dZb, const double* dInletQ, int nProbe, const int* probes, const double* obs,
                     double* Qout, double* dQout, double* loss, double* dloss, int nthreads) {
  return tangent_entry(h, Q0, nsteps, dt, nDir, dManning, dZb, dInletQ, nProbe, probes, obs, Qout, dQout, loss, dloss,
                       nthreads, 1);
}

// Loss of nsteps fixed Tsit5 steps without tangents (for central finite differences).
int ho_tsit5_loss(void* h, const double* Q0, int nsteps, double dt, int nProbe, const int* probes, const double* obs,
                  double* Qout, double* loss, int nthreads) {
  auto* oc = static_cast<OracleCase*>(h);
  try {
    const int N = oc->cs.mesh.nCells;
    std::vector<double> q(Q0, Q0 + 3 * (size_t)N);
    double L = 0.0;
    for (int s = 0; s < nsteps; ++s) {
      tsit5_fixed_step<double>(oc->cs, oc->p, q, dt, nthreads, s * dt);
      for (int pi = 0; pi < nProbe; ++pi) {
        int c = probes[pi];
        double e = (q[c] + oc->cs.hstill[c]) - obs[(size_t)s * nProbe + pi];
        L = L + e * e;
      }
    }
    if (nProbe > 0) L = L / (double(nsteps) * nProbe);
    if (Qout) std::memcpy(Qout, q.data(), q.size() * sizeof(double));
    if (loss) *loss = L;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

// Loss of a forward run without tangents (for central finite differences).
int ho_rk2_loss(void* h, const double* Q0, int nsteps, double dt, int nProbe, const int* probes, const double* obs,
                double* Qout, double* loss, int nthreads) {
  auto* oc = static_cast<OracleCase*>(h);
  try {
    const int N = oc->cs.mesh.nCells;
    std::vector<double> q(Q0, Q0 + 3 * (size_t)N);
    double L = 0.0;
    for (int s = 0; s < nsteps; ++s) {
      rk2_step<double>(oc->cs, oc->p, q, dt, nthreads, s * dt);
      for (int pi = 0; pi < nProbe; ++pi) {
        int c = probes[pi];
        double e = (q[c] + oc->cs.hstill[c]) - obs[(size_t)s * nProbe + pi];
        L = L + e * e;
      }
    }
    if (nProbe > 0) L = L / (double(nsteps) * nProbe);
    if (Qout) std::memcpy(Qout, q.data(), q.size() * sizeof(double));
    if (loss) *loss = L;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}

}  // extern "C"
