// Host driver of the discrete adjoint of SSP-RK2 with checkpointing.
//
// Forward step (fixed dt), C the depth-positivity clamp:
//   Q1 = C(Q0 + dt R(Q0)),   Q2 = C(0.5 (Q0 + (Q1 + dt R(Q1))))
// Loss = mean over steps k and probes p of (h_p^k - obs_kp)^2, h = xi + hstill
// (the probe-depth misfit), plus optionally the final-state WSE / velocity
// misfit of swe_2D_inversion.jl:383-431 (hg_final_loss.cu), which seeds the
// reverse sweep at the last state.
// Reverse step, with mu2 = dL/dQ2 masked by the stage-2 clamp:
//   mu1 = M1 (0.5 mu2 + 0.5 dt J(Q1)^T mu2)
//   mu2' = M0 (0.5 mu2 + mu1 + dt J(Q0)^T mu1)
//   dL/dtheta += 0.5 dt (dR/dtheta)(Q1)^T mu2 + dt (dR/dtheta)(Q0)^T mu1
// The forward pass stores the state at the start of every segment and keeps
// the last segment's stage states; the reverse sweep recomputes the other
// segments one at a time, keeping that segment's stage states.  A segment is
// ckpt_every steps, or as many more as the context's tape budget holds (all of
// them where it fits: no recomputation); the result is the same either way.
// Loss and parameter gradients accumulate in FP64.
#include "hg_adjoint.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "hg_adjoint_state.hpp"
#include "hg_ctx.hpp"
#include "hg_tsit5.hpp"

namespace hg {

struct AdjointBuffers {
  AdjDev dev;
  std::vector<void*> fixed;   // allocations sized by the mesh
  double* ckpt = nullptr;
  size_t ckptStates = 0;
  double* seg = nullptr;
  size_t segStates = 0;
  double *mu1 = nullptr, *mu2 = nullptr, *gzb = nullptr;
  double* userOut = nullptr;   // [2 n] the n and zb gradients in the caller's cell order
  int32_t* probes = nullptr;
  int32_t* probeCsr = nullptr;   // FP32C: probes grouped by cell (ProbeCsr), <= 4 P + 1 entries
  std::vector<int32_t> bndIndexOf;   // device cell -> its index among the boundary cells, or -1
  double* obs = nullptr;
  size_t probeCap = 0, obsCap = 0;
  double* segTot = nullptr;      // FP32C: inlet totals of a segment's states
  size_t segTotCap = 0;
  // Final-state loss: observations (wse, u, v, zbw; device order), dL/dWSE,
  // the two loss sums and the reduction scratch.
  double* fin = nullptr;
  double* lam = nullptr;          // [3n] final-state cotangent (hg_final_vjp), device order
  double* finScratch = nullptr;   // dWse [n], parts [2], partials [2 kFinalLossBlocks]
  unsigned int* finTicket = nullptr;
  double* resGrad = nullptr;      // [4] the parameter gradient of a state-dependent n
  size_t udeCap = 0;              // parameters gTheta and udePart are sized for
  float4* bndJ = nullptr;         // FP32C folded boundary VJP: flux Jacobians of a segment's states
  size_t bndJCap = 0;             // states
  int32_t* tileProbe = nullptr;   // folded: per interior-VJP tile its distinct probe cells (CSR)
  size_t tileProbeCap = 0;
  float* probeSeeds = nullptr;    // folded: a segment's probe seeds [steps][distinct probe cells]
  size_t probeSeedCap = 0;
  double* lossPart = nullptr;     // folded: the probe loss sum of each step's state [K]
  size_t lossPartCap = 0;
  double* tsit5 = nullptr;        // fixed-step Tsit5 adjoint: kTsit5Vectors state vectors (in fixed)
  ~AdjointBuffers() {
    for (void* p : fixed) cudaFree(p);
    cudaFree(ckpt);
    cudaFree(seg);
    cudaFree(probes);
    cudaFree(probeCsr);
    cudaFree(obs);
    cudaFree(segTot);
    cudaFree(fin);
    cudaFree(lam);
    cudaFree(finScratch);
    cudaFree(finTicket);
    cudaFree(dev.gTheta);
    cudaFree(dev.udePart);
    cudaFree(bndJ);
    cudaFree(tileProbe);
    cudaFree(probeSeeds);
    cudaFree(lossPart);
  }
};

namespace {

int fail(hg_ctx* c, int code, const std::string& m) {
  c->err = m;
  return code;
}

#define ADJ_CUDA(c, call)                                                                        \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return fail((c), HG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
cudaError_t falloc(AdjointBuffers* b, T** p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
  if (e == cudaSuccess) {
    b->fixed.push_back(q);
    *p = static_cast<T*>(q);
  }
  return e;
}

int setup(hg_ctx* c) {
  if (c->adj) return HG_OK;
  auto* b = new AdjointBuffers();
  c->adj = b;
  const HostMesh& m = c->hm;
  const int N = c->n;
  AdjDev& a = b->dev;
  ADJ_CUDA(c, falloc(b, &a.gN, N));
  ADJ_CUDA(c, falloc(b, &a.gS0x, N));
  ADJ_CUDA(c, falloc(b, &a.gS0y, N));
  ADJ_CUDA(c, falloc(b, &a.gZb, N));
  if (c->precision == HG_FP32C) ADJ_CUDA(c, falloc(b, &a.accF, (size_t)4 * N));
  ADJ_CUDA(c, falloc(b, &a.bfGradQ, c->dm.nbf));
  ADJ_CUDA(c, falloc(b, &a.bfGradTA, c->dm.nbf));
  ADJ_CUDA(c, falloc(b, &a.gQ, c->dm.nInlet));
  ADJ_CUDA(c, falloc(b, &a.loss, 1));
  ADJ_CUDA(c, falloc(b, &b->mu1, (size_t)3 * N));
  ADJ_CUDA(c, falloc(b, &b->mu2, (size_t)3 * N));
  ADJ_CUDA(c, falloc(b, &b->gzb, N));
  ADJ_CUDA(c, falloc(b, &b->userOut, (size_t)2 * N));
  // Inlet tables: boundary-face index of each inlet CSR entry (faces numbered
  // by face id, as the forward tables), and per group the distinct cells with
  // the sum of L^(5/3) over their faces in the group.
  std::vector<int> bfOf(m.nFaces, -1);
  int nbf = 0;
  for (int f = 0; f < m.nFaces; ++f)
    if (m.faceC1[f] < 0) bfOf[f] = nbf++;
  std::vector<int32_t> inletBf, uOff(1, 0), uCell;
  std::vector<double> uCoef;
  for (int g : m.inletGroups) {
    std::map<int, double> coef;   // caller cell id -> sum L^(5/3)
    std::vector<int> order;
    for (int f : m.bnd[g].faces) {
      inletBf.push_back(bfOf[f]);
      const int cell = m.faceC0[f];
      if (!coef.count(cell)) order.push_back(cell);
      coef[cell] += std::pow(m.faceLen[f], 5.0 / 3.0);
    }
    for (int cell : order) {
      uCell.push_back(c->inv[cell]);
      uCoef.push_back(coef[cell]);
    }
    uOff.push_back((int32_t)uCell.size());
  }
  int32_t *dBf, *dUOff, *dUCell;
  double* dUCoef;
  ADJ_CUDA(c, falloc(b, &dBf, inletBf.size()));
  ADJ_CUDA(c, falloc(b, &dUOff, uOff.size()));
  ADJ_CUDA(c, falloc(b, &dUCell, uCell.size()));
  ADJ_CUDA(c, falloc(b, &dUCoef, uCoef.size()));
  if (!inletBf.empty()) ADJ_CUDA(c, cudaMemcpy(dBf, inletBf.data(), inletBf.size() * 4, cudaMemcpyHostToDevice));
  ADJ_CUDA(c, cudaMemcpy(dUOff, uOff.data(), uOff.size() * 4, cudaMemcpyHostToDevice));
  if (!uCell.empty()) {
    ADJ_CUDA(c, cudaMemcpy(dUCell, uCell.data(), uCell.size() * 4, cudaMemcpyHostToDevice));
    ADJ_CUDA(c, cudaMemcpy(dUCoef, uCoef.data(), uCoef.size() * 8, cudaMemcpyHostToDevice));
  }
  a.inletBf = dBf;
  a.inletUOff = dUOff;
  a.inletUCell = dUCell;
  a.inletUCoef = dUCoef;
  // Cells with a boundary face, in device order, with the inlet (group,
  // sum L^(5/3)) pairs of each.
  std::map<int, std::vector<std::pair<int32_t, double>>> inletOf;   // device cell -> pairs
  for (size_t g = 0; g + 1 < uOff.size(); ++g)
    for (int32_t u = uOff[g]; u < uOff[g + 1]; ++u) inletOf[uCell[u]].push_back({(int32_t)g, uCoef[u]});
  std::vector<int32_t> bnd, bOff(1, 0), bGrp;
  std::vector<double> bCoef;
  for (int i = 0; i < N; ++i) {
    const int o = c->perm[i];
    for (int k = 0; k < m.ncf[o]; ++k)
      if (m.nbr[(size_t)o * 8 + k] < 0) {
        bnd.push_back(i);
        auto it = inletOf.find(i);
        if (it != inletOf.end())
          for (auto& pr : it->second) {
            bGrp.push_back(pr.first);
            bCoef.push_back(pr.second);
          }
        bOff.push_back((int32_t)bGrp.size());
        break;
      }
  }
  int32_t *dBnd, *dBOff, *dBGrp;
  double* dBCoef;
  ADJ_CUDA(c, falloc(b, &dBnd, bnd.size()));
  ADJ_CUDA(c, falloc(b, &dBOff, bOff.size()));
  ADJ_CUDA(c, falloc(b, &dBGrp, bGrp.size()));
  ADJ_CUDA(c, falloc(b, &dBCoef, bCoef.size()));
  if (!bnd.empty()) ADJ_CUDA(c, cudaMemcpy(dBnd, bnd.data(), bnd.size() * 4, cudaMemcpyHostToDevice));
  ADJ_CUDA(c, cudaMemcpy(dBOff, bOff.data(), bOff.size() * 4, cudaMemcpyHostToDevice));
  if (!bGrp.empty()) {
    ADJ_CUDA(c, cudaMemcpy(dBGrp, bGrp.data(), bGrp.size() * 4, cudaMemcpyHostToDevice));
    ADJ_CUDA(c, cudaMemcpy(dBCoef, bCoef.data(), bCoef.size() * 8, cudaMemcpyHostToDevice));
  }
  a.bndCells = dBnd;
  a.nBndCells = (int32_t)bnd.size();
  b->bndIndexOf.assign(N, -1);
  for (size_t i = 0; i < bnd.size(); ++i) b->bndIndexOf[bnd[i]] = (int32_t)i;
  ADJ_CUDA(c, falloc(b, &a.bndProbe, bnd.size()));
  a.bndInOff = dBOff;
  a.bndInGrp = dBGrp;
  a.bndInCoef = dBCoef;
  ADJ_CUDA(c, falloc(b, &a.bndG, (size_t)5 * bnd.size()));
  ADJ_CUDA(c, falloc(b, &a.grpTA, (size_t)c->dm.nInlet));
  ADJ_CUDA(c, falloc(b, &a.tileTicket, 3));
  ADJ_CUDA(c, cudaMemset(a.tileTicket, 0, 3 * sizeof(unsigned int)));
  // Folded boundary VJP (FP32C): the cell and slot of each boundary face, and
  // per interior-VJP tile the inlet groups whose cells it holds.
  if (c->precision == HG_FP32C && (int)m.inletGroups.size() <= kFoldMaxGroups) {
    std::vector<int2> bfSlot((size_t)std::max(nbf, 1), make_int2(0, 0));
    for (int i = 0; i < N; ++i) {
      const int o = c->perm[i];
      for (int k = 0; k < m.ncf[o]; ++k)
        if (m.nbr[(size_t)o * 8 + k] < 0) bfSlot[bfOf[m.cf[(size_t)o * 8 + k]]] = make_int2(i, k);
    }
    const int nTiles = (N + kStageBlockF32 - 1) / kStageBlockF32;
    std::vector<uint32_t> tileGrp((size_t)std::max(nTiles, 1), 0u);
    std::vector<int32_t> grpTile(std::max<size_t>(m.inletGroups.size(), 1), -1);
    for (size_t g = 0; g < m.inletGroups.size(); ++g)
      for (int f : m.bnd[m.inletGroups[g]].faces) {
        const int t = c->inv[m.faceC0[f]] / kStageBlockF32;
        tileGrp[t] |= 1u << g;
        if (grpTile[g] < 0 || t < grpTile[g]) grpTile[g] = t;
      }
    // per inlet CSR entry (the forward's group order): face, cell, len / area
    std::vector<float4> inletW;
    for (size_t g = 0; g < m.inletGroups.size(); ++g)
      for (int f : m.bnd[m.inletGroups[g]].faces) {
        const int bfi = bfOf[f], cell = c->inv[m.faceC0[f]];
        float4 v;
        std::memcpy(&v.x, &bfi, sizeof(float));
        std::memcpy(&v.y, &cell, sizeof(float));
        v.z = (float)m.faceLen[f] / (float)m.area[m.faceC0[f]];
        v.w = 0.0f;
        inletW.push_back(v);
      }
    float4* dInletW;
    ADJ_CUDA(c, falloc(b, &dInletW, std::max<size_t>(inletW.size(), 1)));
    if (!inletW.empty())
      ADJ_CUDA(c, cudaMemcpy(dInletW, inletW.data(), inletW.size() * sizeof(float4), cudaMemcpyHostToDevice));
    a.inletW = dInletW;
    int2* dSlot;
    uint32_t* dTileGrp;
    int32_t* dGrpTile;
    ADJ_CUDA(c, falloc(b, &dSlot, bfSlot.size()));
    ADJ_CUDA(c, falloc(b, &dTileGrp, tileGrp.size()));
    ADJ_CUDA(c, falloc(b, &dGrpTile, grpTile.size()));
    ADJ_CUDA(c, cudaMemcpy(dSlot, bfSlot.data(), bfSlot.size() * sizeof(int2), cudaMemcpyHostToDevice));
    ADJ_CUDA(c, cudaMemcpy(dTileGrp, tileGrp.data(), tileGrp.size() * 4, cudaMemcpyHostToDevice));
    ADJ_CUDA(c, cudaMemcpy(dGrpTile, grpTile.data(), grpTile.size() * 4, cudaMemcpyHostToDevice));
    a.bfSlot = dSlot;
    a.tileGrp = dTileGrp;
    a.grpTile = dGrpTile;
  }
  return HG_OK;
}

// Segment length: at least the caller's spacing C, and as long as the
// stage-state tape of one segment (2 C + 1 states of 24 bytes per cell) fits
// in the context's budget -- all K steps where it fits.
int segment_length(hg_ctx* c, int K, int C) {
  if (c->adjTapeBytes == 0) return C;
  const size_t state = (size_t)24 * c->n;
  size_t budget = (size_t)c->adjTapeBytes;
  if (c->adjTapeBytes < 0) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      cudaGetLastError();
      return C;
    }
    fr += c->adj->segStates * state;   // a longer tape replaces the present one
    budget = std::min(fr / 2, tot / 4);
  }
  const size_t fit = budget / state;   // states
  if (fit < 3) return C;
  return std::max(C, (int)std::min<size_t>((fit - 1) / 2, (size_t)K));
}

int reserve(hg_ctx* c, double** p, size_t* have, size_t states) {
  if (states <= *have) return HG_OK;
  cudaFree(*p);
  *p = nullptr;
  *have = 0;
  ADJ_CUDA(c, cudaMalloc(p, states * 3 * (size_t)c->n * sizeof(double)));
  *have = states;
  return HG_OK;
}

}  // namespace

namespace {

// FP32-compensated state buffer of `states` states: [states][n] float4 then [states][n] float2.
struct F32States {
  float4* x = nullptr;
  float2* q = nullptr;
  StateF32 at(size_t i, int n) const { return StateF32{x + i * (size_t)n, q + i * (size_t)n}; }
};

F32States f32_view(double* base, size_t states, int n) {
  F32States v;
  v.x = reinterpret_cast<float4*>(base);
  v.q = reinterpret_cast<float2*>(reinterpret_cast<char*>(base) + states * (size_t)n * sizeof(float4));
  return v;
}

}  // namespace

int adjoint_time_vjp(hg_ctx* c, int32_t reps, int32_t flushL2, double* avgMs) {
  if (c->precision != HG_FP32C || c->dm.res.kind != kResConstant || c->dm.nHydro != 0)
    return fail(c, HG_ERR_UNSUPPORTED,
                "hg_time_vjp_kernel: the FP32C VJP with constant resistance and inlet discharges only");
  int rc = setup(c);
  if (rc) return rc;
  AdjointBuffers* b = c->adj;
  AdjDev a = b->dev;
  a.wantN = a.wantZb = 1;
  a.resChain = a.udeChain = 0;
  const StateF32 X{c->XA, c->XQA};
  if (!vjp_fold_usable(c->dm, a, X))
    return fail(c, HG_ERR_UNSUPPORTED, "hg_time_vjp_kernel: the pipelined interior VJP cannot run on this mesh");
  cudaStream_t st = c->stream;
  const int N = c->n;
  if (b->bndJCap < 1) {
    cudaFree(b->bndJ);
    b->bndJ = nullptr;
    ADJ_CUDA(c, cudaMalloc(&b->bndJ, (size_t)std::max(c->dm.nbf, 1) * 6 * sizeof(float4)));
    b->bndJCap = 1;
  }
  DevMesh m = c->dm;
  m.totalA = c->d_tot;   // conveyance totals of the resident state
  launch_inlet_total_f32(m, c->ds, X, st);
  launch_bnd_jac_f32(m, a, X.x, 1, c->d_tot, 0, b->bndJ, st);
  a.bndJ = b->bndJ;
  float* mu = reinterpret_cast<float*>(b->mu1);
  float* out = reinterpret_cast<float*>(b->mu2);
  ADJ_CUDA(c, cudaMemsetAsync(mu, 0x3a, (size_t)3 * N * sizeof(float), st));   // about 7e-4 each
  ADJ_CUDA(c, cudaMemsetAsync(a.accF, 0, (size_t)4 * N * sizeof(float2), st));
  ADJ_CUDA(c, cudaMemsetAsync(a.gQ, 0, std::max(c->dm.nInlet, 1) * sizeof(double), st));
  c->launches += 2;
  cudaEvent_t e0, e1;
  ADJ_CUDA(c, cudaEventCreate(&e0));
  ADJ_CUDA(c, cudaEventCreate(&e1));
  double total = 0.0;
  for (int i = 0; i < reps; ++i) {
    if (flushL2) c->launches += launch_flush(c->flushBuf, c->flushBytes, st);
    cudaEventRecord(e0, st);
    c->launches += launch_vjp_f32_folded(m, a, X, mu, nullptr, out, 0.5f, 0.0f, 1e-3, st, nullptr);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    total += ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *avgMs = total / reps;
  ADJ_CUDA(c, cudaGetLastError());
  return HG_OK;
}

int adjoint_loss_and_grad(hg_ctx* c, const double* Q0, int32_t K, double dt, int32_t C, const int32_t* probeCells,
                          const double* obs, int32_t P, double* loss, double* gManning, double* gZb, double* gInlet,
                          double* Qfinal, const FinalObs* fo, double* parts) {
  const bool tsit5 = c->adjIntegrator == 1;
  if (tsit5 && !c->adjSteps.empty() && (size_t)K > c->adjSteps.size())
    return fail(c, HG_ERR_ARG, "more steps than the step sizes set by hg_set_adjoint_steps");
  int rc = setup(c);
  if (rc) return rc;
  AdjointBuffers* b = c->adj;
  AdjDev& a = b->dev;
  a.wantN = gManning ? 1 : 0;   // the FP32C VJP skips the accumulators of gradients not asked for
  a.wantZb = gZb ? 1 : 0;
  a.noMask = tsit5 ? 1 : 0;   // FP32 VJP kernels: the RHS VJP of Tsit5 stages, no clamp masks
  const int N = c->n;
  // A state-dependent Manning n (the n functions): dL/dn is chained into the
  // state and the function's parameters instead of accumulated per cell.
  a.resChain = (c->dm.res.kind >= kResPowerLaw && c->dm.res.kind <= kResHUmagKs) ? 1 : 0;
  if (!a.resChain) std::fill(c->resGrad, c->resGrad + 4, 0.0);
  if (a.resChain && !a.gResP) {
    ADJ_CUDA(c, falloc(b, &a.gResP, (size_t)4 * N));
    if (c->precision == HG_FP32C) ADJ_CUDA(c, falloc(b, &a.accRes, (size_t)4 * N));
    ADJ_CUDA(c, falloc(b, &b->resGrad, 4));
  }
  // A UDE closure: the network's VJP after each stage's VJP.
  const int rk = c->dm.res.kind;
  a.udeChain = (rk == kResUdeManningH || rk == kResUdeManningHUmagKs) ? 1 : rk == kResUdeFlowResistance ? 2 : 0;
  a.udeP = a.udeChain ? (int32_t)c->udeParams : 0;
  c->udeGrad.assign((size_t)a.udeP, 0.0);
  if (a.udeChain) {
    if (!a.udeGn) {
      ADJ_CUDA(c, falloc(b, &a.udeGn, N));
      ADJ_CUDA(c, falloc(b, &a.udeS, 2 * kResMaxLayers));
      ADJ_CUDA(c, falloc(b, &a.udeTicket, 1));
      ADJ_CUDA(c, cudaMemset(a.udeTicket, 0, sizeof(unsigned int)));
    }
    const size_t need = (size_t)std::max(a.udeP, 2);
    if (need > b->udeCap) {
      cudaFree(a.gTheta);
      cudaFree(a.udePart);
      a.gTheta = nullptr;
      a.udePart = nullptr;
      ADJ_CUDA(c, cudaMalloc(&a.gTheta, need * sizeof(double)));
      ADJ_CUDA(c, cudaMalloc(&a.udePart, need * kUdeGrid * sizeof(double)));
      b->udeCap = need;
    }
  }
  const size_t n3 = (size_t)3 * N;
  const bool f64 = c->precision == HG_FP64;
  if (C <= 0) C = K;
  C = segment_length(c, K, std::min(C, K));
  // Segments end at step K: the last one, whose stage states the forward
  // pass keeps, is a full C steps; the first takes the remainder.  Segment g
  // covers steps [seg_start(g), seg_start(g + 1)).
  const int nck = (K + C - 1) / C;
  const int segOff = nck * C - K;   // 0 <= segOff < C
  auto seg_start = [&](int g) { return std::min(K, std::max(0, g * C - segOff)); };
  auto seg_of = [&](int s) { return (s + segOff) / C; };   // the segment holding step s
  // A double-sized state slot holds one FP32-compensated state too (24 B per cell either way).
  rc = reserve(c, &b->ckpt, &b->ckptStates, (size_t)nck);
  if (rc) return rc;
  rc = reserve(c, &b->seg, &b->segStates, (size_t)(2 * C + 1));
  if (rc) return rc;
  cudaStream_t st = c->stream;
  // Probes (device order) and observations.
  if ((size_t)std::max(P, 1) > b->probeCap) {
    cudaFree(b->probes);
    cudaFree(b->probeCsr);
    b->probes = nullptr;
    b->probeCsr = nullptr;
    ADJ_CUDA(c, cudaMalloc(&b->probes, std::max(P, 1) * sizeof(int32_t)));
    ADJ_CUDA(c, cudaMalloc(&b->probeCsr, (4 * (size_t)std::max(P, 1) + 1) * sizeof(int32_t)));
    b->probeCap = std::max(P, 1);
  }
  const size_t nobs = (size_t)K * std::max(P, 0);
  if (std::max<size_t>(nobs, 1) > b->obsCap) {
    cudaFree(b->obs);
    b->obs = nullptr;
    ADJ_CUDA(c, cudaMalloc(&b->obs, std::max<size_t>(nobs, 1) * sizeof(double)));
    b->obsCap = std::max<size_t>(nobs, 1);
  }
  std::vector<int32_t> pdev(std::max(P, 0));
  for (int p = 0; p < P; ++p) pdev[p] = c->inv[probeCells[p]];
  // The same probes grouped by cell (distinct cells in order of first
  // appearance, each with its probe indices in increasing order), whether each
  // is a boundary cell, and for each boundary cell its probe cell, if any.
  std::vector<int32_t> csr, bndProbe(a.nBndCells, -1);
  ProbeCsr pc;
  {
    std::vector<int32_t> cells, off(1, 0), idx;
    std::map<int32_t, std::vector<int32_t>> at;
    for (int p = 0; p < P; ++p) {
      if (!at.count(pdev[p])) cells.push_back(pdev[p]);
      at[pdev[p]].push_back(p);
    }
    for (int32_t cell : cells) {
      for (int32_t p : at[cell]) idx.push_back(p);
      off.push_back((int32_t)idx.size());
    }
    std::vector<int32_t> isBnd(cells.size(), 0);
    for (size_t u = 0; u < cells.size(); ++u) {
      const int32_t i = b->bndIndexOf[cells[u]];
      if (i >= 0) {
        isBnd[u] = 1;
        bndProbe[i] = (int32_t)u;
      }
    }
    csr = cells;
    csr.insert(csr.end(), off.begin(), off.end());
    csr.insert(csr.end(), idx.begin(), idx.end());
    csr.insert(csr.end(), isBnd.begin(), isBnd.end());
    pc.cell = b->probeCsr;
    pc.off = b->probeCsr + cells.size();
    pc.idx = b->probeCsr + 2 * cells.size() + 1;
    pc.isBnd = b->probeCsr + 2 * cells.size() + 1 + P;
    pc.nCells = (int32_t)cells.size();
    if (c->precision == HG_FP32C && P > 0) {   // per interior-VJP tile its distinct probe cells
      const int nTiles = (N + kStageBlockF32 - 1) / kStageBlockF32;
      std::vector<int32_t> tp(nTiles + 1 + cells.size(), 0);
      for (int32_t cell : cells) ++tp[cell / kStageBlockF32 + 1];
      for (int t = 0; t < nTiles; ++t) tp[t + 1] += tp[t];
      std::vector<int32_t> fill(tp.begin(), tp.begin() + nTiles);
      for (size_t u = 0; u < cells.size(); ++u) tp[nTiles + 1 + fill[cells[u] / kStageBlockF32]++] = (int32_t)u;
      if (tp.size() > b->tileProbeCap) {
        cudaFree(b->tileProbe);
        b->tileProbe = nullptr;
        b->tileProbeCap = 0;
        ADJ_CUDA(c, cudaMalloc(&b->tileProbe, tp.size() * sizeof(int32_t)));
        b->tileProbeCap = tp.size();
      }
      ADJ_CUDA(c, cudaMemcpy(b->tileProbe, tp.data(), tp.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
      a.tileProbeOff = b->tileProbe;
      a.tileProbeU = b->tileProbe + nTiles + 1;
      a.probeCell = pc.cell;
    }
  }
  if (P > 0) {
    ADJ_CUDA(c, cudaMemcpyAsync(b->probes, pdev.data(), P * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    ADJ_CUDA(c, cudaMemcpyAsync(b->probeCsr, csr.data(), csr.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    if (a.nBndCells > 0)
      ADJ_CUDA(c, cudaMemcpyAsync(a.bndProbe, bndProbe.data(), bndProbe.size() * sizeof(int32_t),
                                  cudaMemcpyHostToDevice, st));
    ADJ_CUDA(c, cudaMemcpyAsync(b->obs, obs, nobs * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  // Accumulators and dt.
  ADJ_CUDA(c, cudaMemsetAsync(a.gN, 0, N * sizeof(double), st));
  ADJ_CUDA(c, cudaMemsetAsync(a.gS0x, 0, N * sizeof(double), st));
  ADJ_CUDA(c, cudaMemsetAsync(a.gS0y, 0, N * sizeof(double), st));
  ADJ_CUDA(c, cudaMemsetAsync(a.gZb, 0, N * sizeof(double), st));
  if (a.accF) ADJ_CUDA(c, cudaMemsetAsync(a.accF, 0, (size_t)4 * N * sizeof(float2), st));
  if (a.udeChain) ADJ_CUDA(c, cudaMemsetAsync(a.gTheta, 0, (size_t)a.udeP * sizeof(double), st));
  if (a.resChain) {
    ADJ_CUDA(c, cudaMemsetAsync(a.gResP, 0, (size_t)4 * N * sizeof(double), st));
    if (a.accRes) ADJ_CUDA(c, cudaMemsetAsync(a.accRes, 0, (size_t)4 * N * sizeof(float2), st));
  }
  ADJ_CUDA(c, cudaMemsetAsync(a.gQ, 0, std::max(c->dm.nInlet, 1) * sizeof(double), st));
  ADJ_CUDA(c, cudaMemsetAsync(a.loss, 0, sizeof(double), st));
  ADJ_CUDA(c, cudaMemsetAsync(c->ds.flags, 0, sizeof(int32_t), st));
  const float dtf = (float)dt;
  ADJ_CUDA(c, cudaMemcpyAsync(c->ds.dt, &dt, sizeof(double), cudaMemcpyHostToDevice, st));
  ADJ_CUDA(c, cudaMemcpyAsync(c->ds.dtf, &dtf, sizeof(float), cudaMemcpyHostToDevice, st));
  ADJ_CUDA(c, cudaMemcpyAsync(c->Quser, Q0, n3 * sizeof(double), cudaMemcpyHostToDevice, st));
  const double scale = (P > 0) ? 1.0 / ((double)K * P) : 0.0;
  // Final-state loss: its normalisations from the observations, as the
  // reference takes them (WSE_truth range + sqrt(eps); the largest observed
  // speed, at least eps), and the observations in device order.
  FinalLossDev fl;
  const bool useFinal = fo && (fo->wse || (fo->u && fo->v) || fo->lam);
  if (useFinal) {
    if (!b->fin) {
      ADJ_CUDA(c, cudaMalloc(&b->fin, (size_t)4 * N * sizeof(double)));
      ADJ_CUDA(c, cudaMalloc(&b->finScratch, ((size_t)N + 2 + 2 * kFinalLossBlocks) * sizeof(double)));
      ADJ_CUDA(c, cudaMalloc(&b->finTicket, sizeof(unsigned int)));
      ADJ_CUDA(c, cudaMemsetAsync(b->finTicket, 0, sizeof(unsigned int), st));
    }
    std::vector<double> dev((size_t)4 * N);
    auto put = [&](int slot, const double* v) {
      for (int i = 0; i < N; ++i) dev[(size_t)slot * N + i] = v[c->perm[i]];
    };
    fl.invN = 1.0 / (double)N;
    if (fo->wse) {
      put(0, fo->wse);
      const auto mm = std::minmax_element(fo->wse, fo->wse + N);
      fl.wseDen = (*mm.second - *mm.first) + 1.4901161193847656e-08;
      fl.wse = b->fin;
      fl.zbw = fo->zbw ? b->fin + (size_t)3 * N : c->dm.zb;
      if (fo->zbw) put(3, fo->zbw);
    }
    if (fo->u && fo->v) {
      put(1, fo->u);
      put(2, fo->v);
      double vmax = 0.0;
      for (int i = 0; i < N; ++i) vmax = std::max(vmax, std::sqrt(fo->u[i] * fo->u[i] + fo->v[i] * fo->v[i]));
      fl.velScale = std::max(vmax, 2.220446049250313e-16);
      fl.u = b->fin + N;
      fl.v = b->fin + (size_t)2 * N;
    }
    ADJ_CUDA(c, cudaMemcpyAsync(b->fin, dev.data(), dev.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    if (fo->lam) {   // the final-state cotangent, in device order
      if (!b->lam) ADJ_CUDA(c, cudaMalloc(&b->lam, (size_t)3 * N * sizeof(double)));
      std::vector<double> l((size_t)3 * N);
      for (int blk = 0; blk < 3; ++blk)
        for (int i = 0; i < N; ++i) l[(size_t)blk * N + i] = fo->lam[(size_t)blk * N + c->perm[i]];
      ADJ_CUDA(c, cudaMemcpyAsync(b->lam, l.data(), l.size() * sizeof(double), cudaMemcpyHostToDevice, st));
      fl.lam = b->lam;
    }
    fl.dWse = b->finScratch;
    fl.parts = b->finScratch + N;
    fl.partials = b->finScratch + N + 2;
    fl.ticket = b->finTicket;
  }
  const DevMesh& dm = c->dm;
  DevScalars ds = c->ds;
  ds.nMembers = 0;   // the adjoint takes one fixed dt for every member
  const int extraPerStep = 2 * dm.nInlet;
  // Inlet hydrographs at a stage's time (the run starts at t = 0): stage 1 of
  // step s at s dt, stage 2 at (s + 1) dt -- in the forward pass, the
  // recomputation and the VJP of that stage alike.
  auto hydro = [&](double t) { c->launches += launch_hydrograph(dm, ds, kHydroAt, t, st); };
  // Tsit5: the step sizes differentiated -- dt each, or the sequence
  // hg_set_adjoint_steps gave (the accepted steps of an adaptive solve, held
  // fixed), step s then starting at the sum of the sizes before it.
  const bool stepList = tsit5 && !c->adjSteps.empty();
  std::vector<double> tStart;
  if (stepList) {
    tStart.assign((size_t)K + 1, 0.0);
    for (int s = 0; s < K; ++s) tStart[s + 1] = tStart[s] + c->adjSteps[s];
  }
  auto dtOf = [&](int s) { return stepList ? c->adjSteps[s] : dt; };
  auto tOf = [&](int s) { return stepList ? tStart[s] : s * dt; };

  if (tsit5 && !f64) {
    // The fixed-step Tsit5 adjoint below in an FP32-compensated context: the
    // states and stage states as hi + lo records, the stage RHS, the stage
    // cotangents, Kbar and lam as FP32 vectors (the FP32 VJP kernels' own
    // precision); the forward arithmetic is hg_integrate_tsit5's (FP32 sums
    // of the stage terms added to the state's pairs, kModeRhsF32), and the VJP
    // kernels run unmasked (AdjDev::noMask).
    const int n = N;
    const Tsit5Tableau& tb = tsit5_tableau();
    if (!b->tsit5) ADJ_CUDA(c, falloc(b, &b->tsit5, (size_t)kTsit5Vectors * n3));
    const F32States ck = f32_view(b->ckpt, (size_t)nck, n);
    const F32States sg = f32_view(b->seg, (size_t)(2 * C + 1), n);
    // The Tsit5 buffer (18 x 24 B per cell): Y_1 .. Y_5 records (their x
    // parts, then their lo parts), then K_0 .. K_5, Ybar_0 .. Ybar_5 and Kbar.
    char* base = reinterpret_cast<char*>(b->tsit5);
    const F32States yv = f32_view(b->tsit5, 5, n);
    StateF32 Y[6];
    float *Kv[6], *Yb[6];
    for (int i = 1; i < 6; ++i) Y[i] = yv.at((size_t)(i - 1), n);
    float* fbase = reinterpret_cast<float*>(base + (size_t)5 * n * (sizeof(float4) + sizeof(float2)));
    for (int i = 0; i < 6; ++i) {
      Kv[i] = fbase + (size_t)i * n3;
      Yb[i] = fbase + (size_t)(6 + i) * n3;
    }
    float* kb = fbase + (size_t)12 * n3;
    float* lam = reinterpret_cast<float*>(b->mu1);
    float* lamNext = reinterpret_cast<float*>(b->mu2);
    StateF32 XA{c->XA, c->XQA}, XB{c->XB, c->XQB};
    auto rhs = [&](StateF32 X, float* out, double t) {
      hydro(t);
      launch_inlet_total_f32(dm, ds, X, st);   // the RHS's inlet totals (and resistance) of X
      launch_stage_f32(dm, ds, kModeRhsF32, X, StateF32{}, StateF32{}, reinterpret_cast<double*>(out), false, st);
      c->launches += 1 + (dm.nInlet > 0 ? 1 : 0) + resistance_launches(dm);
    };
    auto terms_f = [&](const float* const* K, const double* w, int nk, double h) {
      Tsit5TermsF t{};
      for (int j = 0; j < nk; ++j) {
        t.K[j] = K[j];
        t.w[j] = (float)(w[j] * h);
      }
      t.nk = nk;
      return t;
    };
    // The stages of step s from U (K_0 .. K_nk-1, Y_1 .. Y_5); Unext: the new state, or null.
    auto stages = [&](int s, StateF32 U, int nk, const StateF32* Unext) {
      const double t = tOf(s), h = dtOf(s);
      Y[0] = U;
      rhs(U, Kv[0], t);
      for (int i = 1; i < 6; ++i) {
        launch_tsit5_combine_f32(n, U, terms_f(Kv, tb.a[i], i, h), Y[i], st);
        if (i < nk) rhs(Y[i], Kv[i], t + tb.c[i] * h);
        c->launches += 1;
      }
      if (Unext) {
        launch_tsit5_combine_f32(n, U, terms_f(Kv, tb.a[6], 6, h), *Unext, st);
        c->launches += 1;
      }
    };
    auto copy_state = [&](StateF32 dst, StateF32 src) -> cudaError_t {
      cudaError_t e = cudaMemcpyAsync(dst.x, src.x, (size_t)n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(dst.q, src.q, (size_t)n * sizeof(float2), cudaMemcpyDeviceToDevice, st);
      return e;
    };
    launch_gather_state_f32(N, c->d_perm, c->Quser, XA, st);
    const int sLast = seg_start(nck - 1);
    for (int s = 0; s < K; ++s) {
      const bool last = s >= sLast;
      const size_t i = (size_t)(s - sLast);
      if (!last && s == seg_start(seg_of(s))) ADJ_CUDA(c, copy_state(ck.at(seg_of(s), n), XA));
      if (s == sLast) ADJ_CUDA(c, copy_state(sg.at(0, n), XA));
      const StateF32 u0 = last ? sg.at(i, n) : XA;
      const StateF32 u1 = last ? sg.at(i + 1, n) : XB;
      stages(s, u0, 6, &u1);
      if (!last) std::swap(XA, XB);
    }
    ADJ_CUDA(c, copy_state(XA, sg.at((size_t)(K - sLast), n)));   // the final state
    if (Qfinal) launch_scatter_state_f32(N, c->d_perm, XA, c->Quser, st);   // copied out at the end
    // Reverse sweep: the probe terms (loss and seed) of the final state, unmasked.
    ADJ_CUDA(c, cudaMemsetAsync(lam, 0, n3 * sizeof(float), st));
    launch_probe_f32(dm, a, XA, lam, pc, b->probes, b->obs + (size_t)(K - 1) * P, P, scale, st);
    c->launches += P > 0 ? 1 : 0;
    if (useFinal) {
      fl.mask = 0;
      launch_final_loss_f32(dm, fl, XA, lam, st);
      c->launches += 1;
    }
    for (int seg = nck - 1; seg >= 0; --seg) {
      const int s0 = seg_start(seg), s1 = seg_start(seg + 1);
      if (seg < nck - 1) {   // the segment's states from its checkpoint (the last one's are in place)
        ADJ_CUDA(c, copy_state(sg.at(0, n), ck.at(seg, n)));
        for (int s = s0; s < s1 - 1; ++s) {
          const StateF32 nx = sg.at((size_t)(s - s0 + 1), n);
          stages(s, sg.at((size_t)(s - s0), n), 6, &nx);
        }
      }
      for (int s = s1 - 1; s >= s0; --s) {
        const StateF32 U = sg.at((size_t)(s - s0), n);
        stages(s, U, 5, nullptr);   // K_0 .. K_4 and Y_1 .. Y_5
        for (int i = 5; i >= 0; --i) {
          Tsit5TermsF t{};   // Kbar_i = dt (b_i lam + sum_{k>i} a_ki Ybar_k)
          t.K[0] = lam;
          t.w[0] = (float)(tb.a[6][i] * dtOf(s));
          for (int k = i + 1; k < 6; ++k) {
            t.K[k - i] = Yb[k];
            t.w[k - i] = (float)(tb.a[k][i] * dtOf(s));
          }
          t.nk = 6 - i;
          launch_tsit5_lin_f32(n3, t, kb, st);
          hydro(tOf(s) + tb.c[i] * dtOf(s));
          launch_inlet_total_f32(dm, ds, Y[i], st);   // the stage's inlet totals and resistance
          c->launches += launch_vjp_f32(dm, a, Y[i], kb, nullptr, Yb[i], 0.0f, 0.0f, 1.0, st, nullptr);
          c->launches += launch_ude_vjp_f32(dm, a, Y[i], Yb[i], st);
          c->launches += 1 + (dm.nInlet > 0 ? 1 : 0) + resistance_launches(dm);
        }
        Tsit5TermsF t{};   // lam_s = lam' + sum_i Ybar_i
        t.K[0] = lam;
        t.w[0] = 1.0f;
        for (int i = 0; i < 6; ++i) {
          t.K[1 + i] = Yb[i];
          t.w[1 + i] = 1.0f;
        }
        t.nk = 7;
        launch_tsit5_lin_f32(n3, t, lamNext, st);
        std::swap(lam, lamNext);
        c->launches += 1;
        if (s >= 1) {
          launch_probe_f32(dm, a, U, lam, pc, b->probes, b->obs + (size_t)(s - 1) * P, P, scale, st);
          c->launches += P > 0 ? 1 : 0;
        }
      }
    }
  } else if (tsit5) {
    // Fixed-step Tsit5 (hg_integrate_tsit5 with adaptive = 0): step s takes
    // U_s at t_s = s dt to U_{s+1} = U_s + dt sum_{j<6} b_j K_j, with
    // K_i = f(Y_i, t_s + c_i dt), Y_0 = U_s, Y_i = U_s + dt sum_{j<i} a_ij K_j
    // (b = the tableau's last row).  Its adjoint, from lam' = dL/dU_{s+1}:
    //   Kbar_i = dt (b_i lam' + sum_{k>i} a_ki Ybar_k),  Ybar_i = J(Y_i)^T Kbar_i   (i = 5 .. 0)
    //   lam = lam' + sum_i Ybar_i  (+ the probe seed of U_s)
    // the VJP kernels accumulating the parameter terms (dR/dtheta)^T Kbar_i of
    // each stage at its own state and time.  No clamp acts on a Tsit5 state
    // (the RHS clamps its own copy of h), so nothing is masked.
    const Tsit5Tableau& tb = tsit5_tableau();
    if (!b->tsit5) ADJ_CUDA(c, falloc(b, &b->tsit5, (size_t)kTsit5Vectors * n3));
    double* Y[6];    // Y[0] = U_s (in the segment buffer); Y[1..5] here
    double* Kv[6];   // stage RHS
    double* Yb[6];   // stage cotangents
    for (int i = 0; i < 6; ++i) {
      Y[i] = i == 0 ? nullptr : b->tsit5 + (size_t)(i - 1) * n3;
      Kv[i] = b->tsit5 + (size_t)(5 + i) * n3;
      Yb[i] = b->tsit5 + (size_t)(11 + i) * n3;
    }
    double* kb = b->tsit5 + (size_t)17 * n3;
    double* lam = b->mu1;
    double* lamNext = b->mu2;
    auto rhs = [&](const double* X, double* out, double t) {
      hydro(t);
      launch_inlet_total_f64(dm, ds, X, st);
      launch_stage_f64(dm, ds, kModeRhs, X, nullptr, out, false, st);
      c->launches += 1 + (dm.nInlet > 0 ? 1 : 0) + resistance_launches(dm);
    };
    auto terms_of = [&](int i) {   // a_ij K_j, j < i (i = 6: the new state's weights b)
      Tsit5Terms t{};
      for (int j = 0; j < i; ++j) {
        t.K[j] = Kv[j];
        t.w[j] = tb.a[i][j];
      }
      t.nk = i;
      return t;
    };
    // The stages of step s from U (K_0 .. K_nk-1, Y_1 .. Y_5); Unext: the new state, or null.
    auto stages = [&](int s, const double* U, int nk, double* Unext) {
      const double t = tOf(s), h = dtOf(s);
      Y[0] = const_cast<double*>(U);
      rhs(U, Kv[0], t);
      for (int i = 1; i < 6; ++i) {
        launch_tsit5_combine(n3, U, terms_of(i), h, Y[i], st);
        if (i < nk) rhs(Y[i], Kv[i], t + tb.c[i] * h);
        c->launches += 1;
      }
      if (Unext) {
        launch_tsit5_combine(n3, U, terms_of(6), h, Unext, st);
        c->launches += 1;
      }
    };
    launch_gather_state_f64(N, c->d_perm, c->Quser, c->QA, st);
    // Forward pass: a checkpoint at each segment's start; the last segment's
    // states go straight into the segment buffer (U_s at seg + (s - sLast) n3).
    const int sLast = seg_start(nck - 1);
    for (int s = 0; s < K; ++s) {
      const bool last = s >= sLast;
      const size_t i = (size_t)(s - sLast);
      if (!last && s == seg_start(seg_of(s)))
        ADJ_CUDA(c, cudaMemcpyAsync(b->ckpt + (size_t)seg_of(s) * n3, c->QA, n3 * sizeof(double),
                                    cudaMemcpyDeviceToDevice, st));
      if (s == sLast) ADJ_CUDA(c, cudaMemcpyAsync(b->seg, c->QA, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
      const double* u0 = last ? b->seg + i * n3 : c->QA;
      double* u1 = last ? b->seg + (i + 1) * n3 : c->QB;
      stages(s, u0, 6, u1);
      launch_probe_loss_f64(dm, a, u1, b->probes, b->obs + (size_t)s * P, P, st);
      c->launches += P > 0 ? 1 : 0;
      if (!last) std::swap(c->QA, c->QB);
    }
    const double* uK = b->seg + (size_t)(K - sLast) * n3;
    ADJ_CUDA(c, cudaMemcpyAsync(c->QA, uK, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));   // the final state
    if (Qfinal) launch_scatter_state_f64(N, c->d_perm, c->QA, c->Quser, st);   // copied out at the end
    // Reverse sweep: the seed of the final state.
    ADJ_CUDA(c, cudaMemsetAsync(lam, 0, n3 * sizeof(double), st));
    launch_probe_adjoint_f64(dm, c->QA, lam, b->probes, b->obs + (size_t)(K - 1) * P, P, scale, st, false);
    if (useFinal) {
      fl.mask = 0;
      launch_final_loss_f64(dm, fl, c->QA, lam, st);
      c->launches += 1;
    }
    for (int seg = nck - 1; seg >= 0; --seg) {
      const int s0 = seg_start(seg), s1 = seg_start(seg + 1);
      if (seg < nck - 1) {   // the segment's states from its checkpoint (the last one's are in place)
        ADJ_CUDA(c, cudaMemcpyAsync(b->seg, b->ckpt + (size_t)seg * n3, n3 * sizeof(double),
                                    cudaMemcpyDeviceToDevice, st));
        for (int s = s0; s < s1 - 1; ++s)
          stages(s, b->seg + (size_t)(s - s0) * n3, 6, b->seg + (size_t)(s - s0 + 1) * n3);
      }
      for (int s = s1 - 1; s >= s0; --s) {
        const double* U = b->seg + (size_t)(s - s0) * n3;
        stages(s, U, 5, nullptr);   // K_0 .. K_4 and Y_1 .. Y_5 (K_5 enters only the new state)
        for (int i = 5; i >= 0; --i) {
          Tsit5Terms t{};   // Kbar_i = dt (b_i lam + sum_{k>i} a_ki Ybar_k)
          t.K[0] = lam;
          t.w[0] = tb.a[6][i];
          for (int k = i + 1; k < 6; ++k) {
            t.K[k - i] = Yb[k];
            t.w[k - i] = tb.a[k][i];
          }
          t.nk = 6 - i;
          launch_tsit5_combine(n3, nullptr, t, dtOf(s), kb, st);
          hydro(tOf(s) + tb.c[i] * dtOf(s));
          launch_inlet_total_f64(dm, ds, Y[i], st);   // the stage's inlet totals and resistance
          launch_vjp_f64(dm, a, Y[i], kb, nullptr, Yb[i], 0.0, 0.0, 1.0, st, false);
          launch_inlet_adjoint_f64(dm, a, Y[i], Yb[i], 1.0, st);
          c->launches += launch_ude_vjp_f64(dm, a, Y[i], Yb[i], st);
          c->launches += 3 + (dm.nInlet > 0 ? 1 + dm.nInlet : 0) + resistance_launches(dm);
        }
        Tsit5Terms t{};   // lam_s = lam' + sum_i Ybar_i
        for (int i = 0; i < 6; ++i) {
          t.K[i] = Yb[i];
          t.w[i] = 1.0;
        }
        t.nk = 6;
        launch_tsit5_combine(n3, lam, t, 1.0, lamNext, st);
        std::swap(lam, lamNext);
        if (s >= 1) launch_probe_adjoint_f64(dm, U, lam, b->probes, b->obs + (size_t)(s - 1) * P, P, scale, st, false);
        c->launches += 1 + (s >= 1 && P > 0 ? 1 : 0);
      }
    }
  } else if (f64) {
    launch_gather_state_f64(N, c->d_perm, c->Quser, c->QA, st);
    // Forward pass with checkpoints.  The last segment's steps write their
    // stage states straight into the segment buffer, which the reverse sweep
    // then starts from without recomputing them.
    const int sLast = seg_start(nck - 1);   // = K - C
    double* Q0s = b->seg;                          // Q0 of step s0 + i at Q0s + i n3 (i = 0..C)
    double* Q1s = b->seg + (size_t)(C + 1) * n3;   // Q1 of step s0 + i
    for (int s = 0; s < K; ++s) {
      const bool last = s >= sLast;
      const size_t i = (size_t)(s - sLast);
      if (!last && s == seg_start(seg_of(s)))
        ADJ_CUDA(c, cudaMemcpyAsync(b->ckpt + (size_t)seg_of(s) * n3, c->QA, n3 * sizeof(double),
                                    cudaMemcpyDeviceToDevice, st));
      if (s == sLast) ADJ_CUDA(c, cudaMemcpyAsync(Q0s, c->QA, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
      const double* q0 = last ? Q0s + i * n3 : c->QA;
      double* q1 = last ? Q1s + i * n3 : c->QB;
      double* q2 = last ? Q0s + (i + 1) * n3 : c->QA;
      hydro(s * dt);
      launch_inlet_total_f64(dm, ds, q0, st);
      launch_stage_f64(dm, ds, kModeStage1, q0, nullptr, q1, false, st);
      hydro((s + 1) * dt);
      launch_inlet_total_f64(dm, ds, q1, st);
      launch_stage_f64(dm, ds, kModeStage2, q1, q0, q2, false, st);
      launch_probe_loss_f64(dm, a, q2, b->probes, b->obs + (size_t)s * P, P, st);
      c->launches += 3 + extraPerStep;
    }
    ADJ_CUDA(c, cudaMemcpyAsync(c->QA, Q0s + (size_t)(K - sLast) * n3, n3 * sizeof(double),
                                cudaMemcpyDeviceToDevice, st));   // the final state
    if (Qfinal) launch_scatter_state_f64(N, c->d_perm, c->QA, c->Quser, st);   // copied out at the end
    // Reverse sweep.
    ADJ_CUDA(c, cudaMemsetAsync(b->mu2, 0, n3 * sizeof(double), st));
    launch_probe_adjoint_f64(dm, c->QA, b->mu2, b->probes, b->obs + (size_t)(K - 1) * P, P, scale, st);
    if (useFinal) {
      launch_final_loss_f64(dm, fl, c->QA, b->mu2, st);
      c->launches += 1;
    }
    for (int seg = nck - 1; seg >= 0; --seg) {
      const int s0 = seg_start(seg), s1 = seg_start(seg + 1);
      if (seg < nck - 1)   // the last segment's states are in place from the forward pass
        ADJ_CUDA(c, cudaMemcpyAsync(Q0s, b->ckpt + (size_t)seg * n3, n3 * sizeof(double), cudaMemcpyDeviceToDevice,
                                    st));
      for (int s = s0; s < s1 && seg < nck - 1; ++s) {
        const size_t i = (size_t)(s - s0);
        hydro(s * dt);
        launch_inlet_total_f64(dm, ds, Q0s + i * n3, st);
        launch_stage_f64(dm, ds, kModeStage1, Q0s + i * n3, nullptr, Q1s + i * n3, false, st);
        hydro((s + 1) * dt);
        launch_inlet_total_f64(dm, ds, Q1s + i * n3, st);
        launch_stage_f64(dm, ds, kModeStage2, Q1s + i * n3, Q0s + i * n3, Q0s + (i + 1) * n3, false, st);
        c->launches += 2 + extraPerStep;
      }
      for (int s = s1 - 1; s >= s0; --s) {
        const size_t i = (size_t)(s - s0);
        const double* q0 = Q0s + i * n3;
        const double* q1 = Q1s + i * n3;
        hydro((s + 1) * dt);
        launch_inlet_total_f64(dm, ds, q1, st);
        launch_vjp_f64(dm, a, q1, b->mu2, nullptr, b->mu1, 0.5, 0.0, 0.5 * dt, st);
        launch_inlet_adjoint_f64(dm, a, q1, b->mu1, 0.5 * dt, st);
        c->launches += launch_ude_vjp_f64(dm, a, q1, b->mu1, st);
        hydro(s * dt);
        launch_inlet_total_f64(dm, ds, q0, st);
        launch_vjp_f64(dm, a, q0, b->mu1, b->mu2, b->mu2, 1.0, 0.5, dt, st);
        launch_inlet_adjoint_f64(dm, a, q0, b->mu2, dt, st);
        c->launches += launch_ude_vjp_f64(dm, a, q0, b->mu2, st);
        if (s >= 1) launch_probe_adjoint_f64(dm, q0, b->mu2, b->probes, b->obs + (size_t)(s - 1) * P, P, scale, st);
        c->launches += 2 + 2 * extraPerStep + (s >= 1 && P > 0 ? 1 : 0);
      }
    }
  } else {
    const int n = N;
    const F32States ck = f32_view(b->ckpt, (size_t)nck, n);
    const F32States sg = f32_view(b->seg, (size_t)(2 * C + 1), n);
    float* mu1 = reinterpret_cast<float*>(b->mu1);
    float* mu2 = reinterpret_cast<float*>(b->mu2);
    const StateF32 XA{c->XA, c->XQA}, XB{c->XB, c->XQB};
    // Inlet conveyance totals of every state a VJP or a stage reads, kept
    // instead of recomputed: T0[i] of Q0s[i] (i = 0..C) and T1[i] of Q1s[i].
    // When the inlet groups fit the fused stage kernels, those kernels produce
    // the totals of their output states; otherwise k_inlet_total does.
    // (with a constant n, or an n(h, Umag, ks) function the fused stages evaluate
    // themselves -- as hg_integrate's steps do; not with a UDE closure)
    const bool fz = dm.nInlet <= kMaxFusedInlets &&
                    (dm.res.kind == kResConstant || (dm.res.kind >= kResPowerLaw && dm.res.kind <= kResHUmagKs));
    const size_t stride = (size_t)std::max(dm.nInlet, kMaxFusedInlets);
    const size_t totNeed = (size_t)(2 * C + 1) * stride;
    if (totNeed > b->segTotCap) {
      cudaFree(b->segTot);
      b->segTot = nullptr;
      ADJ_CUDA(c, cudaMalloc(&b->segTot, totNeed * sizeof(double)));
      b->segTotCap = totNeed;
    }
    double* T0 = b->segTot;
    double* T1 = b->segTot + (size_t)(C + 1) * stride;
    auto totals = [&](StateF32 q, double* t) {   // totals of q into t
      if (dm.nInlet == 0) return;
      DevMesh mm = dm;
      mm.totalA = t;
      launch_inlet_total_f32(mm, ds, q, st);
      c->launches += 1;
    };
    // One SSP-RK2 step q0 -> (q1) -> q2 at the fixed dt, with the totals t0 of q0
    // on entry and those of q1 and q2 on exit.
    auto step = [&](int s, StateF32 q0, StateF32 q1, StateF32 q2, double* t0, double* t1, double* t2) {
      if (fz) {
        StageFuse f;
        f.partials = c->d_partials;
        f.ticket = c->d_ticket;
        f.blockSlot = c->d_blockSlot;
        f.nSlots = c->nSlots;
        f.nWarps = c->nWarps;
        f.totalIn = t0;
        f.totalOut = t1;
        hydro(s * dt);
        launch_stage_f32_fused(dm, ds, kModeStage1, q0, StateF32{}, q1, f, st);
        f.totalIn = t1;
        f.totalOut = t2;
        hydro((s + 1) * dt);
        launch_stage_f32_fused(dm, ds, kModeStage2, q1, q0, q2, f, st);
        c->launches += 2;
      } else {
        DevMesh mm = dm;
        mm.totalA = t0;
        hydro(s * dt);
        launch_stage_f32(mm, ds, kModeStage1, q0, StateF32{}, q1, nullptr, false, st);
        totals(q1, t1);
        mm.totalA = t1;
        hydro((s + 1) * dt);
        launch_stage_f32(mm, ds, kModeStage2, q1, q0, q2, nullptr, false, st);
        totals(q2, t2);
        c->launches += 2;
      }
    };
    launch_gather_state_f32(N, c->d_perm, c->Quser, XA, st);
    auto copy_state = [&](StateF32 dst, StateF32 src) -> cudaError_t {
      cudaError_t e = cudaMemcpyAsync(dst.x, src.x, (size_t)n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(dst.q, src.q, (size_t)n * sizeof(float2), cudaMemcpyDeviceToDevice, st);
      return e;
    };
    // Forward pass with checkpoints (totals ping-pong in T0[0] / T0[1]).  The
    // last segment's steps write their stage states and totals straight into
    // the segment buffers, which the reverse sweep starts from.
    const int sLast = seg_start(nck - 1);   // = K - C
    totals(XA, T0);
    for (int s = 0; s < K; ++s) {
      if (s < sLast) {
        if (s == seg_start(seg_of(s))) ADJ_CUDA(c, copy_state(ck.at(seg_of(s), n), XA));
        step(s, XA, XB, XA, T0, T0 + stride, T0);
      } else {
        const size_t i = (size_t)(s - sLast);
        if (s == sLast) ADJ_CUDA(c, copy_state(sg.at(0, n), XA));   // its totals are in T0 already
        step(s, sg.at(i, n), sg.at(C + 1 + i, n), sg.at(i + 1, n), T0 + i * stride, T1 + i * stride,
             T0 + (i + 1) * stride);
      }
    }
    ADJ_CUDA(c, copy_state(XA, sg.at(K - sLast, n)));   // the final state
    if (Qfinal) launch_scatter_state_f32(N, c->d_perm, XA, c->Quser, st);   // copied out at the end
    // Boundary faces folded into the interior VJP where it can run (constant
    // inlet discharges and resistance: a segment's face Jacobians are then
    // formed in one launch before its reverse steps).
    const bool fold = vjp_fold_usable(dm, a, XA) && !a.resChain && !a.udeChain && dm.nHydro == 0;
    if (fold && (size_t)(2 * C + 1) > b->bndJCap) {
      cudaFree(b->bndJ);
      b->bndJ = nullptr;
      b->bndJCap = 0;
      ADJ_CUDA(c, cudaMalloc(&b->bndJ, (size_t)(2 * C + 1) * std::max(dm.nbf, 1) * 6 * sizeof(float4)));
      b->bndJCap = (size_t)(2 * C + 1);
    }
    const size_t jStride = (size_t)dm.nbf * 6;   // float4 per state
    const bool foldProbes = fold && P > 0;
    if (foldProbes) {
      const size_t seedNeed = (size_t)C * std::max(pc.nCells, 1);
      if (seedNeed > b->probeSeedCap) {
        cudaFree(b->probeSeeds);
        b->probeSeeds = nullptr;
        b->probeSeedCap = 0;
        ADJ_CUDA(c, cudaMalloc(&b->probeSeeds, seedNeed * sizeof(float)));
        b->probeSeedCap = seedNeed;
      }
      if ((size_t)K > b->lossPartCap) {
        cudaFree(b->lossPart);
        b->lossPart = nullptr;
        b->lossPartCap = 0;
        ADJ_CUDA(c, cudaMalloc(&b->lossPart, (size_t)K * sizeof(double)));
        b->lossPartCap = (size_t)K;
      }
    }
    ADJ_CUDA(c, cudaMemsetAsync(mu2, 0, n3 * sizeof(float), st));
    // The probe loss of each state after step s and its seed, in one kernel
    // in the reverse sweep (the state after the last step first).
    launch_probe_f32(dm, a, XA, mu2, pc, b->probes, b->obs + (size_t)(K - 1) * P, P, scale, st);
    c->launches += P > 0 ? 1 : 0;
    if (useFinal) {
      launch_final_loss_f32(dm, fl, XA, mu2, st);
      c->launches += 1;
    }
    for (int seg = nck - 1; seg >= 0; --seg) {
      const int s0 = seg_start(seg), s1 = seg_start(seg + 1);
      if (seg < nck - 1) {   // the last segment's states and totals are in place from the forward pass
        ADJ_CUDA(c, copy_state(sg.at(0, n), ck.at(seg, n)));
        totals(sg.at(0, n), T0);
        for (int s = s0; s < s1; ++s) {
          const size_t i = (size_t)(s - s0);
          step(s, sg.at(i, n), sg.at(C + 1 + i, n), sg.at(i + 1, n), T0 + i * stride, T1 + i * stride,
               T0 + (i + 1) * stride);
        }
      }
      const int sFirst = std::max(s0, 1);   // steps whose stage-1 VJP adds probe seeds
      if (fold) c->launches += launch_bnd_jac_f32(dm, a, sg.x, 2 * C + 1, b->segTot, stride, b->bndJ, st);
      if (foldProbes)
        c->launches += launch_probe_seg_f32(dm, sg.x, s0, sFirst, s1 - sFirst, pc, b->probes, b->obs, P, scale,
                                            b->probeSeeds, b->lossPart, st);
      for (int s = s1 - 1; s >= s0; --s) {
        const size_t i = (size_t)(s - s0);
        const StateF32 q0 = sg.at(i, n), q1 = sg.at(C + 1 + i, n);
        DevMesh m1 = dm, m0 = dm;
        m1.totalA = T1 + i * stride;
        m0.totalA = T0 + i * stride;
        hydro((s + 1) * dt);
        const bool resState = a.resChain || a.udeChain;
        if (resState) c->launches += launch_resistance_f32(dm, q1, st);   // n (or F) of the VJP's state
        AdjDev aj = a;   // folded: the face Jacobians of the VJP's state
        if (fold) {
          aj.bndJ = b->bndJ + (C + 1 + i) * jStride;
          c->launches += launch_vjp_f32_folded(m1, aj, q1, mu2, nullptr, mu1, 0.5f, 0.0f, 0.5 * dt, st, nullptr);
        } else {
          c->launches += launch_vjp_f32(m1, a, q1, mu2, nullptr, mu1, 0.5f, 0.0f, 0.5 * dt, st);
        }
        c->launches += launch_ude_vjp_f32(dm, a, q1, mu1, st);
        hydro(s * dt);
        if (resState) c->launches += launch_resistance_f32(dm, q0, st);
        // with the probe terms of q0, the state after step s - 1, in the same launches
        ProbeJob pj;
        if (s >= 1 && P > 0) {
          pj.pc = pc;
          pj.probes = b->probes;
          pj.obs = b->obs + (size_t)(s - 1) * P;
          pj.np = P;
          pj.scale = scale;
        }
        if (fold) {
          aj.bndJ = b->bndJ + i * jStride;
          aj.probeSeed = (foldProbes && s >= 1) ? b->probeSeeds + (size_t)(s - sFirst) * pc.nCells : nullptr;
          c->launches += launch_vjp_f32_folded(m0, aj, q0, mu1, mu2, mu2, 1.0f, 0.5f, dt, st, nullptr);
        } else {
          c->launches += launch_vjp_f32(m0, a, q0, mu1, mu2, mu2, 1.0f, 0.5f, dt, st, &pj);
        }
        c->launches += launch_ude_vjp_f32(dm, a, q0, mu2, st);
      }
    }
    if (foldProbes) c->launches += launch_loss_parts(a, b->lossPart, K - 1, st);   // states K-1 .. 1, in order
  }
  if (a.accF) {
    launch_fold_accumulators_f32(dm, a, st);
    c->launches += 1;
  }
  if (gZb) {
    launch_zb_gradient(dm, a, b->gzb, st);
    c->launches += 2;
  }
  if (a.resChain) {
    launch_res_param_sum(a, N, b->resGrad, st);
    c->launches += 1;
    ADJ_CUDA(c, cudaMemcpyAsync(c->resGrad, b->resGrad, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
  }
  if (a.udeChain && a.udeP > 0)
    ADJ_CUDA(c, cudaMemcpyAsync(c->udeGrad.data(), a.gTheta, (size_t)a.udeP * sizeof(double), cudaMemcpyDeviceToHost,
                                st));
  ADJ_CUDA(c, cudaGetLastError());
  // Results, put in the caller's cell order on the device and copied out
  // after the last kernel.
  const bool direct = useFinal && fl.wse && !fo->zbw;   // WSE_pred = h + (active zb): dL/dzb += dL/dWSE
  if (gManning) launch_scatter_field_f64(N, c->d_perm, a.gN, nullptr, b->userOut, st);
  if (gZb) launch_scatter_field_f64(N, c->d_perm, b->gzb, direct ? fl.dWse : nullptr, b->userOut + N, st);
  c->launches += (gManning ? 1 : 0) + (gZb ? 1 : 0);
  double hl = 0.0;
  ADJ_CUDA(c, cudaMemcpyAsync(&hl, a.loss, sizeof(double), cudaMemcpyDeviceToHost, st));
  if (gManning) ADJ_CUDA(c, cudaMemcpyAsync(gManning, b->userOut, N * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (gZb) ADJ_CUDA(c, cudaMemcpyAsync(gZb, b->userOut + N, N * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (gInlet && dm.nInlet > 0)
    ADJ_CUDA(c, cudaMemcpyAsync(gInlet, a.gQ, dm.nInlet * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (Qfinal) ADJ_CUDA(c, cudaMemcpyAsync(Qfinal, c->Quser, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  double fparts[2] = {0.0, 0.0};
  if (useFinal) ADJ_CUDA(c, cudaMemcpyAsync(fparts, fl.parts, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  int32_t flags = 0;
  ADJ_CUDA(c, cudaMemcpyAsync(&flags, ds.flags, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  ADJ_CUDA(c, cudaStreamSynchronize(st));
  if (flags & 2) return fail(c, HG_ERR_INLET, "inlet-Q total conveyance is not positive during the run");
  if (flags & 1) return fail(c, HG_ERR_STATE, "non-finite value in the state during the run");
  *loss = hl * scale + fparts[0] + fparts[1];
  if (parts) {
    parts[0] = fparts[0] + fparts[1];
    parts[1] = fparts[0];
    parts[2] = fparts[1];
  }
  return HG_OK;
}

void adjoint_release_tape(hg_ctx* ctx) {
  AdjointBuffers* b = ctx->adj;
  if (!b) return;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(b->seg);
  cudaFree(b->ckpt);
  b->seg = b->ckpt = nullptr;
  b->segStates = b->ckptStates = 0;
}

void adjoint_release(hg_ctx* ctx) {
  delete ctx->adj;
  ctx->adj = nullptr;
}

}  // namespace hg
