// Host side of the GB300 solid solver: device memory, once-per-mesh upload,
// the solve orchestration and the C ABI (include/s4g.h).
//
// The solve mirrors linGeomTotalDispSolid::evolve (linGeomTotalDispSolid.C:
// 111-232) and nonLinGeomTotalLagSolid::evolve (nonLinGeomTotalLagSolid.C:
// 125-260): per corrector the right-hand side, the three component PCG solves
// and the post-solve pass run on the device; the loop conditions (PCG
// convergence, converged()) are decided on the device and only read back by
// the host between launch batches.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <map>
#include <vector>

#include "kernels.cuh"
#include "s4g_internal.hpp"

namespace s4g {

thread_local std::string gLastError;

void setLastError(const std::string& msg) { gLastError = msg; }

static s4g_status setErr(s4g_status st, const std::string& msg) {
  gLastError = msg;
  return st;
}

#define S4G_CUDA(call)                                                              \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      return setErr(e_ == cudaErrorMemoryAllocation ? S4G_OOM : S4G_CUDA_ERROR,     \
                    std::string(#call) + ": " + cudaGetErrorString(e_));            \
    }                                                                               \
  } while (0)

struct Ctx {
  int device = 0;
  int verbose = 0;
  int profile = 0;
  int noGraphs = 0;
  int spinLimit = kSpinLimit;
  int numSMs = 0;
  cudaStream_t stream = nullptr;
};

// CUDA-event timer of each kernel kind on the library's stream.  Events are
// resolved after the host waits on the stream anyway (between launch batches).
struct EventTimer : LaunchTimer {
  struct Pending { int kind; int tag; cudaEvent_t a, b; };
  std::vector<cudaEvent_t> pool;
  std::vector<Pending> pending;
  cudaEvent_t open = nullptr;
  int tag = -1;  // PCG iteration index of the launches being recorded (-1: not PCG)
  double ms[S4G_K_KINDS] = {};
  long long count[S4G_K_KINDS] = {};
  ~EventTimer() {
    for (auto& p : pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : pool) cudaEventDestroy(e);
  }
  cudaEvent_t get() {
    if (pool.empty()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      return e;
    }
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  void before(int, cudaStream_t s) override {
    open = get();
    cudaEventRecord(open, s);
  }
  void after(int kind, cudaStream_t s) override {
    cudaEvent_t b = get();
    cudaEventRecord(b, s);
    pending.push_back({kind, tag, open, b});
  }
  // Launches of PCG iterations at or past keepBelow ran as no-ops (the
  // device had already stopped the loop) and are not counted.
  void resolve(int keepBelow = 1 << 30) {
    for (auto& p : pending) {
      float t = 0;
      if (p.tag < keepBelow && cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) {
        ms[p.kind] += t;
        count[p.kind] += 1;
      }
      pool.push_back(p.a);
      pool.push_back(p.b);
    }
    pending.clear();
  }
  void reset() {
    resolve();
    for (int k = 0; k < S4G_K_KINDS; ++k) { ms[k] = 0; count[k] = 0; }
  }
};

struct Engine {
  Ctx* ctx = nullptr;
  HostPrep hp;
  std::vector<void*> allocs;
  size_t bytes = 0;
  MeshView mv{};
  GeomOutputs geo{};
  // boundary condition host mirror (storage boundary order)
  int nPatches = 0;
  std::vector<int> patchStart, patchSize;
  std::vector<int> patchType;
  std::vector<double> patchRelax;  // relaxationFactor per patch
  std::vector<double> bvalH, bpressH, brelaxH;
  std::vector<int> btypeH;
  bool bcDirty = true;
  // device arrays not in MeshView
  int* dBtype = nullptr;
  double* dBval = nullptr;
  double* dBpress = nullptr;
  double* dBrelax = nullptr;
  int* dC2s = nullptr;
  double* dVal = nullptr;
  double* dDiag = nullptr;
  double* dRD = nullptr;
  double* dRDa = nullptr;
  FieldPtrs f{};
  PcgPtrs<double> pc{};    // plain FP64 inner solve
  PcgPtrs<float> pc32{};   // FP32 inner solve of the mixed-precision path
  bool fp32Allocated = false;
  bool fp32Valid = false;  // FP32 copies match the FP64 matrix/factor
  int sweepGrid32 = 1;
  // processor-local DIC path (subdomain runs with DIC)
  int nLoc = 0;
  int* dLocSrc = nullptr;
  LocalTuning tune64, tune32;   // fused-iteration variants (FP64 / FP32 inner solve)
  bool tuned64 = false, tuned32 = false;
  bool autotune = true;
  double tuneUs[2][kLocNumNT + kLocNumU] = {};  // last timings (us), for perf
  DevState* dState = nullptr;  // one per load case ([caseCap])
  DevState* hState = nullptr;  // pinned mirror
  int caseCap = 1;             // load cases the per-case arrays hold
  int nRun = 1;                // load cases of the solve in progress
  std::vector<int> pcgBase;    // per case: PCG iterations before the current loop
  double* dPartials = nullptr;
  double* dOut = nullptr;
  bool tlAllocated = false;
  // s4g_solve_step: the fields hold a finished step of model kind stepTl
  bool stepLive = false;
  int stepTl = -1;
  // material / controls
  bool materialSet = false;
  s4g_law law{};
  double mu = 0, K = 0, lambda = 0, impK = 0;
  s4g_lin_solver lin{};
  s4g_outer outer{};
  s4g_precision precision = S4G_FP64;
  bool matrixValid = false;
  int matrixPrecond = -1;
  int sweepGrid = 1;
  int lastModel = -1;
  long long launches = 0;
  EventTimer timer;
  LaunchTimer* tm() { return ctx->profile ? &timer : nullptr; }

  // CUDA graphs of the PCG launch batches: one per (value type, batch
  // length, case count), captured on first use and replayed with one launch.
  // A graph holds the kernels' arguments, so it is dropped when buffers are
  // reallocated (generation) and recaptured when the controls or the tuned
  // variants differ from the captured ones.
  struct PcgGraph {
    cudaGraphExec_t exec = nullptr;
    int generation = -1, ntIdx = -1, uIdx = -1, grid = -1;
    Controls c{};
  };
  std::map<long, PcgGraph> pcgGraphs;
  int generation = 0;
  bool graphsOk = true;
  // The device-resident corrector loop: one graph per (value type, model,
  // case count) whose conditional WHILE nodes run the correctors and, inside
  // each, the PCG iterations, with the loop decisions taken on the device.
  std::map<long, PcgGraph> loopGraphs;
  bool loopGraphsOk = true;
  bool ranOnDevice = false;  // the last solve's corrector loop ran device-resident

  void dropGraphs() {
    for (auto* m : {&pcgGraphs, &loopGraphs}) {
      for (auto& kv : *m)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
      m->clear();
    }
  }

  ~Engine() {
    dropGraphs();
    for (void* p : allocs) cudaFree(p);
    if (hState) cudaFreeHost(hState);
  }

  template <class T>
  s4g_status alloc(T** p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) return setErr(S4G_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    allocs.push_back(*p);
    bytes += n * sizeof(T);
    return S4G_OK;
  }
  template <class T>
  s4g_status upload(T** p, const std::vector<T>& h) {
    s4g_status st = alloc(p, h.size());
    if (st != S4G_OK) return st;
    if (!h.empty()) S4G_CUDA(cudaMemcpyAsync(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    return S4G_OK;
  }
#define S4G_TRY(x)                      \
  do {                                  \
    s4g_status st_ = (x);               \
    if (st_ != S4G_OK) return st_;      \
  } while (0)

  s4g_status uploadMesh(const s4g_mesh_desc* d, const s4g_mesh_opts* o) {
    std::string err;
    s4g_status st = prepareMesh(d, o, hp, err);
    if (st != S4G_OK) return setErr(st, err);
    const int nC = hp.nC, nI = hp.nI, nB = hp.nB;
    cudaStream_t s = ctx->stream;
    int *dRow, *dCol, *dFidx, *dFown, *dFnei, *dBrow, *dPartStart, *dLvlOff, *dLvlStart, *dUpPtr,
        *dUpIdx, *dDnPtr, *dDnIdx, *dS2c, *dFcaller, *dBcaller, *dBcell;
    S4G_TRY(upload(&dRow, hp.rowptr));
    S4G_TRY(upload(&dCol, hp.col));
    S4G_TRY(upload(&dFidx, hp.fidx));
    S4G_TRY(upload(&dFown, hp.fown));
    S4G_TRY(upload(&dFnei, hp.fnei));
    S4G_TRY(upload(&dBrow, hp.browptr));
    S4G_TRY(upload(&dPartStart, hp.partStart));
    S4G_TRY(upload(&dLvlOff, hp.lvlOff));
    S4G_TRY(upload(&dLvlStart, hp.lvlStart));
    S4G_TRY(upload(&dUpPtr, hp.upPtr));
    S4G_TRY(upload(&dUpIdx, hp.upIdx));
    S4G_TRY(upload(&dDnPtr, hp.dnPtr));
    S4G_TRY(upload(&dDnIdx, hp.dnIdx));
    S4G_TRY(upload(&dS2c, hp.s2c));
    S4G_TRY(upload(&dC2s, hp.c2s));
    S4G_TRY(upload(&dFcaller, hp.fcaller));
    S4G_TRY(upload(&dBcaller, hp.bcaller));
    S4G_TRY(upload(&dBcell, hp.bcell));
    char* dFflip;
    S4G_TRY(upload(&dFflip, hp.fflip));
    // caller geometry, consumed by the geometry kernels
    const int nF = d->n_faces;
    double *dCc, *dCfc, *dSfc;
    S4G_TRY(alloc(&dCc, 3 * (size_t)nC));
    S4G_TRY(alloc(&dCfc, 3 * (size_t)nF));
    S4G_TRY(alloc(&dSfc, 3 * (size_t)nF));
    S4G_CUDA(cudaMemcpyAsync(dCc, d->C, sizeof(double) * 3 * nC, cudaMemcpyHostToDevice, s));
    S4G_CUDA(cudaMemcpyAsync(dCfc, d->Cf, sizeof(double) * 3 * (size_t)nF, cudaMemcpyHostToDevice, s));
    S4G_CUDA(cudaMemcpyAsync(dSfc, d->Sf, sizeof(double) * 3 * (size_t)nF, cudaMemcpyHostToDevice, s));
    S4G_TRY(alloc(&geo.C, 3 * (size_t)nC));
    S4G_TRY(alloc(&geo.invDd, 6 * (size_t)nC));
    S4G_TRY(alloc(&geo.fS, 3 * (size_t)nI));
    S4G_TRY(alloc(&geo.fmagS, nI));
    S4G_TRY(alloc(&geo.fw, nI));
    S4G_TRY(alloc(&geo.fdelta, nI));
    S4G_TRY(alloc(&geo.bS, 3 * (size_t)nB));
    S4G_TRY(alloc(&geo.bmagS, nB));
    S4G_TRY(alloc(&geo.bn, 3 * (size_t)nB));
    S4G_TRY(alloc(&geo.bk, 3 * (size_t)nB));
    S4G_TRY(alloc(&geo.bdelta, nB));
    S4G_TRY(alloc(&geo.bls, 3 * (size_t)nB));
    S4G_TRY(alloc(&geo.lsv, 6 * (size_t)nI));
    S4G_TRY(alloc(&dBtype, nB));
    S4G_TRY(alloc(&dBval, 3 * (size_t)nB));
    S4G_TRY(alloc(&dBpress, nB));
    S4G_TRY(alloc(&dBrelax, nB));

    mv.nC = nC; mv.nI = nI; mv.nB = nB; mv.nParts = hp.nParts;
    mv.subdomains = (o && o->dic_subdomains) ? 1 : 0;
    mv.emptyDir = o ? o->empty_direction : 0;
    mv.rowGrid = std::max(1, std::min((nC + kRowBlock - 1) / kRowBlock,
                                      ctx->numSMs * kRowBlocksPerSM));
    mv.spinLimit = ctx->spinLimit;
    mv.rowptr = dRow; mv.col = dCol; mv.fidx = dFidx; mv.fown = dFown; mv.fnei = dFnei;
    mv.fS = geo.fS; mv.fmagS = geo.fmagS; mv.fw = geo.fw; mv.fdelta = geo.fdelta;
    mv.C = geo.C; mv.invDd = geo.invDd;
    mv.browptr = dBrow; mv.btype = dBtype;
    mv.bS = geo.bS; mv.bmagS = geo.bmagS; mv.bn = geo.bn; mv.bk = geo.bk;
    mv.bdelta = geo.bdelta; mv.bls = geo.bls; mv.bval = dBval; mv.bpress = dBpress;
    mv.brelax = dBrelax;
    mv.lsv = geo.lsv;
    mv.partStart = dPartStart; mv.lvlOff = dLvlOff; mv.lvlStart = dLvlStart;
    mv.upPtr = dUpPtr; mv.upIdx = dUpIdx; mv.dnPtr = dDnPtr; mv.dnIdx = dDnIdx;
    {
      int *dHfp, *dHfi, *dHbp, *dHbi, *dSlot, *dLow;
      S4G_TRY(upload(&dLow, hp.lowCnt));
      mv.lowCnt = dLow;
      S4G_TRY(upload(&dHfp, hp.haloFPtr));
      S4G_TRY(upload(&dHfi, hp.haloFIdx));
      S4G_TRY(upload(&dHbp, hp.haloBPtr));
      S4G_TRY(upload(&dHbi, hp.haloBIdx));
      S4G_TRY(upload(&dSlot, hp.slot));
      mv.haloFPtr = dHfp; mv.haloFIdx = dHfi; mv.haloBPtr = dHbp; mv.haloBIdx = dHbi;
      mv.slot = dSlot;
      mv.maxRows = hp.maxRows; mv.maxHalo = hp.maxHalo; mv.maxEntries = hp.maxEntries;
      mv.maxLevels = hp.maxLocalLevels;
    }

    GeomInputs gi{dCc, dCfc, dSfc, dS2c, dFcaller, dFflip, dBcaller, dBcell,
                  o ? o->ls_boundary_delta : 0};
    launchGeometry(mv, gi, geo, s);
    launches += 5;
    S4G_CUDA(cudaGetLastError());

    // boundary condition mirror: default traction-free on every patch
    nPatches = d->n_patches;
    patchStart.assign(d->patch_start, d->patch_start + nPatches);
    patchSize.assign(d->patch_size, d->patch_size + nPatches);
    patchType.assign(nPatches, S4G_SOLID_TRACTION);
    patchRelax.assign(nPatches, 1.0);
    bvalH.assign(3 * (size_t)nB, 0.0);
    bpressH.assign(nB, 0.0);
    brelaxH.assign(nB, 1.0);
    btypeH.assign(nB, 1);
    bcDirty = true;

    // fields and solver work arrays
    S4G_TRY(alloc(&dVal, 2 * (size_t)nI));
    S4G_TRY(alloc(&dDiag, nC));
    S4G_TRY(alloc(&dRD, nC));
    S4G_TRY(alloc(&dRDa, 2 * (size_t)nI));
    for (int k = 0; k < 2; ++k) S4G_TRY(alloc(&f.D[k], 3 * (size_t)nC));
    S4G_TRY(alloc(&f.D0, 3 * (size_t)nC));
    S4G_TRY(alloc(&f.D0b, 3 * (size_t)nB));
    S4G_TRY(alloc(&f.G, 9 * (size_t)nC));
    S4G_TRY(alloc(&f.sig, 6 * (size_t)nC));
    S4G_TRY(alloc(&f.Gb, 9 * (size_t)nB));
    S4G_TRY(alloc(&f.sigb, 6 * (size_t)nB));
    S4G_TRY(alloc(&f.g, 3 * (size_t)nB));
    S4G_TRY(alloc(&f.gPrev, 3 * (size_t)nB));
    S4G_TRY(alloc(&f.Ubr, 3 * (size_t)nB));
    S4G_TRY(alloc(&f.flux, 6 * (size_t)nI));
    S4G_TRY(alloc(&pc.x, 3 * (size_t)nC));
    S4G_TRY(alloc(&pc.r, 3 * (size_t)nC));
    S4G_TRY(alloc(&pc.w, 3 * (size_t)nC));
    S4G_TRY(alloc(&pc.p, 3 * (size_t)nC));
    S4G_TRY(alloc(&pc.q, 3 * (size_t)nC));
    S4G_TRY(alloc(&pc.flags[0], hp.nParts));
    S4G_TRY(alloc(&pc.flags[1], hp.nParts));
    pc.val = dVal; pc.diag = dDiag; pc.rD = dRD; pc.rDa = dRDa;
    S4G_TRY(alloc(&dState, 1));
    S4G_CUDA(cudaMallocHost((void**)&hState, sizeof(DevState)));
    const size_t rowBlocks = (nC + kRowBlock - 1) / kRowBlock;
    // per case: block or part records, then the preconditioner's group
    // records and group counters (zero between launches)
    mv.locGroups = (hp.nParts + 31) / 32;
    mv.locGrpOff = (long)std::max(8 * rowBlocks, 8 * (size_t)hp.nParts);
    mv.caseRec = (mv.locGrpOff + 8 * (long)mv.locGroups + (mv.locGroups + 1) / 2 + 7) / 8 * 8;
    S4G_TRY(alloc(&dPartials, (size_t)mv.caseRec));
    S4G_CUDA(cudaMemsetAsync(dPartials, 0, sizeof(double) * (size_t)mv.caseRec, s));
    S4G_TRY(alloc(&dOut, 9 * (size_t)nC));
    S4G_CUDA(cudaMemsetAsync(dState, 0, sizeof(DevState), s));

    int maxSmem = 0;
    S4G_CUDA(cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    if (sweepSmemBytes<double>(mv) + 1024 > (size_t)maxSmem)
      return setErr(S4G_BAD_ARG, "a DIC scheduling part does not fit in shared memory; use a smaller part_size");
    int perSM = 0;
    S4G_CUDA(sweepPrepare<double>(mv, &perSM));
    if (perSM < 1) return setErr(S4G_BAD_ARG, "DIC sweep kernel cannot be resident; use a smaller part_size");
    sweepGrid = std::max(1, std::min(hp.nParts, perSM * ctx->numSMs));
    S4G_CUDA(sweepPrepare<float>(mv, &perSM));
    sweepGrid32 = std::max(1, std::min(hp.nParts, std::max(1, perSM) * ctx->numSMs));
    if (mv.subdomains) {
      nLoc = (int)hp.locSrc.size();
      int *dEs, *dMs;
      uint16_t* dIdx;
      uint32_t* dMeta;
      S4G_TRY(upload(&dLocSrc, hp.locSrc));
      S4G_TRY(upload(&dEs, hp.locEntStart));
      S4G_TRY(upload(&dMs, hp.locMetaStart));
      S4G_TRY(upload(&dIdx, hp.locIdx));
      S4G_TRY(upload(&dMeta, hp.locMeta));
      mv.locSrc = dLocSrc; mv.locEntStart = dEs; mv.locMetaStart = dMs;
      mv.locIdx = dIdx; mv.locMeta = dMeta;
      int* dDesc;
      S4G_TRY(upload(&dDesc, hp.locDesc));
      mv.locDesc = reinterpret_cast<const int4*>(dDesc);
      mv.maxLocEntries = hp.maxLocEntries; mv.maxLocMeta = hp.maxLocMeta;
      mv.locSlots = hp.locSlots ? 1 : 0;
      if (localSmemBytes<double>(mv) + 2048 > (size_t)maxSmem)
        return setErr(S4G_BAD_ARG, "a DIC part does not fit in shared memory; use a smaller part_size");
      int per[kLocNumNT];
      // slot tables: the second variant is the first on the smallest grid
      // that gives every CTA the same number of parts
      auto grids = [&](LocalTuning& t, const int* per) {
        for (int k = 0; k < kLocNumNT; ++k)
          t.grid[k] = std::max(1, std::min(hp.nParts, std::max(1, per[k]) * ctx->numSMs));
        if (mv.locSlots) {
          const int waves = (hp.nParts + t.grid[0] - 1) / t.grid[0];
          t.grid[1] = (hp.nParts + waves - 1) / waves;
        }
      };
      S4G_CUDA(localPrepare<double>(mv, per));
      grids(tune64, per);
      S4G_CUDA(localPrepare<float>(mv, per));
      grids(tune32, per);
      autotune = !(o && o->no_autotune);
      S4G_TRY(alloc(&pc.p2, 3 * (size_t)nC));
      double* lc;
      S4G_TRY(alloc(&lc, (size_t)nLoc));
      pc.lcoef = lc;
    }
    S4G_CUDA(cudaStreamSynchronize(s));
    // caller geometry is no longer needed
    for (double* p : {dCc, dCfc, dSfc}) {
      cudaFree(p);
      allocs.erase(std::find(allocs.begin(), allocs.end(), (void*)p));
    }
    bytes -= sizeof(double) * 3 * ((size_t)nC + 2 * (size_t)nF);
    return S4G_OK;
  }

  s4g_status allocTL() {
    if (tlAllocated) return S4G_OK;
    const size_t nC = hp.nC, nB = hp.nB;
    S4G_TRY(alloc(&f.GD, 9 * nC)); S4G_TRY(alloc(&f.GD0, 9 * nC));
    S4G_TRY(alloc(&f.GDb, 9 * nB)); S4G_TRY(alloc(&f.GD0b, 9 * nB));
    S4G_TRY(alloc(&f.Finv, 9 * nC)); S4G_TRY(alloc(&f.Finvb, 9 * nB));
    S4G_TRY(alloc(&f.J, nC)); S4G_TRY(alloc(&f.Jb, nB));
    S4G_TRY(alloc(&f.FL, 9 * nC)); S4G_TRY(alloc(&f.FL0, 9 * nC));
    S4G_TRY(alloc(&f.FLb, 9 * nB)); S4G_TRY(alloc(&f.FL0b, 9 * nB));
    S4G_TRY(alloc(&f.sig0, 6 * nC)); S4G_TRY(alloc(&f.sig0b, 6 * nB));
    tlAllocated = true;
    return S4G_OK;
  }

  // Aitken relaxation: a factor and a residual per cell and boundary face
  // and load case, allocated when a solve first selects it.  Their values
  // before an increment's first corrector are never read.
  s4g_status ensureAitken() {
    if (outer.relaxation_method != 1 || f.aitA) return S4G_OK;
    const size_t nCB = (size_t)hp.nC + hp.nB;
    S4G_TRY(alloc(&f.aitA, nCB * caseCap));
    S4G_TRY(alloc(&f.aitR, 3 * nCB * caseCap));
    ++generation;  // captured graphs hold the field pointers
    dropGraphs();
    return S4G_OK;
  }

  s4g_status setMaterial(const s4g_law* l) {
    if (!l || (l->type != S4G_LINEAR_ELASTIC && l->type != S4G_NEO_HOOKEAN))
      return setErr(S4G_BAD_ARG, "unknown law");
    double E = l->E, nu = l->nu;
    if (l->use_mu_K) {
      if (!(l->mu > 0) || !(l->K > 0)) return setErr(S4G_BAD_ARG, "mu and K must be positive");
      mu = l->mu; K = l->K;
      E = 9.0 * K * mu / (3.0 * K + mu);
      nu = (3.0 * K - 2.0 * mu) / (2.0 * (3.0 * K + mu));
    } else {
      // linearElastic.C:126-133: nu must lie in [-1, 0.5]
      if (!(E > 0) || !(nu >= -1.0 && nu < 0.5)) return setErr(S4G_BAD_ARG, "need E > 0 and -1 <= nu < 0.5");
      mu = E / (2.0 * (1.0 + nu));
      K = (nu * E / ((1.0 + nu) * (1.0 - 2.0 * nu))) + (2.0 / 3.0) * mu;
    }
    lambda = nu * E / ((1.0 + nu) * (1.0 - 2.0 * nu));
    if (l->type == S4G_LINEAR_ELASTIC) {
      K = E / (3.0 * (1.0 - 2.0 * nu));  // linearElastic.C:118-123
      impK = 2.0 * mu + lambda;          // linearElastic.C:204-245
    } else {
      impK = (4.0 / 3.0) * mu + K;       // neoHookeanElastic.C:101-119
    }
    law = *l;
    materialSet = true;
    matrixValid = false;
    return S4G_OK;
  }

  s4g_status setBC(int patch, s4g_bc_type type, const double* vec3, const double* pressure) {
    if (patch < 0 || patch >= nPatches) return setErr(S4G_BAD_ARG, "patch index out of range");
    if (type != S4G_FIXED_DISPLACEMENT && type != S4G_SOLID_TRACTION) return setErr(S4G_BAD_ARG, "unknown BC type");
    const int nI = hp.nI;
    const int ps = patchStart[patch], sz = patchSize[patch];
    for (int i = 0; i < sz; ++i) {
      if (vec3) for (int k = 0; k < 3; ++k) if (!std::isfinite(vec3[3 * i + k])) return setErr(S4G_BAD_ARG, "non-finite BC value");
      if (pressure && !std::isfinite(pressure[i])) return setErr(S4G_BAD_ARG, "non-finite pressure");
    }
    if (patchType[patch] != type) matrixValid = false;
    patchType[patch] = type;
    // storage positions of this patch's faces
    for (int k = 0; k < hp.nB; ++k) {
      int b = hp.bcaller[k];
      int i = b + nI - ps;
      if (i < 0 || i >= sz) continue;
      btypeH[k] = (int)type;
      for (int j = 0; j < 3; ++j) bvalH[3 * (size_t)k + j] = vec3 ? vec3[3 * i + j] : 0.0;
      bpressH[k] = (type == S4G_SOLID_TRACTION && pressure) ? pressure[i] : 0.0;
      brelaxH[k] = type == S4G_SOLID_TRACTION ? patchRelax[patch] : 1.0;
    }
    bcDirty = true;
    return S4G_OK;
  }

  s4g_status setRelaxation(int patch, double factor) {
    if (patch < 0 || patch >= nPatches) return setErr(S4G_BAD_ARG, "patch index out of range");
    if (!(factor > 0.0 && factor <= 1.0)) return setErr(S4G_BAD_ARG, "relaxation factor must be in (0, 1]");
    patchRelax[patch] = factor;
    const int nI = hp.nI;
    const int ps = patchStart[patch], sz = patchSize[patch];
    for (int k = 0; k < hp.nB; ++k) {
      const int i = hp.bcaller[k] + nI - ps;
      if (i < 0 || i >= sz) continue;
      brelaxH[k] = btypeH[k] == S4G_SOLID_TRACTION ? factor : 1.0;
    }
    bcDirty = true;
    return S4G_OK;
  }

  s4g_status syncBC() {
    if (!bcDirty) return S4G_OK;
    cudaStream_t s = ctx->stream;
    S4G_CUDA(cudaMemcpyAsync(dBtype, btypeH.data(), sizeof(int) * hp.nB, cudaMemcpyHostToDevice, s));
    S4G_CUDA(cudaMemcpyAsync(dBval, bvalH.data(), sizeof(double) * 3 * hp.nB, cudaMemcpyHostToDevice, s));
    S4G_CUDA(cudaMemcpyAsync(dBpress, bpressH.data(), sizeof(double) * hp.nB, cudaMemcpyHostToDevice, s));
    S4G_CUDA(cudaMemcpyAsync(dBrelax, brelaxH.data(), sizeof(double) * hp.nB, cudaMemcpyHostToDevice, s));
    bcDirty = false;
    return S4G_OK;
  }

  Controls controls(int tl) const {
    Controls c{};
    c.law = law.type == S4G_NEO_HOOKEAN ? 1 : 0;
    c.tl = tl;
    c.mu = mu; c.K = K; c.lambda = lambda; c.impK = impK; c.rImpK = 1.0 / impK;
    c.gamma = impK;
    c.gammaS = outer.stab_scale * impK;
    c.loadFactor = 1.0;
    c.tol = lin.tolerance; c.relTol = lin.rel_tol; c.maxIter = lin.max_iter;
    c.nCorr = outer.n_correctors;
    c.solTol = outer.solution_tol; c.altTol = outer.alternative_tol; c.matTol = outer.material_tol;
    c.precond = lin.preconditioner == S4G_PRECOND_DIC ? 0 : 1;
    // relaxationFactors { fields { D f; } }: 0 or 1 leave the field as solved
    const double fr = outer.field_relaxation;
    c.fieldRelax = (fr > 0.0 && fr < 1.0) ? fr : 1.0;
    c.aitken = outer.relaxation_method == 1 ? 1 : 0;
    c.aitkenA0 = c.fieldRelax;
    if (c.aitken) c.fieldRelax = 1.0;
    return c;
  }

  s4g_status resetSweepState() {
    cudaStream_t s = ctx->stream;
    S4G_CUDA(cudaMemsetAsync(pc.flags[0], 0, sizeof(unsigned) * hp.nParts, s));
    S4G_CUDA(cudaMemsetAsync(pc.flags[1], 0, sizeof(unsigned) * hp.nParts, s));
    S4G_CUDA(cudaMemsetAsync(dState, 0, sizeof(DevState) * nRun, s));
    std::memset(hState, 0, sizeof(DevState) * nRun);  // the host mirror starts alike
    DevState init{};
    init.epoch[0] = 1; init.epoch[1] = 1;
    for (int cs = 0; cs < nRun; ++cs)
      S4G_CUDA(cudaMemcpyAsync(&dState[cs].epoch, &init.epoch, sizeof(init.epoch), cudaMemcpyHostToDevice, s));
    return S4G_OK;
  }

  // Every case of the solve starts its corrector loop.
  s4g_status setLive() {
    static const int one = 1;
    for (int cs = 0; cs < nRun; ++cs)
      S4G_CUDA(cudaMemcpyAsync(&dState[cs].caseLive, &one, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    return S4G_OK;
  }

  // Matrix and preconditioner (constant across correctors: impKf is fixed at
  // construction, linGeomTotalDispSolid.C:72, and the mesh is static).
  s4g_status ensureMatrix() {
    if (!materialSet) return setErr(S4G_BAD_ARG, "material not set");
    S4G_TRY(syncBC());
    const int pre = lin.preconditioner == S4G_PRECOND_DIC ? 0 : 1;
    if (matrixValid && matrixPrecond == pre) return S4G_OK;
    cudaStream_t s = ctx->stream;
    launchMatrix(mv, impK, dVal, dDiag, s);
    launches++;
    if (pre == 0) {
      S4G_TRY(resetSweepState());
      S4G_CUDA(cudaMemcpyAsync(dRD, dDiag, sizeof(double) * hp.nC, cudaMemcpyDeviceToDevice, s));
      launchDicFactor(mv, dVal, dDiag, dRD, dRDa, pc.flags[0], dState, sweepGrid, s);
      launches += 2;
      if (mv.subdomains) {
        launchLocalGather<double>(nLoc, dLocSrc, dRDa, const_cast<double*>(pc.lcoef), s);
        launches++;
      }
    } else {
      launchReciprocal(hp.nC, dDiag, dRD, s);  // diagonalPreconditioner: rD = 1/diag
      launches++;
    }
    S4G_CUDA(cudaGetLastError());
    S4G_CUDA(cudaStreamSynchronize(s));
    S4G_TRY(readState());
    if (hState->status & kErrTimeout) return setErr(S4G_TIMEOUT, "DIC factor sweep wait gave up");
    matrixValid = true;
    matrixPrecond = pre;
    fp32Valid = false;
    return S4G_OK;
  }

  // FP32 copies of the matrix, factor and work vectors (mixed precision).
  s4g_status ensureFp32() {
    const size_t nC = hp.nC, nE = 2 * (size_t)hp.nI;
    if (!fp32Allocated) {
      float *val, *diag, *rD, *rDa;
      S4G_TRY(alloc(&val, nE)); S4G_TRY(alloc(&diag, nC)); S4G_TRY(alloc(&rD, nC)); S4G_TRY(alloc(&rDa, nE));
      pc32.val = val; pc32.diag = diag; pc32.rD = rD; pc32.rDa = rDa;
      const size_t nv = 3 * nC * (size_t)caseCap;  // one vector per load case
      S4G_TRY(alloc(&pc32.x, nv)); S4G_TRY(alloc(&pc32.r, nv)); S4G_TRY(alloc(&pc32.w, nv));
      S4G_TRY(alloc(&pc32.p, nv)); S4G_TRY(alloc(&pc32.q, nv));
      pc32.flags[0] = pc.flags[0]; pc32.flags[1] = pc.flags[1];
      ++generation;
      if (mv.subdomains) {
        float* lc;
        S4G_TRY(alloc(&pc32.p2, 3 * nC * (size_t)caseCap));
        S4G_TRY(alloc(&lc, (size_t)nLoc));
        pc32.lcoef = lc;
      }
      fp32Allocated = true;
    }
    if (!fp32Valid) {
      cudaStream_t s = ctx->stream;
      launchToFloat(nE, dVal, const_cast<float*>(pc32.val), s);
      launchToFloat(nC, dDiag, const_cast<float*>(pc32.diag), s);
      launchToFloat(nC, dRD, const_cast<float*>(pc32.rD), s);
      launchToFloat(nE, dRDa, const_cast<float*>(pc32.rDa), s);
      launches += 4;
      if (mv.subdomains) {
        launchLocalGather<float>(nLoc, dLocSrc, dRDa, const_cast<float*>(pc32.lcoef), s);
        launches++;
      }
      S4G_CUDA(cudaGetLastError());
      fp32Valid = true;
    }
    return S4G_OK;
  }

  // Reads the device state of the nRun cases.  In a PCG loop (inPcg), the
  // profiler drops the launches past the last iteration any case ran.
  s4g_status readState(bool inPcg = false) {
    S4G_CUDA(cudaMemcpyAsync(hState, dState, sizeof(DevState) * nRun, cudaMemcpyDeviceToHost, ctx->stream));
    S4G_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->profile) {
      int keep = 1 << 30;
      if (inPcg) {
        keep = 0;
        for (int cs = 0; cs < nRun; ++cs) keep = std::max(keep, hState[cs].pcgIter - pcgBase[cs]);
      }
      timer.resolve(keep);
    }
    return S4G_OK;
  }
  bool anyCase(int DevState::*flag) const {
    for (int cs = 0; cs < nRun; ++cs)
      if (hState[cs].*flag) return true;
    return false;
  }

  s4g_status initFields(int tl) {
    cudaStream_t s = ctx->stream;
    stepLive = false;
    // per-case arrays of the nRun cases of this solve
    const size_t nC = hp.nC * (size_t)nRun, nB = hp.nB * (size_t)nRun;
    auto z = [&](double* p, size_t n) { return cudaMemsetAsync(p, 0, n * sizeof(double), s); };
    S4G_CUDA(z(f.D[0], 3 * nC)); S4G_CUDA(z(f.D[1], 3 * nC)); S4G_CUDA(z(f.D0, 3 * nC));
    S4G_CUDA(z(f.D0b, 3 * nB)); S4G_CUDA(z(f.G, 9 * nC)); S4G_CUDA(z(f.sig, 6 * nC));
    S4G_CUDA(z(f.Gb, 9 * nB)); S4G_CUDA(z(f.sigb, 6 * nB)); S4G_CUDA(z(f.g, 3 * nB));
    S4G_CUDA(z(f.Ubr, 3 * nB)); S4G_CUDA(z(f.gPrev, 3 * nB));
    S4G_CUDA(z(pc.x, 3 * nC)); S4G_CUDA(z(pc.r, 3 * nC)); S4G_CUDA(z(pc.w, 3 * nC));
    S4G_CUDA(z(pc.p, 3 * nC)); S4G_CUDA(z(pc.q, 3 * nC));
    if (fp32Allocated)
      for (float* p : {pc32.x, pc32.r, pc32.w, pc32.p, pc32.q})
        S4G_CUDA(cudaMemsetAsync(p, 0, 3 * nC * sizeof(float), s));
    if (tl) {
      S4G_CUDA(z(f.GD, 9 * nC)); S4G_CUDA(z(f.GD0, 9 * nC)); S4G_CUDA(z(f.GDb, 9 * nB));
      S4G_CUDA(z(f.GD0b, 9 * nB)); S4G_CUDA(z(f.sig0, 6 * nC)); S4G_CUDA(z(f.sig0b, 6 * nB));
      // F = I, F^-1 = I, J = 1 (nonLinGeomTotalLagSolid.C:57-93)
      std::vector<double> I9(9 * std::max(nC, nB), 0.0), one(std::max(nC, nB), 1.0);
      for (size_t i = 0; i < std::max(nC, nB); ++i) { I9[9 * i] = 1; I9[9 * i + 4] = 1; I9[9 * i + 8] = 1; }
      for (double* p : {f.Finv, f.FL, f.FL0}) S4G_CUDA(cudaMemcpyAsync(p, I9.data(), 9 * nC * sizeof(double), cudaMemcpyHostToDevice, s));
      for (double* p : {f.Finvb, f.FLb, f.FL0b}) S4G_CUDA(cudaMemcpyAsync(p, I9.data(), 9 * nB * sizeof(double), cudaMemcpyHostToDevice, s));
      S4G_CUDA(cudaMemcpyAsync(f.J, one.data(), nC * sizeof(double), cudaMemcpyHostToDevice, s));
      S4G_CUDA(cudaMemcpyAsync(f.Jb, one.data(), nB * sizeof(double), cudaMemcpyHostToDevice, s));
      S4G_CUDA(cudaStreamSynchronize(s));
    }
    return S4G_OK;
  }

  template <class T>
  s4g_status regrow(T*& ptr, size_t nOld, size_t nNew) {
    if (ptr) {
      cudaFree(ptr);
      allocs.erase(std::find(allocs.begin(), allocs.end(), (void*)ptr));
      bytes -= nOld * sizeof(T);
    }
    ptr = nullptr;
    return alloc(&ptr, nNew);
  }

  // Per-case arrays for C load cases: fields, boundary values, PCG vectors,
  // device states and reduction records.  Contents are not kept.
  s4g_status ensureCases(int C) {
    if (C <= caseCap) return S4G_OK;
    S4G_CUDA(cudaStreamSynchronize(ctx->stream));
    const size_t nC = hp.nC, nB = hp.nB, nI = hp.nI, o = caseCap, n = C;
    for (int k = 0; k < 2; ++k) S4G_TRY(regrow(f.D[k], 3 * nC * o, 3 * nC * n));
    S4G_TRY(regrow(f.D0, 3 * nC * o, 3 * nC * n));
    S4G_TRY(regrow(f.D0b, 3 * nB * o, 3 * nB * n));
    S4G_TRY(regrow(f.G, 9 * nC * o, 9 * nC * n));
    S4G_TRY(regrow(f.sig, 6 * nC * o, 6 * nC * n));
    S4G_TRY(regrow(f.Gb, 9 * nB * o, 9 * nB * n));
    S4G_TRY(regrow(f.sigb, 6 * nB * o, 6 * nB * n));
    S4G_TRY(regrow(f.g, 3 * nB * o, 3 * nB * n));
    S4G_TRY(regrow(f.Ubr, 3 * nB * o, 3 * nB * n));
    S4G_TRY(regrow(f.gPrev, 3 * nB * o, 3 * nB * n));
    if (f.aitA) {
      S4G_TRY(regrow(f.aitA, (nC + nB) * o, (nC + nB) * n));
      S4G_TRY(regrow(f.aitR, 3 * (nC + nB) * o, 3 * (nC + nB) * n));
    }
    S4G_TRY(regrow(f.flux, 6 * nI * o, 6 * nI * n));
    S4G_TRY(regrow(dBval, 3 * nB * o, 3 * nB * n));
    S4G_TRY(regrow(dBpress, nB * o, nB * n));
    mv.bval = dBval; mv.bpress = dBpress;
    bcDirty = true;
    for (double** v : {&pc.x, &pc.r, &pc.w, &pc.p, &pc.q}) S4G_TRY(regrow(*v, 3 * nC * o, 3 * nC * n));
    if (pc.p2) S4G_TRY(regrow(pc.p2, 3 * nC * o, 3 * nC * n));
    if (fp32Allocated) {
      for (float** v : {&pc32.x, &pc32.r, &pc32.w, &pc32.p, &pc32.q}) S4G_TRY(regrow(*v, 3 * nC * o, 3 * nC * n));
      if (pc32.p2) S4G_TRY(regrow(pc32.p2, 3 * nC * o, 3 * nC * n));
    }
    S4G_TRY(regrow(dState, o, n));
    S4G_TRY(regrow(dPartials, (size_t)mv.caseRec * o, (size_t)mv.caseRec * n));
    S4G_CUDA(cudaMemsetAsync(dPartials, 0, sizeof(double) * (size_t)mv.caseRec * n, ctx->stream));
    cudaFreeHost(hState);
    hState = nullptr;
    S4G_CUDA(cudaMallocHost((void**)&hState, sizeof(DevState) * n));
    std::memset(hState, 0, sizeof(DevState) * n);
    caseCap = C;
    stepLive = false;
    ++generation;  // captured graphs refer to the old buffers
    dropGraphs();
    return S4G_OK;
  }

  // Batched load cases of the linear-geometry model on this mesh: C
  // independent corrector loops (each case its own convergence, PCG state
  // and boundary values) advanced together, every kernel launched once for
  // all live cases (blockIdx.y = case).  Each case computes exactly what a
  // single solve with its boundary values computes.
  s4g_status solveCases(int C, const double* bval, const double* bpress, double* Dout,
                        double* sigOut, s4g_perf* perfs) {
    if (C < 1) return setErr(S4G_BAD_ARG, "n_cases must be >= 1");
    if (!bval) return setErr(S4G_BAD_ARG, "bval is required");
    if (!materialSet) return setErr(S4G_BAD_ARG, "material not set");
    if (law.type != S4G_LINEAR_ELASTIC) return setErr(S4G_BAD_ARG, "batched load cases need a linearElastic law");
    if (!(mv.subdomains && lin.preconditioner == S4G_PRECOND_DIC))
      return setErr(S4G_BAD_ARG, "batched load cases run the processor-local DIC: upload the mesh with dic_subdomains=1 and use the DIC preconditioner");
    const size_t nB = hp.nB, nC = hp.nC;
    for (size_t i = 0; i < 3 * nB * C; ++i)
      if (!std::isfinite(bval[i])) return setErr(S4G_BAD_ARG, "non-finite boundary value");
    if (bpress)
      for (size_t i = 0; i < nB * C; ++i)
        if (!std::isfinite(bpress[i])) return setErr(S4G_BAD_ARG, "non-finite pressure");
    cudaStream_t s = ctx->stream;
    const long long launches0 = launches;
    S4G_TRY(ensureCases(C));
    S4G_TRY(ensureAitken());
    S4G_TRY(ensureMatrix());
    const bool mixed = precision == S4G_FP32_REFINE;
    if (mixed) S4G_TRY(ensureFp32());
    {
      const Controls ct = controls(0);
      if (mixed) S4G_TRY(tuneLocal<float>(ct, pc32));
      else S4G_TRY(tuneLocal<double>(ct, pc));
    }
    // the cases' boundary values in storage order (types are the mesh's)
    std::vector<double> hv(3 * nB * C), hpr(nB * C);
    for (int cs = 0; cs < C; ++cs)
      for (size_t k = 0; k < nB; ++k) {
        const size_t b = (size_t)hp.bcaller[k];
        for (int j = 0; j < 3; ++j) hv[3 * (cs * nB + k) + j] = bval[3 * (cs * nB + b) + j];
        hpr[cs * nB + k] = (btypeH[k] == S4G_SOLID_TRACTION && bpress) ? bpress[cs * nB + b] : 0.0;
      }
    S4G_CUDA(cudaMemcpyAsync(dBval, hv.data(), sizeof(double) * hv.size(), cudaMemcpyHostToDevice, s));
    S4G_CUDA(cudaMemcpyAsync(dBpress, hpr.data(), sizeof(double) * hpr.size(), cudaMemcpyHostToDevice, s));
    bcDirty = true;  // a later single solve uploads the mesh's own values again
    cudaEvent_t e0, e1;
    S4G_CUDA(cudaEventCreate(&e0));
    S4G_CUDA(cudaEventCreate(&e1));
    nRun = C;
    ranOnDevice = false;
    S4G_TRY(initFields(0));
    S4G_TRY(resetSweepState());
    S4G_TRY(setLive());
    timer.reset();
    S4G_CUDA(cudaEventRecord(e0, s));
    Controls c = controls(0);
    launchTractionInit(mv, c, f, s, C);
    launchPost<double>(mv, c, f, pc.x, dState, dPartials, 0, s, nullptr, C);
    launches += 2;
    s4g_status st = mixed ? correctorLoop<float>(c, 0, pc32, sweepGrid32)
                          : correctorLoop<double>(c, 0, pc, sweepGrid);
    if (st != S4G_OK) { nRun = 1; return st; }
    S4G_CUDA(cudaEventRecord(e1, s));
    S4G_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    S4G_TRY(readState());
    auto t0 = std::chrono::steady_clock::now();
    for (int cs = 0; cs < C; ++cs) {
      const FieldPtrs fc = caseFields(f, cs, hp.nC, hp.nB, hp.nI);
      if (Dout) {
        launchGather(hp.nC, 3, dC2s, fc.D[hState[cs].dcur], dOut, s);
        S4G_CUDA(cudaMemcpyAsync(Dout + 3 * nC * cs, dOut, sizeof(double) * 3 * nC, cudaMemcpyDeviceToHost, s));
      }
      if (sigOut) {
        launchGather(hp.nC, 6, dC2s, fc.sig, dOut + 3 * nC, s);
        S4G_CUDA(cudaMemcpyAsync(sigOut + 6 * nC * cs, dOut + 3 * nC, sizeof(double) * 6 * nC, cudaMemcpyDeviceToHost, s));
      }
      S4G_CUDA(cudaStreamSynchronize(s));  // dOut is reused by the next case
    }
    auto t1 = std::chrono::steady_clock::now();
    lastModel = S4G_LIN_GEOM_TOTAL_DISP;
    s4g_status ret = S4G_OK;
    timer.resolve();
    for (int cs = 0; cs < C; ++cs) {
      const DevState& h = hState[cs];
      if (perfs) {
        s4g_perf* perf = perfs + cs;
        std::memset(perf, 0, sizeof(*perf));
        perf->n_correctors = h.nCorrDone;
        perf->converged = h.converged;
        perf->total_lin_iters = h.totalLinIters;
        perf->last_max_lin_iters = h.lastMaxIters;
        perf->initial_residual = h.initResMag;
        perf->rel_residual = h.relRes;
        perf->solve_ms = ms;
        perf->d2h_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        perf->kernel_launches = launches - launches0;
        perf->device_status = (int)h.status;
        const LocalTuning& lt = mixed ? tune32 : tune64;
        perf->part_threads = localPartThreads(mv, lt.ntIdx);
        perf->spmv_unroll = kLocVariantsU[lt.uIdx];
        for (int k = 0; k < 6; ++k)
          perf->tune_us[k] = k < kLocNumNT + kLocNumU ? tuneUs[mixed ? 1 : 0][k] : 0.0;
        for (int k = 0; k < S4G_K_KINDS; ++k) {
          perf->kernel_ms[k] = timer.ms[k];
          perf->kernel_launches_by[k] = timer.count[k];
        }
        perf->device_loop = ranOnDevice ? 1 : 0;
      }
      if (h.status & kErrNaN) ret = setErr(S4G_NAN_DETECTED, "non-finite value in a load case");
      else if (h.status & kErrIndefinite && ret == S4G_OK) ret = setErr(S4G_INDEFINITE, "PCG met p.Ap <= 0 in a load case");
      else if (!h.converged && ret == S4G_OK) ret = S4G_NOT_CONVERGED;
    }
    nRun = 1;
    return ret;
  }

  // PCG loop of one corrector: launch batches, read the device decision.
  template <typename T>
  LocalTuning& tuning() { return sizeof(T) == 4 ? tune32 : tune64; }

  // Autotuner of the fused processor-local iteration: times every variant of
  // its two kernels on this mesh and keeps the fastest.  Each timed launch
  // starts from the same state (a scratch DevState reset before it, all
  // components active, one pending update) on zeroed vectors, so every
  // launch does the full work.  The vectors are reset by the corrector's
  // right-hand side pass afterwards.  Variants give bit-identical results, so
  // the choice changes only the speed.
  template <typename T>
  s4g_status tuneLocal(const Controls& c, const PcgPtrs<T>& p) {
    bool& done = sizeof(T) == 4 ? tuned32 : tuned64;
    if (done || !autotune) { done = true; return S4G_OK; }
    cudaStream_t s = ctx->stream;
    const size_t n3 = 3 * (size_t)hp.nC;
    T* vecs[6] = {p.x, p.r, p.w, p.p, p.q, p.p2};
    for (T* v : vecs) S4G_CUDA(cudaMemsetAsync(v, 0, n3 * sizeof(T), s));
    DevState* dTune = nullptr;
    S4G_TRY(alloc(&dTune, 1));
    DevState init{};
    init.pcgContinue = 1;
    for (int k = 0; k < 3; ++k) {
      init.active[k] = 1; init.pending[k] = 1; init.nIter[k] = 1;
      init.normFactor[k] = 1; init.initRes[k] = 1; init.wArA[k] = 1; init.beta[k] = 0.5;
    }
    cudaEvent_t a, b;
    S4G_CUDA(cudaEventCreate(&a));
    S4G_CUDA(cudaEventCreate(&b));
    LocalTuning& t = tuning<T>();
    double* us = tuneUs[sizeof(T) == 4 ? 1 : 0];
    auto timeIt = [&](auto launch) -> double {
      float best = 1e30f;
      for (int rep = 0; rep < 7; ++rep) {
        cudaMemcpyAsync(dTune, &init, sizeof(DevState), cudaMemcpyHostToDevice, s);
        cudaEventRecord(a, s);
        launch();
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (rep >= 2) best = std::min(best, ms);
      }
      return 1000.0 * best;
    };
    LocalTuning cand = t;
    int bestNT = 0;
    for (int k = 0; k < kLocNumNT; ++k) {
      cand.ntIdx = k;
      us[k] = timeIt([&] { launchLocalPrecond<T>(mv, c, p, dTune, dPartials, cand, s); });
      launches += 7;
      if (us[k] < us[bestNT]) bestNT = k;
    }
    int bestU = 0;
    for (int k = 0; k < kLocNumU; ++k) {
      cand.uIdx = k;
      us[kLocNumNT + k] = timeIt([&] { launchLocalSpmv<T>(mv, p, dTune, dPartials, cand, s); });
      launches += 7 * (kLocVariantsU[k] == 0 ? 2 : 1);
      if (us[kLocNumNT + k] < us[kLocNumNT + bestU]) bestU = k;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    S4G_CUDA(cudaGetLastError());
    S4G_CUDA(cudaStreamSynchronize(s));
    allocs.erase(std::find(allocs.begin(), allocs.end(), (void*)dTune));
    cudaFree(dTune);
    bytes -= sizeof(DevState);
    t.ntIdx = bestNT;
    t.uIdx = bestU;
    done = true;
    return S4G_OK;
  }

  // The graph of a batch of n PCG iterations for the current state of the
  // engine (captured on first use); nullptr if capture is not possible, in
  // which case the caller launches directly.
  template <typename T, typename F>
  cudaGraphExec_t pcgGraph(const Controls& c, const PcgPtrs<T>& p, int grid, int n, F& launchBatch) {
    const long key = ((long)(sizeof(T)) << 40) | ((long)nRun << 8) | (long)n;
    PcgGraph& g = pcgGraphs[key];
    const LocalTuning& t = tuning<T>();
    if (g.exec && g.generation == generation && g.ntIdx == t.ntIdx && g.uIdx == t.uIdx &&
        g.grid == grid && std::memcmp(&g.c, &c, sizeof(Controls)) == 0)
      return g.exec;
    if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      graphsOk = false;
      cudaGetLastError();
      return nullptr;
    }
    long long dummy = 0;
    launchBatch(n, &dummy);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g.exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      graphsOk = false;
      g.exec = nullptr;
      cudaGetLastError();
      return nullptr;
    }
    g.generation = generation; g.ntIdx = t.ntIdx; g.uIdx = t.uIdx; g.grid = grid; g.c = c;
    (void)p;
    return g.exec;
  }

  // Adds a conditional WHILE node on h after the work captured so far on s;
  // work captured later depends on it.  body: the node's body graph.
  bool addWhile(cudaStream_t s, cudaGraphConditionalHandle h, cudaGraph_t* body) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &nd) != cudaSuccess ||
        cs != cudaStreamCaptureStatusActive)
      return false;
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, cg, deps, nullptr, nd, &np) != cudaSuccess) return false;
    *body = np.conditional.phGraph_out[0];
    return cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                               cudaStreamSetCaptureDependencies) == cudaSuccess;
  }

  // Builds the device-resident corrector loop of evolve() (one increment):
  //   loop count = 0; cond(correctors) = any case live
  //   WHILE correctors: right-hand side; cond(pcg) = any component active
  //                     WHILE pcg: one PCG iteration; cond(pcg)
  //                     post-solve pass; cond(correctors)
  // Each loop is also bounded on the device (nCorrectors + 4 correctors,
  // maxIter + 4 PCG iterations per corrector).
  template <typename T>
  bool buildLoopGraph(cudaGraph_t g, const Controls& c, int tl, const PcgPtrs<T>& p, int grid) {
    cudaStream_t s = ctx->stream;
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    cudaGraphConditionalHandle hOut, hPcg;
    if (cudaGraphConditionalHandleCreate(&hOut, g, 0, cudaGraphCondAssignDefault) != cudaSuccess ||
        cudaGraphConditionalHandleCreate(&hPcg, g, 0, cudaGraphCondAssignDefault) != cudaSuccess)
      return false;
    const unsigned outerLimit = (unsigned)c.nCorr + 4, pcgLimit = (unsigned)c.maxIter + 4;
    cudaGraph_t outerBody = nullptr, pcgBody = nullptr, ended = nullptr;
    bool ok;
    if (cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, mode) != cudaSuccess) return false;
    launchSetLoopCond(hOut, dState, nRun, 1, 1, outerLimit, s);
    ok = addWhile(s, hOut, &outerBody);
    ok = cudaStreamEndCapture(s, &ended) == cudaSuccess && ok;
    if (!ok || cudaStreamBeginCaptureToGraph(s, outerBody, nullptr, nullptr, 0, mode) != cudaSuccess)
      return false;
    launchRhs<T>(mv, c, f, p.x, p.r, dState, dPartials, s, nullptr, nRun);
    launchSetLoopCond(hPcg, dState, nRun, 0, 1, pcgLimit, s);
    ok = addWhile(s, hPcg, &pcgBody);
    launchPost<T>(mv, c, f, p.x, dState, dPartials, 1, s, nullptr, nRun, p.p, p.p2);
    launchSetLoopCond(hOut, dState, nRun, 1, 0, outerLimit, s);
    ok = cudaStreamEndCapture(s, &ended) == cudaSuccess && ok;
    if (!ok || cudaStreamBeginCaptureToGraph(s, pcgBody, nullptr, nullptr, 0, mode) != cudaSuccess)
      return false;
    long long dummy = 0;
    if (mv.subdomains && c.precond == 0)
      launchLocalIteration<T>(mv, c, p, dState, dPartials, tuning<T>(), s, &dummy, nullptr, nRun);
    else
      launchPcgIteration<T>(mv, c, p, dState, dPartials, grid, s, &dummy, nullptr);
    launchSetLoopCond(hPcg, dState, nRun, 0, 0, pcgLimit, s);
    ok = cudaStreamEndCapture(s, &ended) == cudaSuccess;
    (void)tl;
    return ok && cudaGetLastError() == cudaSuccess;
  }

  // The loop graph for the current state of the engine (built on first use);
  // nullptr if it cannot be built, in which case the host drives the loop.
  template <typename T>
  cudaGraphExec_t loopGraph(const Controls& c, int tl, const PcgPtrs<T>& p, int grid) {
    const long key = ((long)(sizeof(T)) << 40) | ((long)tl << 32) | ((long)nRun << 8);
    PcgGraph& g = loopGraphs[key];
    const LocalTuning& t = tuning<T>();
    if (g.exec && g.generation == generation && g.ntIdx == t.ntIdx && g.uIdx == t.uIdx &&
        g.grid == grid && std::memcmp(&g.c, &c, sizeof(Controls)) == 0)
      return g.exec;
    if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
    cudaGraph_t graph = nullptr;
    bool ok = cudaGraphCreate(&graph, 0) == cudaSuccess && buildLoopGraph<T>(graph, c, tl, p, grid);
    if (ok) ok = cudaGraphInstantiate(&g.exec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {
      loopGraphsOk = false;
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
      cudaGetLastError();
      return nullptr;
    }
    g.generation = generation; g.ntIdx = t.ntIdx; g.uIdx = t.uIdx; g.grid = grid; g.c = c;
    return g.exec;
  }

  template <typename T>
  s4g_status pcgLoop(const Controls& c, const PcgPtrs<T>& p, int grid) {
    // Iterations are launched in growing batches; the launches after the
    // device's stop decision return at once.
    int chunk = 2, launched = 0;
    pcgBase.resize(nRun);
    for (int cs = 0; cs < nRun; ++cs) pcgBase[cs] = hState[cs].pcgIter;
    auto launchBatch = [&](int n, long long* count) {
      for (int i = 0; i < n; ++i) {
        if (tm()) timer.tag = launched++;
        if (mv.subdomains && c.precond == 0)
          launchLocalIteration<T>(mv, c, p, dState, dPartials, tuning<T>(), ctx->stream,
                                  count, tm(), nRun);
        else
          launchPcgIteration<T>(mv, c, p, dState, dPartials, grid, ctx->stream, count, tm());
      }
    };
    for (int guard = 0; guard < 1000000; ++guard) {
      cudaGraphExec_t exec = (!ctx->profile && !ctx->noGraphs && graphsOk)
                                 ? pcgGraph<T>(c, p, grid, chunk, launchBatch)
                                 : nullptr;
      if (exec) {
        S4G_CUDA(cudaGraphLaunch(exec, ctx->stream));
        long long perBatch = 0;  // count what the batch launches
        const int ut = tuning<T>().uIdx;
        perBatch = (mv.subdomains && c.precond == 0) ? (long long)chunk * (ut == 2 ? 3 : 2)
                                                     : (long long)chunk * (c.precond == 0 ? 5 : 4);
        launches += perBatch;
      } else {
        launchBatch(chunk, &launches);
      }
      timer.tag = -1;
      S4G_CUDA(cudaGetLastError());
      S4G_TRY(readState(true));
      if (!anyCase(&DevState::pcgContinue)) return S4G_OK;
      if (nRun == 1 && (hState->status & (kErrTimeout | kErrNaN))) return S4G_OK;
      chunk = std::min(chunk * 2, 16);
    }
    return setErr(S4G_TIMEOUT, "PCG loop did not end");
  }

  // One evolve(): correctors until converged() or nCorrectors.  The inner
  // PCG runs in T; the right-hand side, the correction of D and every
  // convergence test stay in FP64.
  template <typename T>
  s4g_status correctorLoop(Controls& c, int tl, const PcgPtrs<T>& p, int grid) {
    cudaStream_t s = ctx->stream;
    if (!ctx->profile && !ctx->noGraphs && !ctx->verbose && loopGraphsOk) {
      cudaGraphExec_t exec = loopGraph<T>(c, tl, p, grid);
      if (exec) {
        // one launch runs every corrector on the device; the host waits once
        const int corr0 = hState->nCorrDone, it0 = hState->pcgIter;
        S4G_CUDA(cudaGraphLaunch(exec, s));
        S4G_CUDA(cudaGetLastError());
        S4G_TRY(readState());
        const bool local = mv.subdomains && c.precond == 0;
        const long long perIt = local ? (tuning<T>().uIdx == 2 ? 3 : 2) : (c.precond == 0 ? 5 : 4);
        launches += 1 + (long long)(hState->nCorrDone - corr0) * (tl ? 6 : 5) +
                    (long long)(hState->pcgIter - it0) * (perIt + 1);
        ranOnDevice = true;
        return S4G_OK;
      }
    }
    for (;;) {
      launchRhs<T>(mv, c, f, p.x, p.r, dState, dPartials, s, tm(), nRun);
      launches += 2;
      S4G_TRY(readState());
      if (anyCase(&DevState::pcgContinue)) S4G_TRY(pcgLoop<T>(c, p, grid));
      launchPost<T>(mv, c, f, p.x, dState, dPartials, 1, s, tm(), nRun, p.p, p.p2);
      launches += tl ? 3 : 2;
      S4G_CUDA(cudaGetLastError());
      S4G_TRY(readState());
      if (ctx->verbose && outer.info_frequency > 0 &&
          ((hState->iCorr - 1) % outer.info_frequency == 0 || hState->converged))
        std::printf("    %d, %g, %g, 0, %d\n", hState->iCorr - 1, hState->initResMag, hState->relRes,
                    hState->lastMaxIters);
      if (nRun == 1 && (hState->status & (kErrTimeout | kErrNaN))) return S4G_OK;
      if (!anyCase(&DevState::caseLive)) return S4G_OK;
    }
  }

  // step: one evolve() of a time step (s4g_solve_step) with the boundary
  // values as set (load factor 1), from the state the previous step left;
  // the first step, a step after s4g_state_reset or after a full solve, and
  // a step of another model start from zero as s4g_solve does.
  s4g_status solve(s4g_model model, int nInc, double* Dout, double* sigOut, s4g_perf* perf,
                   bool step = false) {
    if (model != S4G_LIN_GEOM_TOTAL_DISP && model != S4G_NONLIN_GEOM_TOTAL_LAG &&
        model != S4G_NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP)
      return setErr(S4G_BAD_ARG, "unknown model");
    if (!materialSet) return setErr(S4G_BAD_ARG, "material not set");
    // Controls::tl: 0 linear geometry, 1 TL incremental, 2 TL total
    const int tl = model == S4G_NONLIN_GEOM_TOTAL_LAG ? 1
                 : model == S4G_NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP ? 2 : 0;
    if (tl && law.type != S4G_NEO_HOOKEAN) return setErr(S4G_BAD_ARG, "the TL model needs a neoHookeanElastic law");
    if (!tl && law.type != S4G_LINEAR_ELASTIC) return setErr(S4G_BAD_ARG, "the linear-geometry model needs a linearElastic law");
    if (tl) S4G_TRY(allocTL());
    S4G_TRY(ensureAitken());
    if (!tl || step) nInc = 1;
    if (nInc < 1) return setErr(S4G_BAD_ARG, "n_increments must be >= 1");
    cudaStream_t s = ctx->stream;
    const long long launches0 = launches;
    const bool cont = step && stepLive && stepTl == tl;
    stepLive = false;
    S4G_TRY(ensureMatrix());
    const bool mixed = precision == S4G_FP32_REFINE;
    if (mixed) S4G_TRY(ensureFp32());
    cudaEvent_t e0, e1;
    S4G_CUDA(cudaEventCreate(&e0));
    S4G_CUDA(cudaEventCreate(&e1));
    if (mv.subdomains && lin.preconditioner == S4G_PRECOND_DIC) {
      const Controls ct = controls(tl);
      if (mixed) S4G_TRY(tuneLocal<float>(ct, pc32));
      else S4G_TRY(tuneLocal<double>(ct, pc));
    }
    nRun = 1;
    ranOnDevice = false;
    const int corr0 = cont ? hState->nCorrDone : 0;
    const long long lin0 = cont ? hState->totalLinIters : 0;
    if (!cont) {
      S4G_TRY(initFields(tl));
      S4G_TRY(resetSweepState());
    } else {
      // a later time step: evolve() restarts iCorr (and enforceLinear); the
      // linear model's D.oldTime is the last step's D (the TL forms shifted
      // theirs at the end of the last step)
      int zero = 0;
      S4G_CUDA(cudaMemcpyAsync(&dState->iCorr, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
      S4G_CUDA(cudaMemcpyAsync(&dState->enforceLinear, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
      if (!tl)
        S4G_CUDA(cudaMemcpyAsync(f.D0, f.D[hState->dcur], sizeof(double) * 3 * hp.nC,
                                 cudaMemcpyDeviceToDevice, s));
    }
    S4G_TRY(setLive());
    timer.reset();
    S4G_CUDA(cudaEventRecord(e0, s));
    Controls c = controls(tl);
    int nCorrTotal = 0;
    auto loop = [&](int isTl) -> s4g_status {
      return mixed ? correctorLoop<float>(c, isTl, pc32, sweepGrid32)
                   : correctorLoop<double>(c, isTl, pc, sweepGrid);
    };
    if (!tl) {
      launchTractionInit(mv, c, f, s);
      if (!cont) launchPost<double>(mv, c, f, pc.x, dState, dPartials, 0, s);
      launches += cont ? 1 : 2;
      S4G_TRY(loop(0));
      nCorrTotal = hState->nCorrDone - corr0;
    } else {
      for (int n = 1; n <= nInc; ++n) {
        c.loadFactor = step ? 1.0 : (double)n / nInc;
        // evolve(): enforceLinear = false; iCorr restarts
        int zero = 0;
        S4G_CUDA(cudaMemcpyAsync(&dState->enforceLinear, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
        S4G_CUDA(cudaMemcpyAsync(&dState->iCorr, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
        S4G_TRY(setLive());
        launchTractionInit(mv, c, f, s);
        launches++;
        S4G_TRY(loop(1));
        launchTlShift(mv, c, f, dState, s);
        launches += c.tl == 1 ? 2 : 1;
        if (hState->status & (kErrTimeout | kErrNaN)) break;
      }
      S4G_TRY(readState());
      nCorrTotal = hState->nCorrDone - corr0;
    }
    S4G_CUDA(cudaEventRecord(e1, s));
    S4G_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // outputs in caller order
    auto t0 = std::chrono::steady_clock::now();
    if (Dout) {
      const double* src = tl ? f.D0 : f.D[hState->dcur];
      launchGather(hp.nC, 3, dC2s, src, dOut, s);
      S4G_CUDA(cudaMemcpyAsync(Dout, dOut, sizeof(double) * 3 * hp.nC, cudaMemcpyDeviceToHost, s));
    }
    if (sigOut) {
      launchGather(hp.nC, 6, dC2s, f.sig, dOut + 3 * (size_t)hp.nC, s);
      S4G_CUDA(cudaMemcpyAsync(sigOut, dOut + 3 * (size_t)hp.nC, sizeof(double) * 6 * hp.nC, cudaMemcpyDeviceToHost, s));
    }
    S4G_CUDA(cudaStreamSynchronize(s));
    auto t1 = std::chrono::steady_clock::now();
    lastModel = model;
    if (perf) {
      std::memset(perf, 0, sizeof(*perf));
      perf->n_correctors = nCorrTotal;
      perf->converged = hState->converged;
      perf->total_lin_iters = hState->totalLinIters - lin0;
      perf->last_max_lin_iters = hState->lastMaxIters;
      perf->initial_residual = hState->initResMag;
      perf->rel_residual = hState->relRes;
      perf->solve_ms = ms;
      perf->d2h_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
      perf->kernel_launches = launches - launches0;
      perf->enforce_linear = hState->enforceLinear;
      perf->device_status = (int)hState->status;
      const bool local = mv.subdomains && lin.preconditioner == S4G_PRECOND_DIC;
      const LocalTuning& lt = mixed ? tune32 : tune64;
      perf->part_threads = local ? localPartThreads(mv, lt.ntIdx) : 0;
      perf->spmv_unroll = local ? kLocVariantsU[lt.uIdx] : 0;
      for (int k = 0; k < 6; ++k)
        perf->tune_us[k] = (local && k < kLocNumNT + kLocNumU) ? tuneUs[mixed ? 1 : 0][k] : 0.0;
      timer.resolve();
      for (int k = 0; k < S4G_K_KINDS; ++k) {
        perf->kernel_ms[k] = timer.ms[k];
        perf->kernel_launches_by[k] = timer.count[k];
      }
      perf->device_loop = ranOnDevice ? 1 : 0;
    }
    if (hState->status & kErrTimeout) return setErr(S4G_TIMEOUT, "a bounded device wait gave up");
    if (hState->status & kErrNaN) return setErr(S4G_NAN_DETECTED, "non-finite value in the iteration");
    if (hState->status & kErrIndefinite) return setErr(S4G_INDEFINITE, "PCG met p.Ap <= 0");
    // a later step may continue from a step's state
    stepLive = step;
    stepTl = tl;
    if (!hState->converged) return S4G_NOT_CONVERGED;
    return S4G_OK;
  }

  // ------------------------------------------------------ many meshes ---
  // s4g_solve_batch: each mesh of the batch prepares its solve on the
  // context's stream (matrix, FP32 copies, tuning, initial fields and the
  // constructor's gradient pass), captures its device-resident corrector
  // loop as an independent branch of one shared graph, and after the one
  // launch of that graph reads back its own state and fields.
  s4g_status batchPrepare() {
    if (!materialSet) return setErr(S4G_BAD_ARG, "material not set");
    if (law.type != S4G_LINEAR_ELASTIC)
      return setErr(S4G_BAD_ARG, "s4g_solve_batch runs the linearGeometryTotalDisplacement model "
                                 "(linearElastic law)");
    S4G_TRY(ensureAitken());
    S4G_TRY(ensureMatrix());
    const bool mixed = precision == S4G_FP32_REFINE;
    if (mixed) S4G_TRY(ensureFp32());
    if (mv.subdomains && lin.preconditioner == S4G_PRECOND_DIC) {
      const Controls ct = controls(0);
      if (mixed) S4G_TRY(tuneLocal<float>(ct, pc32));
      else S4G_TRY(tuneLocal<double>(ct, pc));
    }
    nRun = 1;
    ranOnDevice = false;
    S4G_TRY(initFields(0));
    S4G_TRY(resetSweepState());
    S4G_TRY(setLive());
    timer.reset();
    batchLaunches0 = launches;
    const Controls c = controls(0);
    launchTractionInit(mv, c, f, ctx->stream);
    launchPost<double>(mv, c, f, pc.x, dState, dPartials, 0, ctx->stream);
    launches += 2;
    S4G_CUDA(cudaGetLastError());
    return S4G_OK;
  }
  bool batchCapture(cudaGraph_t g) {
    const Controls c = controls(0);
    return precision == S4G_FP32_REFINE ? buildLoopGraph<float>(g, c, 0, pc32, sweepGrid32)
                                        : buildLoopGraph<double>(g, c, 0, pc, sweepGrid);
  }
  s4g_status batchFinish(double* Dout, double* sigOut, s4g_perf* perf, float ms) {
    cudaStream_t s = ctx->stream;
    S4G_TRY(readState());
    ranOnDevice = true;
    const bool local = mv.subdomains && lin.preconditioner == S4G_PRECOND_DIC;
    const long long perIt = local ? (tuning32or64().uIdx == 2 ? 3 : 2)
                                  : (lin.preconditioner == S4G_PRECOND_DIC ? 5 : 4);
    launches += 1 + (long long)hState->nCorrDone * 5 + (long long)hState->pcgIter * (perIt + 1);
    if (Dout) {
      launchGather(hp.nC, 3, dC2s, f.D[hState->dcur], dOut, s);
      S4G_CUDA(cudaMemcpyAsync(Dout, dOut, sizeof(double) * 3 * hp.nC, cudaMemcpyDeviceToHost, s));
    }
    if (sigOut) {
      launchGather(hp.nC, 6, dC2s, f.sig, dOut + 3 * (size_t)hp.nC, s);
      S4G_CUDA(cudaMemcpyAsync(sigOut, dOut + 3 * (size_t)hp.nC, sizeof(double) * 6 * hp.nC,
                               cudaMemcpyDeviceToHost, s));
    }
    S4G_CUDA(cudaStreamSynchronize(s));
    lastModel = S4G_LIN_GEOM_TOTAL_DISP;
    if (perf) {
      std::memset(perf, 0, sizeof(*perf));
      perf->n_correctors = hState->nCorrDone;
      perf->converged = hState->converged;
      perf->total_lin_iters = hState->totalLinIters;
      perf->last_max_lin_iters = hState->lastMaxIters;
      perf->initial_residual = hState->initResMag;
      perf->rel_residual = hState->relRes;
      perf->solve_ms = ms;
      perf->kernel_launches = launches - batchLaunches0;
      perf->device_status = (int)hState->status;
      const LocalTuning& lt = tuning32or64();
      perf->part_threads = local ? localPartThreads(mv, lt.ntIdx) : 0;
      perf->spmv_unroll = local ? kLocVariantsU[lt.uIdx] : 0;
      perf->device_loop = 1;
    }
    if (hState->status & kErrTimeout) return setErr(S4G_TIMEOUT, "a bounded device wait gave up");
    if (hState->status & kErrNaN) return setErr(S4G_NAN_DETECTED, "non-finite value in the iteration");
    if (hState->status & kErrIndefinite) return setErr(S4G_INDEFINITE, "PCG met p.Ap <= 0");
    if (!hState->converged) return S4G_NOT_CONVERGED;
    return S4G_OK;
  }
  const LocalTuning& tuning32or64() const { return precision == S4G_FP32_REFINE ? tune32 : tune64; }
  long long batchLaunches0 = 0;

  // ---------------------------------------------------------- operators ---
  // All copies go through the library's stream (non-blocking: it does not
  // order against the legacy default stream), then wait for it.
  s4g_status copySync(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    S4G_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, ctx->stream));
    S4G_CUDA(cudaStreamSynchronize(ctx->stream));
    return S4G_OK;
  }

  s4g_status opMatrix(double* diag, double* upper) {
    S4G_TRY(ensureMatrix());
    std::vector<double> v(2 * (size_t)hp.nI), dg(hp.nC);
    S4G_TRY(copySync(v.data(), dVal, sizeof(double) * v.size(), cudaMemcpyDeviceToHost));
    S4G_TRY(copySync(dg.data(), dDiag, sizeof(double) * dg.size(), cudaMemcpyDeviceToHost));
    for (int s = 0; s < hp.nC; ++s) {
      if (diag) diag[hp.s2c[s]] = dg[s];
      for (int e = hp.rowptr[s]; e < hp.rowptr[s + 1]; ++e)
        if (hp.fidx[e] >= 0 && upper) upper[hp.fcaller[hp.fidx[e]]] = v[e];
    }
    return S4G_OK;
  }

  s4g_status toStorage(int k, const double* in, std::vector<double>& out) {
    out.assign(3 * (size_t)hp.nC, 0.0);
    for (int s = 0; s < hp.nC; ++s)
      for (int j = 0; j < k; ++j) out[3 * (size_t)s + j] = in[(size_t)hp.s2c[s] * k + j];
    return S4G_OK;
  }
  void fromStorage(int k, const std::vector<double>& in, double* out) {
    for (int s = 0; s < hp.nC; ++s)
      for (int j = 0; j < k; ++j) out[(size_t)hp.s2c[s] * k + j] = in[3 * (size_t)s + j];
  }

  s4g_status opAmul(int k, const double* x, double* y) {
    if (k < 1 || k > 3 || !x || !y) return setErr(S4G_BAD_ARG, "k must be 1..3");
    S4G_TRY(ensureMatrix());
    std::vector<double> hx, hy(3 * (size_t)hp.nC);
    toStorage(k, x, hx);
    S4G_TRY(copySync(pc.w, hx.data(), sizeof(double) * hx.size(), cudaMemcpyHostToDevice));
    launchAmul<double>(mv, (const double*)dVal, dDiag, pc.w, pc.q, ctx->stream);
    launches++;
    S4G_CUDA(cudaGetLastError());
    S4G_TRY(copySync(hy.data(), pc.q, sizeof(double) * hy.size(), cudaMemcpyDeviceToHost));
    fromStorage(k, hy, y);
    return S4G_OK;
  }

  s4g_status opPrecondition(int k, const double* r, double* w) {
    if (k < 1 || k > 3 || !r || !w) return setErr(S4G_BAD_ARG, "k must be 1..3");
    S4G_TRY(ensureMatrix());
    std::vector<double> hr, hw(3 * (size_t)hp.nC);
    toStorage(k, r, hr);
    S4G_TRY(copySync(pc.r, hr.data(), sizeof(double) * hr.size(), cudaMemcpyHostToDevice));
    S4G_TRY(resetSweepState());
    DevState init{};
    init.pcgContinue = 1;
    S4G_CUDA(cudaMemcpyAsync(&dState->pcgContinue, &init.pcgContinue, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    Controls c = controls(0);
    launchPrecondOnly<double>(mv, c, pc, dState, dPartials, sweepGrid, ctx->stream);
    launches += 2;
    S4G_CUDA(cudaGetLastError());
    S4G_CUDA(cudaStreamSynchronize(ctx->stream));
    S4G_TRY(readState());
    if (hState->status & kErrTimeout) return setErr(S4G_TIMEOUT, "sweep wait gave up");
    S4G_TRY(copySync(hw.data(), pc.w, sizeof(double) * hw.size(), cudaMemcpyDeviceToHost));
    fromStorage(k, hw, w);
    return S4G_OK;
  }

  s4g_status opAmulDotNoAlloc(int k, const double* x, double* y, double* xAx) {
    if (!matrixValid)
      return setErr(S4G_BAD_ARG, "the matrix is not assembled yet: call s4g_op_matrix or s4g_solve "
                                 "first (s4g_op_amul_dot_noalloc does no set-up work)");
    std::string err;
    const s4g_status st = s4g::opAmulDotNoAlloc(mv, dC2s, dVal, dDiag, pc.w, pc.q, ctx->device,
                                                ctx->stream, k, x, y, xAx, err);
    if (st != S4G_OK) return setErr(st, err);
    launches += 3;
    return S4G_OK;
  }

  // Points of the mesh for the device point interpolation (s4g_mesh_set_points).
  int nPoints = -1;
  double* dPts = nullptr;
  int* dPcs = nullptr;
  int* dPcc = nullptr;
  double* dPointD = nullptr;

  s4g_status setPoints(int nP, const double* pts, const int* pcs, const int* pcc) {
    if (nP < 0 || (nP > 0 && (!pts || !pcs || !pcc)))
      return setErr(S4G_BAD_ARG, "s4g_mesh_set_points: bad arguments");
    if (nP > 0 && pcs[0] != 0) return setErr(S4G_BAD_ARG, "point_cell_start[0] must be 0");
    for (int p = 0; p < nP; ++p)
      if (pcs[p + 1] < pcs[p]) return setErr(S4G_BAD_ARG, "point_cell_start must not decrease");
    const int nE = nP > 0 ? pcs[nP] : 0;
    for (int k = 0; k < nE; ++k)
      if (pcc[k] < 0 || pcc[k] >= hp.nC) return setErr(S4G_BAD_ARG, "point cell out of range");
    S4G_CUDA(cudaStreamSynchronize(ctx->stream));
    for (void* q : {(void*)dPts, (void*)dPcs, (void*)dPcc, (void*)dPointD})
      if (q) {
        cudaFree(q);
        allocs.erase(std::find(allocs.begin(), allocs.end(), q));
      }
    dPts = nullptr; dPcs = nullptr; dPcc = nullptr; dPointD = nullptr;
    S4G_TRY(alloc(&dPts, 3 * (size_t)nP));
    S4G_TRY(alloc(&dPcs, (size_t)nP + 1));
    S4G_TRY(alloc(&dPcc, (size_t)nE));
    S4G_TRY(alloc(&dPointD, 3 * (size_t)nP));
    cudaStream_t s = ctx->stream;
    if (nP > 0) {
      S4G_CUDA(cudaMemcpyAsync(dPts, pts, sizeof(double) * 3 * nP, cudaMemcpyHostToDevice, s));
      S4G_CUDA(cudaMemcpyAsync(dPcs, pcs, sizeof(int) * (nP + 1), cudaMemcpyHostToDevice, s));
      if (nE) S4G_CUDA(cudaMemcpyAsync(dPcc, pcc, sizeof(int) * nE, cudaMemcpyHostToDevice, s));
    }
    S4G_CUDA(cudaStreamSynchronize(s));
    nPoints = nP;
    return S4G_OK;
  }

  s4g_status getPointD(double* out) {
    if (lastModel < 0) return setErr(S4G_BAD_ARG, "no solve has run");
    if (nPoints < 0) return setErr(S4G_BAD_ARG, "no points: call s4g_mesh_set_points first");
    if (!out) return setErr(S4G_BAD_ARG, "null output");
    const bool tlm = lastModel != S4G_LIN_GEOM_TOTAL_DISP;
    const double* U = tlm ? f.D0 : f.D[hState->dcur];
    const double* G = tlm ? f.GD : f.G;
    launchPointInterp(nPoints, dPts, dPcs, dPcc, dC2s, geo.C, U, G, dPointD, ctx->stream);
    launches++;
    S4G_CUDA(cudaGetLastError());
    S4G_CUDA(cudaMemcpyAsync(out, dPointD, sizeof(double) * 3 * (size_t)nPoints,
                             cudaMemcpyDeviceToHost, ctx->stream));
    S4G_CUDA(cudaStreamSynchronize(ctx->stream));
    return S4G_OK;
  }

  s4g_status getGradD(double* out) {
    if (lastModel < 0) return setErr(S4G_BAD_ARG, "no solve has run");
    const double* src = lastModel != S4G_LIN_GEOM_TOTAL_DISP ? f.GD : f.G;
    launchGather(hp.nC, 9, dC2s, src, dOut, ctx->stream);
    S4G_CUDA(cudaMemcpyAsync(out, dOut, sizeof(double) * 9 * hp.nC, cudaMemcpyDeviceToHost, ctx->stream));
    S4G_CUDA(cudaStreamSynchronize(ctx->stream));
    return S4G_OK;
  }
};

}  // namespace s4g

// ------------------------------------------------------------------ C ABI ---

struct s4g_mesh;
// A context owns its meshes: destroying it frees the meshes still alive.
struct s4g_ctx {
  s4g::Ctx c;
  std::vector<s4g_mesh*> meshes;
};
struct s4g_mesh {
  s4g::Engine e;
  s4g_ctx* owner = nullptr;
};

using s4g::setErr;

extern "C" {

const char* s4g_status_str(s4g_status st) {
  switch (st) {
    case S4G_OK: return "OK";
    case S4G_BAD_ARG: return "BAD_ARG";
    case S4G_OOM: return "OOM";
    case S4G_NOT_CONVERGED: return "NOT_CONVERGED";
    case S4G_NAN_DETECTED: return "NAN_DETECTED";
    case S4G_INDEFINITE: return "INDEFINITE";
    case S4G_TIMEOUT: return "TIMEOUT";
    case S4G_CUDA_ERROR: return "CUDA_ERROR";
    case S4G_NO_DEVICE: return "NO_DEVICE";
    case S4G_ADMISSION_REJECTED: return "ADMISSION_REJECTED";
    case S4G_PENDING: return "PENDING";
    case S4G_CANCELLED: return "CANCELLED";
    case S4G_NOT_BUILT: return "NOT_BUILT";
  }
  return "UNKNOWN";
}

int s4g_abi_version(void) { return S4G_ABI_VERSION; }

const char* s4g_last_error(void) { return s4g::gLastError.c_str(); }

s4g_status s4g_ctx_create(s4g_ctx** out, const s4g_ctx_opts* opts) {
  if (!out) return setErr(S4G_BAD_ARG, "null output");
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return setErr(S4G_NO_DEVICE, "no CUDA device");
  int dev = opts ? opts->device : 0;
  if (dev < 0 || dev >= n) return setErr(S4G_BAD_ARG, "device ordinal out of range");
  std::unique_ptr<s4g_ctx> c(new s4g_ctx());
  c->c.device = dev;
  c->c.verbose = opts ? opts->verbose : 0;
  c->c.profile = opts ? opts->profile : 0;
  c->c.noGraphs = opts ? opts->no_graphs : 0;
  if (opts && opts->spin_limit < 0) return setErr(S4G_BAD_ARG, "spin_limit must be >= 0");
  c->c.spinLimit = (opts && opts->spin_limit > 0) ? opts->spin_limit : s4g::kSpinLimit;
  if (cudaSetDevice(dev) != cudaSuccess) return setErr(S4G_CUDA_ERROR, "cudaSetDevice failed");
  cudaDeviceGetAttribute(&c->c.numSMs, cudaDevAttrMultiProcessorCount, dev);
  if (cudaStreamCreateWithFlags(&c->c.stream, cudaStreamNonBlocking) != cudaSuccess)
    return setErr(S4G_CUDA_ERROR, "cudaStreamCreate failed");
  *out = c.release();
  return S4G_OK;
}

s4g_status s4g_ctx_destroy(s4g_ctx* ctx) {
  if (!ctx) return S4G_BAD_ARG;
  cudaSetDevice(ctx->c.device);
  if (ctx->c.stream) cudaStreamSynchronize(ctx->c.stream);
  for (s4g_mesh* m : ctx->meshes) delete m;
  ctx->meshes.clear();
  if (ctx->c.stream) cudaStreamDestroy(ctx->c.stream);
  delete ctx;
  return S4G_OK;
}

s4g_status s4g_mesh_upload(s4g_ctx* ctx, const s4g_mesh_desc* desc, const s4g_mesh_opts* opts,
                           s4g_mesh** out) {
  if (!ctx || !desc || !out) return setErr(S4G_BAD_ARG, "null argument");
  *out = nullptr;
  cudaSetDevice(ctx->c.device);
  std::unique_ptr<s4g_mesh> m(new s4g_mesh());
  m->e.ctx = &ctx->c;
  s4g_lin_solver lin;
  s4g_outer outer;
  s4g_default_controls(&lin, &outer);
  m->e.lin = lin;
  m->e.outer = outer;
  s4g_status st = m->e.uploadMesh(desc, opts);
  if (st != S4G_OK) return st;
  m->owner = ctx;
  ctx->meshes.push_back(m.get());
  *out = m.release();
  return S4G_OK;
}

s4g_status s4g_mesh_get_permutation(const s4g_mesh* mesh, int* perm) {
  if (!mesh || !perm) return setErr(S4G_BAD_ARG, "null argument");
  const s4g::HostPrep& hp = mesh->e.hp;
  // solver rank r -> caller cell
  for (int s = 0; s < hp.nC; ++s) perm[hp.solverRank[s]] = hp.s2c[s];
  return S4G_OK;
}

s4g_status s4g_mesh_get_parts(const s4g_mesh* mesh, int* part_of_cell) {
  if (!mesh || !part_of_cell) return setErr(S4G_BAD_ARG, "null argument");
  const s4g::HostPrep& hp = mesh->e.hp;
  for (int p = 0; p < hp.nParts; ++p)
    for (int s = hp.partStart[p]; s < hp.partStart[p + 1]; ++s) part_of_cell[hp.s2c[s]] = p;
  return S4G_OK;
}

s4g_status s4g_mesh_plan(const s4g_mesh_desc* desc, const s4g_mesh_opts* opts, int* perm_out,
                         s4g_mesh_info* info) {
  if (!desc) return setErr(S4G_BAD_ARG, "null mesh");
  s4g::HostPrep hp;
  std::string err;
  s4g_status st = s4g::prepareMesh(desc, opts, hp, err);
  if (st != S4G_OK) return setErr(st, err);
  if (perm_out)
    for (int s = 0; s < hp.nC; ++s) perm_out[hp.solverRank[s]] = hp.s2c[s];
  if (info) {
    std::memset(info, 0, sizeof(*info));
    info->n_cells = hp.nC;
    info->n_internal_faces = hp.nI;
    info->n_boundary_faces = hp.nB;
    info->n_parts = hp.nParts;
    info->part_depth = hp.partDepth;
    info->max_local_levels = hp.maxLocalLevels;
    info->n_levels_global = hp.globalLevels;
    info->n_local_entries = (long long)hp.locSrc.size();
    info->local_slots = hp.locSlots ? 1 : 0;
  }
  return S4G_OK;
}

s4g_status s4g_mesh_get_info(const s4g_mesh* mesh, s4g_mesh_info* info) {
  if (!mesh || !info) return setErr(S4G_BAD_ARG, "null argument");
  const s4g::HostPrep& hp = mesh->e.hp;
  info->n_cells = hp.nC;
  info->n_internal_faces = hp.nI;
  info->n_boundary_faces = hp.nB;
  info->n_parts = hp.nParts;
  info->part_depth = hp.partDepth;
  info->max_local_levels = hp.maxLocalLevels;
  info->n_levels_global = hp.globalLevels;
  info->device_bytes = (long long)mesh->e.bytes;
  info->n_local_entries = (long long)hp.locSrc.size();
  info->local_slots = hp.locSlots ? 1 : 0;
  return S4G_OK;
}

s4g_status s4g_mesh_destroy(s4g_mesh* mesh) {
  if (!mesh) return S4G_BAD_ARG;
  cudaSetDevice(mesh->e.ctx->device);
  cudaStreamSynchronize(mesh->e.ctx->stream);
  if (mesh->owner) {
    auto& v = mesh->owner->meshes;
    v.erase(std::remove(v.begin(), v.end(), mesh), v.end());
  }
  delete mesh;
  return S4G_OK;
}

s4g_status s4g_material_set(s4g_mesh* mesh, const s4g_law* law) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  return mesh->e.setMaterial(law);
}

s4g_status s4g_bc_set(s4g_mesh* mesh, int patch, s4g_bc_type type, const double* vec3,
                      const double* pressure) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  return mesh->e.setBC(patch, type, vec3, pressure);
}

s4g_status s4g_bc_set_relaxation(s4g_mesh* mesh, int patch, double factor) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  return mesh->e.setRelaxation(patch, factor);
}

void s4g_default_controls(s4g_lin_solver* lin, s4g_outer* outer) {
  if (lin) {
    lin->preconditioner = S4G_PRECOND_DIC;
    lin->tolerance = 1e-9;
    lin->rel_tol = 0.1;
    lin->max_iter = 1000;
  }
  if (outer) {
    outer->n_correctors = 10000;
    outer->solution_tol = 1e-6;
    outer->alternative_tol = 1e-7;
    outer->material_tol = 1e-5;
    outer->stab_scale = 0.1;
    outer->info_frequency = 100;
    outer->field_relaxation = 1.0;
    outer->relaxation_method = 0;
  }
}

s4g_status s4g_solver_set(s4g_mesh* mesh, const s4g_lin_solver* lin, const s4g_outer* outer,
                          s4g_precision precision) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  if (lin) {
    if (lin->max_iter < 0 || !(lin->tolerance >= 0) || !(lin->rel_tol >= 0) ||
        (lin->preconditioner != S4G_PRECOND_DIC && lin->preconditioner != S4G_PRECOND_DIAGONAL))
      return setErr(S4G_BAD_ARG, "invalid linear solver controls");
    mesh->e.lin = *lin;
  }
  if (outer) {
    if (outer->n_correctors < 1 || !(outer->stab_scale >= 0))
      return setErr(S4G_BAD_ARG, "invalid outer controls");
    if (!(outer->field_relaxation >= 0.0 && outer->field_relaxation <= 1.0))
      return setErr(S4G_BAD_ARG, "field_relaxation must be in (0, 1] (0: none)");
    if (outer->relaxation_method != 0 && outer->relaxation_method != 1)
      return setErr(S4G_BAD_ARG, "relaxation_method must be 0 (fixed) or 1 (Aitken)");
    mesh->e.outer = *outer;
  }
  if (precision != S4G_FP64 && precision != S4G_FP32_REFINE) return setErr(S4G_BAD_ARG, "unknown precision");
  mesh->e.precision = precision;
  return S4G_OK;
}

s4g_status s4g_solve(s4g_mesh* mesh, s4g_model model, int n_increments, double* D_out,
                     double* sigma_out, s4g_perf* perf) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  cudaSetDevice(mesh->e.ctx->device);
  return mesh->e.solve(model, n_increments, D_out, sigma_out, perf);
}

s4g_status s4g_solve_step(s4g_mesh* mesh, s4g_model model, double* D_out, double* sigma_out,
                          s4g_perf* perf) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  cudaSetDevice(mesh->e.ctx->device);
  return mesh->e.solve(model, 1, D_out, sigma_out, perf, true);
}

s4g_status s4g_state_reset(s4g_mesh* mesh) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  mesh->e.stepLive = false;
  return S4G_OK;
}

s4g_status s4g_get_gradD(s4g_mesh* mesh, double* gradD_out) {
  if (!mesh || !gradD_out) return setErr(S4G_BAD_ARG, "null argument");
  return mesh->e.getGradD(gradD_out);
}

s4g_status s4g_mesh_set_points(s4g_mesh* mesh, int n_points, const double* points,
                               const int* point_cell_start, const int* point_cells) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  if (cudaSetDevice(mesh->e.ctx->device) != cudaSuccess)
    return setErr(S4G_CUDA_ERROR, "cudaSetDevice failed");
  return mesh->e.setPoints(n_points, points, point_cell_start, point_cells);
}

s4g_status s4g_get_pointD(s4g_mesh* mesh, double* pointD_out) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  if (cudaSetDevice(mesh->e.ctx->device) != cudaSuccess)
    return setErr(S4G_CUDA_ERROR, "cudaSetDevice failed");
  return mesh->e.getPointD(pointD_out);
}

s4g_status s4g_op_matrix(s4g_mesh* mesh, double* diag, double* upper) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  return mesh->e.opMatrix(diag, upper);
}

s4g_status s4g_op_amul(s4g_mesh* mesh, int k, const double* x, double* y) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  return mesh->e.opAmul(k, x, y);
}

s4g_status s4g_op_precondition(s4g_mesh* mesh, int k, const double* r, double* w) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  return mesh->e.opPrecondition(k, r, w);
}

s4g_status s4g_solve_cases(s4g_mesh* mesh, int n_cases, const double* bval,
                           const double* bpress, double* D_out, double* sigma_out,
                           s4g_perf* perf) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  if (cudaSetDevice(mesh->e.ctx->device) != cudaSuccess)
    return setErr(S4G_CUDA_ERROR, "cudaSetDevice failed");
  return mesh->e.solveCases(n_cases, bval, bpress, D_out, sigma_out, perf);
}

s4g_status s4g_solve_batch(s4g_mesh* const* meshes, int n_meshes, double* const* D_out,
                           double* const* sigma_out, s4g_perf* perf) {
  if (!meshes || n_meshes < 1) return setErr(S4G_BAD_ARG, "need at least one mesh");
  s4g_ctx* owner = meshes[0] ? meshes[0]->owner : nullptr;
  if (!owner) return setErr(S4G_BAD_ARG, "null mesh");
  for (int i = 0; i < n_meshes; ++i) {
    if (!meshes[i] || meshes[i]->owner != owner)
      return setErr(S4G_BAD_ARG, "every mesh of a batch must belong to the same context");
    for (int j = 0; j < i; ++j)
      if (meshes[j] == meshes[i]) return setErr(S4G_BAD_ARG, "a mesh appears twice in the batch");
  }
  s4g::Ctx& cx = owner->c;
  if (cx.profile || cx.noGraphs || cx.verbose)
    return setErr(S4G_BAD_ARG, "s4g_solve_batch runs one CUDA graph: the context must not set "
                               "profile, verbose or no_graphs");
  if (cudaSetDevice(cx.device) != cudaSuccess) return setErr(S4G_CUDA_ERROR, "cudaSetDevice failed");
  for (int i = 0; i < n_meshes; ++i) {
    const s4g_status st = meshes[i]->e.batchPrepare();
    if (st != S4G_OK) return st;
  }
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return setErr(S4G_CUDA_ERROR, "cudaGraphCreate failed");
  for (int i = 0; i < n_meshes; ++i)
    if (!meshes[i]->e.batchCapture(g)) {
      cudaGraphDestroy(g);
      cudaGetLastError();
      return setErr(S4G_CUDA_ERROR, "capturing a mesh's corrector loop into the batch graph failed");
    }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) return setErr(S4G_CUDA_ERROR, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, cx.stream);
  cudaError_t le = cudaGraphLaunch(exec, cx.stream);
  cudaEventRecord(e1, cx.stream);
  cudaError_t se = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGraphExecDestroy(exec);
  if (le != cudaSuccess || se != cudaSuccess)
    return setErr(S4G_CUDA_ERROR, std::string("batch graph: ") + cudaGetErrorString(le != cudaSuccess ? le : se));
  s4g_status ret = S4G_OK;
  for (int i = 0; i < n_meshes; ++i) {
    const s4g_status st = meshes[i]->e.batchFinish(D_out ? D_out[i] : nullptr,
                                                   sigma_out ? sigma_out[i] : nullptr,
                                                   perf ? perf + i : nullptr, ms);
    if (st == S4G_NOT_CONVERGED) { if (ret == S4G_OK) ret = st; }
    else if (st != S4G_OK) ret = st;
  }
  return ret;
}

s4g_status s4g_op_amul_dot_noalloc(s4g_mesh* mesh, int k, const double* x, double* y,
                                   double* xAx) {
  if (!mesh) return setErr(S4G_BAD_ARG, "null mesh");
  if (cudaSetDevice(mesh->e.ctx->device) != cudaSuccess)
    return setErr(S4G_CUDA_ERROR, "cudaSetDevice failed");
  return mesh->e.opAmulDotNoAlloc(k, x, y, xAx);
}

}  // extern "C"
