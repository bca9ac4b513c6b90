// Serving: continuous admission of solid solves of uneven sizes onto one GPU.
//
// The server owns max_slots worker threads.  Each worker owns an s4g_ctx
// (its own CUDA stream) and runs one request at a time through the public C
// ABI: upload the mesh, set the law, the boundary conditions and the
// controls, solve, copy the results out, free the mesh.  Requests wait in
// a queue in submission order; a free worker takes the first waiting
// request whose device footprint fits in what the admitted requests leave
// of the memory budget (first fit), so small requests pass a large one that
// has to wait for memory.  Admitted requests run at the same time on their
// own streams, so their kernels overlap on the device, and each keeps its
// fields, matrix and solver state resident across all its correctors.  A
// request whose footprint exceeds the whole budget is rejected at submit.
//
// Every request computes exactly what a lone s4g_solve of the same inputs
// computes: it has its own context, mesh and state, and the kernel variants
// the autotuner can pick give bit-identical results.
//
// Latency is measured from submit to the end of the solve (results ready).

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "s4g.h"
#include "s4g_internal.hpp"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id = 0;
  // copies of the caller's inputs
  int nCells = 0, nFaces = 0, nInternal = 0, nPatches = 0;
  std::vector<int> owner, neighbour, patchStart, patchSize;
  std::vector<double> C, V, Cf, Sf;
  s4g_mesh_opts meshOpts{};
  s4g_law law{};
  std::vector<int> bcPatch;
  std::vector<s4g_bc_type> bcType;
  std::vector<std::vector<double>> bcVec, bcPress;
  std::vector<char> bcHasVec, bcHasPress;
  std::vector<double> bcRelax;      // solidTraction relaxationFactor per entry
  std::vector<int> partOfCell;      // copy of mesh_opts.part_of_cell (may be empty)
  s4g_lin_solver lin{};
  s4g_outer outer{};
  s4g_precision precision = S4G_FP64;
  s4g_model model = S4G_LIN_GEOM_TOTAL_DISP;
  int nIncrements = 1;
  long long footprint = 0;
  // state and results
  enum State { QUEUED, RUNNING, DONE, CANCELLED } state = QUEUED;
  Clock::time_point submitted, finished;
  s4g_status status = S4G_PENDING;
  std::string error;
  std::vector<double> D, sigma;
  s4g_perf perf{};
};

}  // namespace

struct s4g_server {
  s4g_server_opts opts{};
  std::mutex m;
  std::condition_variable cv;    // workers: work or stop
  std::condition_variable done;  // waiters: a request finished
  bool stop = false;
  uint64_t nextId = 1;
  std::deque<Request*> queue;
  std::map<uint64_t, Request*> all;
  long long inUse = 0;
  int running = 0;
  long long submitted = 0, completed = 0, rejected = 0, cancelled = 0;
  std::vector<double> latencies;  // ms, completed requests
  Clock::time_point firstSubmit{}, lastFinish{};
  bool anySubmit = false;
  std::vector<std::thread> workers;
};

namespace {

// Device bytes a request holds while it runs, from its sizes: mesh
// addressing and geometry, FP64 fields and matrix, PCG work vectors, the
// FP32 copies of the mixed-precision path, the processor-local DIC tables
// and the total Lagrangian fields -- the allocations of s4g_mesh_upload
// and s4g_solve, rounded up.
long long estimateFootprint(const Request& r) {
  const double N = r.nCells, F = r.nInternal, B = (double)r.nFaces - r.nInternal;
  double b = 0;
  b += N * (4 * 8 + 24 + 48 + 8 * 5) + F * (4 * 6 + 8 * 6 + 48 + 48 + 16 * 2) + B * (8 * 20);
  b += N * (8 * 3 + 24 * 3 + 72 + 48 + 72) + F * (48) + B * (24 + 72 + 48 + 24);
  b += N * 24 * 6;
  if (r.precision == S4G_FP32_REFINE) b += N * (8 + 12 * 6) + F * 16;
  if (r.meshOpts.dic_subdomains) b += F * 2 * 18 + N * 8;
  if (r.model != S4G_LIN_GEOM_TOTAL_DISP) b += N * (72 * 6 + 48 + 8) + B * (72 * 6 + 48 + 8);
  return (long long)(b * 1.15) + (16ll << 20);
}

s4g_status runOne(s4g_ctx* ctx, Request& r) {
  s4g_mesh_desc d{};
  d.n_cells = r.nCells; d.n_faces = r.nFaces; d.n_internal_faces = r.nInternal;
  d.owner = r.owner.data(); d.neighbour = r.neighbour.data();
  d.C = r.C.data(); d.V = r.V.data(); d.Cf = r.Cf.data(); d.Sf = r.Sf.data();
  d.n_patches = r.nPatches; d.patch_start = r.patchStart.data(); d.patch_size = r.patchSize.data();
  s4g_mesh* mesh = nullptr;
  s4g_mesh_opts mo = r.meshOpts;
  mo.part_of_cell = r.partOfCell.empty() ? nullptr : r.partOfCell.data();
  s4g_status st = s4g_mesh_upload(ctx, &d, &mo, &mesh);
  if (st != S4G_OK) { r.error = s4g_last_error(); return st; }
  st = s4g_material_set(mesh, &r.law);
  for (size_t i = 0; st == S4G_OK && i < r.bcPatch.size(); ++i)
    st = s4g_bc_set(mesh, r.bcPatch[i], r.bcType[i], r.bcHasVec[i] ? r.bcVec[i].data() : nullptr,
                    r.bcHasPress[i] ? r.bcPress[i].data() : nullptr);
  for (size_t i = 0; st == S4G_OK && i < r.bcPatch.size(); ++i)
    if (r.bcType[i] == S4G_SOLID_TRACTION && r.bcRelax[i] != 1.0)
      st = s4g_bc_set_relaxation(mesh, r.bcPatch[i], r.bcRelax[i]);
  if (st == S4G_OK) st = s4g_solver_set(mesh, &r.lin, &r.outer, r.precision);
  if (st == S4G_OK) {
    r.D.assign(3 * (size_t)r.nCells, 0.0);
    r.sigma.assign(6 * (size_t)r.nCells, 0.0);
    st = s4g_solve(mesh, r.model, r.nIncrements, r.D.data(), r.sigma.data(), &r.perf);
  }
  if (st != S4G_OK && st != S4G_NOT_CONVERGED) r.error = s4g_last_error();
  s4g_mesh_destroy(mesh);
  return st;
}

void workerLoop(s4g_server* sv, int slot) {
  s4g_ctx* ctx = nullptr;
  s4g_status ctxStatus = S4G_OK;
  if (!sv->opts.dry_run) {
    s4g_ctx_opts co{sv->opts.device, 0, 0, 0};
    ctxStatus = s4g_ctx_create(&ctx, &co);
  }
  (void)slot;
  std::unique_lock<std::mutex> lk(sv->m);
  for (;;) {
    Request* r = nullptr;
    sv->cv.wait(lk, [&] {
      if (sv->stop) return true;
      for (Request* q : sv->queue)
        if (q->footprint <= sv->opts.memory_budget - sv->inUse) return true;
      return false;
    });
    if (sv->stop) break;
    for (auto it = sv->queue.begin(); it != sv->queue.end(); ++it)
      if ((*it)->footprint <= sv->opts.memory_budget - sv->inUse) {
        r = *it;
        sv->queue.erase(it);
        break;
      }
    if (!r) continue;
    r->state = Request::RUNNING;
    sv->inUse += r->footprint;
    sv->running++;
    lk.unlock();
    s4g_status st;
    if (sv->opts.dry_run) {
      // scheduling checks without a GPU: a solve takes time in proportion to
      // its cells and gives zero fields
      std::this_thread::sleep_for(std::chrono::microseconds(
          (long long)(sv->opts.dry_run_us_per_kcell * r->nCells / 1000.0)));
      r->D.assign(3 * (size_t)r->nCells, 0.0);
      r->sigma.assign(6 * (size_t)r->nCells, 0.0);
      std::memset(&r->perf, 0, sizeof(r->perf));
      st = S4G_OK;
    } else if (ctxStatus != S4G_OK) {
      st = ctxStatus;
      r->error = "worker context could not be created";
    } else {
      st = runOne(ctx, *r);
    }
    lk.lock();
    r->status = st;
    r->state = Request::DONE;
    r->finished = Clock::now();
    sv->inUse -= r->footprint;
    sv->running--;
    sv->completed++;
    sv->lastFinish = r->finished;
    sv->latencies.push_back(std::chrono::duration<double, std::milli>(r->finished - r->submitted).count());
    sv->done.notify_all();
    sv->cv.notify_all();  // memory freed: others may fit now
  }
  lk.unlock();
  if (ctx) s4g_ctx_destroy(ctx);
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = p * (v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - i;
  return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" {

s4g_status s4g_server_create(const s4g_server_opts* opts, s4g_server** out) {
  if (!out) return S4G_BAD_ARG;
  *out = nullptr;
  s4g_server_opts o{};
  if (opts) o = *opts;
  if (o.max_slots <= 0) o.max_slots = 8;
  if (o.max_slots > 64) return S4G_BAD_ARG;
  if (o.dry_run_us_per_kcell <= 0) o.dry_run_us_per_kcell = 50.0;
  if (o.memory_budget <= 0) {
    if (o.dry_run) {
      o.memory_budget = 8ll << 30;
    } else {
      int n = 0;
      if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return S4G_NO_DEVICE;
      if (o.device < 0 || o.device >= n) return S4G_BAD_ARG;
      cudaSetDevice(o.device);
      size_t freeB = 0, totalB = 0;
      if (cudaMemGetInfo(&freeB, &totalB) != cudaSuccess) return S4G_CUDA_ERROR;
      o.memory_budget = (long long)(0.8 * (double)freeB);
    }
  } else if (!o.dry_run) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return S4G_NO_DEVICE;
  }
  s4g_server* sv = new s4g_server();
  sv->opts = o;
  for (int i = 0; i < o.max_slots; ++i) sv->workers.emplace_back(workerLoop, sv, i);
  *out = sv;
  return S4G_OK;
}

s4g_status s4g_server_submit(s4g_server* sv, const s4g_request* rq, uint64_t* id) {
  if (!sv || !rq || !rq->mesh || !id) return S4G_BAD_ARG;
  const s4g_mesh_desc* d = rq->mesh;
  if (d->n_cells <= 0 || d->n_faces < d->n_internal_faces || d->n_internal_faces < 0 ||
      !d->owner || (d->n_internal_faces > 0 && !d->neighbour) || !d->C || !d->V || !d->Cf ||
      !d->Sf || d->n_patches < 0 || (d->n_patches > 0 && (!d->patch_start || !d->patch_size)))
    return S4G_BAD_ARG;
  if (rq->n_bc < 0 || (rq->n_bc > 0 && (!rq->bc_patch || !rq->bc_type))) return S4G_BAD_ARG;
  Request* r = new Request();
  r->nCells = d->n_cells; r->nFaces = d->n_faces; r->nInternal = d->n_internal_faces;
  r->nPatches = d->n_patches;
  r->owner.assign(d->owner, d->owner + d->n_faces);
  if (d->n_internal_faces) r->neighbour.assign(d->neighbour, d->neighbour + d->n_internal_faces);
  r->C.assign(d->C, d->C + 3 * (size_t)d->n_cells);
  r->V.assign(d->V, d->V + d->n_cells);
  r->Cf.assign(d->Cf, d->Cf + 3 * (size_t)d->n_faces);
  r->Sf.assign(d->Sf, d->Sf + 3 * (size_t)d->n_faces);
  r->patchStart.assign(d->patch_start, d->patch_start + d->n_patches);
  r->patchSize.assign(d->patch_size, d->patch_size + d->n_patches);
  r->meshOpts = rq->mesh_opts;
  if (rq->mesh_opts.part_of_cell)
    r->partOfCell.assign(rq->mesh_opts.part_of_cell, rq->mesh_opts.part_of_cell + d->n_cells);
  r->meshOpts.part_of_cell = nullptr;  // the copy above is used at upload
  r->law = rq->law;
  for (int i = 0; i < rq->n_bc; ++i) {
    const int p = rq->bc_patch[i];
    if (p < 0 || p >= d->n_patches) { delete r; return S4G_BAD_ARG; }
    const size_t sz = (size_t)d->patch_size[p];
    r->bcPatch.push_back(p);
    r->bcType.push_back(rq->bc_type[i]);
    const double* v = rq->bc_vec3 ? rq->bc_vec3[i] : nullptr;
    const double* pr = rq->bc_pressure ? rq->bc_pressure[i] : nullptr;
    r->bcHasVec.push_back(v != nullptr);
    r->bcHasPress.push_back(pr != nullptr);
    r->bcVec.emplace_back(v ? std::vector<double>(v, v + 3 * sz) : std::vector<double>());
    r->bcPress.emplace_back(pr ? std::vector<double>(pr, pr + sz) : std::vector<double>());
    const double rf = rq->bc_relaxation ? rq->bc_relaxation[i] : 1.0;
    if (!(rf > 0.0 && rf <= 1.0)) { delete r; return S4G_BAD_ARG; }
    r->bcRelax.push_back(rf);
  }
  r->lin = rq->lin; r->outer = rq->outer; r->precision = rq->precision;
  r->model = rq->model; r->nIncrements = rq->n_increments < 1 ? 1 : rq->n_increments;
  r->footprint = estimateFootprint(*r);
  std::lock_guard<std::mutex> lk(sv->m);
  if (r->footprint > sv->opts.memory_budget) {
    sv->rejected++;
    delete r;
    return S4G_ADMISSION_REJECTED;
  }
  r->id = sv->nextId++;
  r->submitted = Clock::now();
  if (!sv->anySubmit) { sv->firstSubmit = r->submitted; sv->anySubmit = true; }
  sv->submitted++;
  sv->all[r->id] = r;
  sv->queue.push_back(r);
  *id = r->id;
  sv->cv.notify_all();
  return S4G_OK;
}

s4g_status s4g_server_poll(s4g_server* sv, uint64_t id, int wait, double* D_out,
                           double* sigma_out, s4g_perf* perf) {
  if (!sv) return S4G_BAD_ARG;
  std::unique_lock<std::mutex> lk(sv->m);
  auto it = sv->all.find(id);
  if (it == sv->all.end()) return S4G_BAD_ARG;
  Request* r = it->second;
  if (wait)
    sv->done.wait(lk, [&] { return r->state == Request::DONE || r->state == Request::CANCELLED; });
  if (r->state == Request::CANCELLED) {
    sv->all.erase(it);
    delete r;
    return S4G_CANCELLED;
  }
  if (r->state != Request::DONE) return S4G_PENDING;
  if (D_out && !r->D.empty()) std::memcpy(D_out, r->D.data(), sizeof(double) * r->D.size());
  if (sigma_out && !r->sigma.empty())
    std::memcpy(sigma_out, r->sigma.data(), sizeof(double) * r->sigma.size());
  if (perf) *perf = r->perf;
  const s4g_status st = r->status;
  if (!r->error.empty()) s4g::setLastError(r->error);
  sv->all.erase(it);
  delete r;
  return st;
}

s4g_status s4g_server_cancel(s4g_server* sv, uint64_t id) {
  if (!sv) return S4G_BAD_ARG;
  std::lock_guard<std::mutex> lk(sv->m);
  auto it = sv->all.find(id);
  if (it == sv->all.end()) return S4G_BAD_ARG;
  Request* r = it->second;
  if (r->state != Request::QUEUED) return S4G_BAD_ARG;  // running or finished: too late
  sv->queue.erase(std::find(sv->queue.begin(), sv->queue.end(), r));
  r->state = Request::CANCELLED;
  sv->cancelled++;
  sv->done.notify_all();
  return S4G_OK;
}

s4g_status s4g_server_get_stats(s4g_server* sv, s4g_server_stats* out) {
  if (!sv || !out) return S4G_BAD_ARG;
  std::lock_guard<std::mutex> lk(sv->m);
  std::memset(out, 0, sizeof(*out));
  out->submitted = sv->submitted;
  out->completed = sv->completed;
  out->rejected = sv->rejected;
  out->cancelled = sv->cancelled;
  out->running = sv->running;
  out->queued = (int)sv->queue.size();
  out->bytes_in_use = sv->inUse;
  out->memory_budget = sv->opts.memory_budget;
  out->p50_ms = percentile(sv->latencies, 0.50);
  out->p99_ms = percentile(sv->latencies, 0.99);
  double mean = 0;
  for (double l : sv->latencies) mean += l;
  out->mean_ms = sv->latencies.empty() ? 0.0 : mean / sv->latencies.size();
  const double span = sv->anySubmit && sv->completed
                          ? std::chrono::duration<double>(sv->lastFinish - sv->firstSubmit).count()
                          : 0.0;
  out->solves_per_s = span > 0 ? sv->completed / span : 0.0;
  return S4G_OK;
}

s4g_status s4g_server_destroy(s4g_server* sv) {
  if (!sv) return S4G_BAD_ARG;
  {
    std::lock_guard<std::mutex> lk(sv->m);
    sv->stop = true;
    for (Request* r : sv->queue) {
      r->state = Request::CANCELLED;
      sv->cancelled++;
    }
    sv->queue.clear();
    sv->cv.notify_all();
    sv->done.notify_all();
  }
  for (auto& t : sv->workers) t.join();
  for (auto& kv : sv->all) delete kv.second;
  delete sv;
  return S4G_OK;
}

}  // extern "C"
