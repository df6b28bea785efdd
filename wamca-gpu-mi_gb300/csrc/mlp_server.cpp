// mlp_server.cpp -- serving form: continuous batching of arriving DVND searches.
//
// Requests (coordinates, start tour, neighbourhood mask, sweep limit) arrive at
// any time through mlp_server_submit().  Each mlp_server_step()
//   1. admits queued requests in arrival order while a slot is free and their
//      device footprint (n x n distances, coordinates and the job arena) fits
//      the memory budget.  Admission is stream-ordered: the memory comes from
//      the server's own pool with cudaMallocFromPoolAsync, the distance matrix
//      is built on the device from the coordinates, the start tour is uploaded
//      and the ADS prefix arrays are prepared, with no host synchronisation;
//   2. runs `iters` DVND iterations over every admitted search in shared
//      launches: one sweep over all searches' tiles, then one merge launch for
//      the searches whose merge fits shared memory and one for the rest (one
//      CTA per search when many are active, a six-CTA cluster per search
//      otherwise).  A search that converged or used its sweep limit turns
//      into no-op CTAs;
//   3. reads every slot's statistics (one copy) and retires the finished
//      searches: tour and statistics become the request's result, the memory
//      returns to the pool in stream order and the slot is free again.
// Searches join and leave between iterations, so requests that arrive while
// others run on the GPU start as soon as a slot and memory free up.  A search's
// trajectory depends only on its own data (its candidate keys, merge and apply
// are per job), so its result is identical alone and in any mix.
//
// Thread safety: submit, result, finished, cancel and status may be called
// from any thread while one thread drives step().
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/mlp_gpu.h"
#include "mlp_capi_internal.h"
#include "mlp_engine.h"
#include "mlp_kernels.cuh"

using namespace mlp;

namespace {

struct Request {
  int64_t id = 0;
  int n = 0;
  int dist_round = 1;
  int mask = 0x1f;
  int64_t max_iters = 0;
  std::vector<int32_t> x, y, tour;
  double arrival = 0;
  size_t footprint = 0;
};

struct Active {
  std::unique_ptr<Request> req;
  std::unique_ptr<Problem> prob;
  std::unique_ptr<Job> job;
  int slot = -1;
  double admitted = 0;
};

struct Result {
  int status = kOk;
  int n = 0;
  int64_t cost = 0, iterations = 0, sweeps = 0, moves = 0, evals = 0;
  int converged = 0;
  std::vector<int32_t> tour;
  double arrival = 0, admitted = 0, finished = 0;
};

size_t al256(size_t v) { return (v + 255) / 256 * 256; }

int64_t evals_per_sweep(int size, int mask) {
  int64_t e = 0;
  for (int nb = 0; nb < kNumNb; nb++)
    if ((mask >> nb) & 1) e += (int64_t)nb_blocks(nb, size) * nb_threads(nb, size);
  return e;
}

}  // namespace

struct mlp_server {
  size_t budget = 0;
  bool wide = false;
  int max_slots = 0;
  int shape = -1;  // -1: chosen per step from the largest admitted search
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;
  std::chrono::steady_clock::time_point t0;

  // Guarded by mu: the request queue, results, cancellations and counters.
  std::mutex mu;
  std::deque<std::unique_ptr<Request>> queue;
  std::unordered_map<int64_t, Result> results;
  std::unordered_set<int64_t> pending;  // queued or admitted, no result yet
  std::vector<int64_t> finished_ids;
  std::vector<int64_t> cancel_ids;
  int64_t next_id = 1;
  size_t in_use = 0;
  int n_active = 0;
  int fail_next = 0;  // admissions to fail on the host (failure-handling tests)

  // Owned by the stepping thread.
  std::vector<Active> active;
  std::vector<int> free_slots;
  JobDev* djobs = nullptr;   // launch order of the active searches
  JobDev* dnew = nullptr;    // searches admitted in this step
  int64_t* dstats = nullptr; // kStatWords per slot
  SweepTile* dtiles = nullptr;
  size_t tiles_cap = 0;
  JobDev* hjobs = nullptr;   // pinned staging
  JobDev* hnew = nullptr;
  int64_t* hstats = nullptr;
  int64_t* hinit = nullptr;  // initial statistics row per slot
  SweepTile* htiles = nullptr;
  size_t htiles_cap = 0;
  std::vector<SweepTile> job_tile_buf;

  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
  ~mlp_server();
};

static int arg_error(const char* msg) {
  set_error(msg);
  return kErrArg;
}

#define MLP_CUDA(call, what)             \
  do {                                   \
    int st_ = cuda_status((call), what); \
    if (st_ != kOk) return st_;          \
  } while (0)

#define MLP_TRY(expr)           \
  do {                          \
    int st_ = (expr);           \
    if (st_ != kOk) return st_; \
  } while (0)

static size_t server_footprint(int n, bool wide) {
  return al256(sizeof(int32_t) * (size_t)n * n + 16) + 2 * al256(sizeof(int32_t) * (size_t)n) +
         job_bytes(n + 1, wide, 0);
}

mlp_server::~mlp_server() {
  if (stream) cudaStreamSynchronize(stream);
  active.clear();  // frees every job and problem in stream order
  if (stream) cudaStreamSynchronize(stream);
  if (djobs) cudaFree(djobs);
  if (dnew) cudaFree(dnew);
  if (dstats) cudaFree(dstats);
  if (dtiles) cudaFree(dtiles);
  if (hjobs) cudaFreeHost(hjobs);
  if (hnew) cudaFreeHost(hnew);
  if (hstats) cudaFreeHost(hstats);
  if (hinit) cudaFreeHost(hinit);
  if (htiles) cudaFreeHost(htiles);
  if (pool) cudaMemPoolDestroy(pool);
  if (stream) cudaStreamDestroy(stream);
}

// Records the result of a request that ends without a search on the device.
static void finish_without_search(mlp_server* s, std::unique_ptr<Request> r, int status, double admitted) {
  Result res;
  res.status = status;
  res.n = r->n;
  res.arrival = r->arrival;
  res.admitted = admitted;
  res.finished = s->now();
  std::lock_guard<std::mutex> lock(s->mu);
  s->pending.erase(r->id);
  s->results[r->id] = std::move(res);
  s->finished_ids.push_back(r->id);
}

static int admit_one(mlp_server* s, Active& a) {
  Request& r = *a.req;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->fail_next > 0) {
      s->fail_next--;
      set_error("host allocation failure injected at admission");
      return kErrNoMem;
    }
  }
  Problem* p = nullptr;
  MLP_TRY(problem_from_coords_async(r.n, r.x.data(), r.y.data(), r.dist_round, s->pool, s->stream, &p));
  a.prob.reset(p);
  Job* j = nullptr;
  MLP_TRY(job_create_async(p, s->wide, s->pool, s->stream, &j));
  a.job.reset(j);
  j->dev.nb_mask = r.mask;
  j->dev.stats = s->dstats + (size_t)a.slot * kStatWords;
  MLP_CUDA(cudaMemcpyAsync(j->dev.tour, r.tour.data(), sizeof(int32_t) * r.tour.size(), cudaMemcpyHostToDevice,
                           s->stream),
           "copy tour");
  int64_t* row = s->hinit + (size_t)a.slot * kStatWords;
  std::memset(row, 0, sizeof(int64_t) * kStatWords);
  row[kStatLimit] = r.max_iters;
  MLP_CUDA(cudaMemcpyAsync(j->dev.stats, row, sizeof(int64_t) * kStatWords, cudaMemcpyHostToDevice, s->stream),
           "init stats");
  return kOk;
}

static int ensure_tiles(mlp_server* s, size_t count) {
  if (count > s->htiles_cap) {
    if (s->htiles) cudaFreeHost(s->htiles);
    s->htiles = nullptr;
    s->htiles_cap = 0;
    const size_t cap = std::max<size_t>(count + count / 2, 4096);
    MLP_CUDA(cudaMallocHost(&s->htiles, sizeof(SweepTile) * cap), "cudaMallocHost(tiles)");
    s->htiles_cap = cap;
  }
  if (count > s->tiles_cap) {
    if (s->dtiles) MLP_CUDA(cudaFreeAsync(s->dtiles, s->stream), "cudaFreeAsync(tiles)");
    s->dtiles = nullptr;
    s->tiles_cap = 0;
    const size_t cap = std::max<size_t>(count + count / 2, 4096);
    MLP_CUDA(cudaMallocAsync(&s->dtiles, sizeof(SweepTile) * cap, s->stream), "cudaMallocAsync(tiles)");
    s->tiles_cap = cap;
  }
  return kOk;
}

static int server_step(mlp_server* s, int iters) {
  // 1. Admission, in arrival order, while a slot is free and memory fits.
  std::vector<std::unique_ptr<Request>> admit;
  std::vector<int64_t> cancels;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    while (!s->queue.empty() && s->active.size() + admit.size() < (size_t)s->max_slots) {
      Request* r = s->queue.front().get();
      if (s->in_use + r->footprint > s->budget) break;
      s->in_use += r->footprint;
      admit.push_back(std::move(s->queue.front()));
      s->queue.pop_front();
    }
    cancels.swap(s->cancel_ids);
  }
  const double t_admit = s->now();
  int nfresh = 0;
  for (auto& r : admit) {
    Active a;
    a.req = std::move(r);
    a.admitted = t_admit;
    a.slot = s->free_slots.back();
    s->free_slots.pop_back();
    const int st = admit_one(s, a);
    if (st != kOk) {
      // The request ends with the error; whatever it allocated goes back.
      const size_t fp = a.req->footprint;
      a.job.reset();
      a.prob.reset();
      s->free_slots.push_back(a.slot);
      {
        std::lock_guard<std::mutex> lock(s->mu);
        s->in_use -= fp;
      }
      finish_without_search(s, std::move(a.req), st, t_admit);
      if (st == kErrCuda) return st;  // the stream is unusable
      continue;
    }
    s->hnew[nfresh++] = a.job->dev;
    s->active.push_back(std::move(a));
  }
  if (nfresh > 0) {
    MLP_CUDA(cudaMemcpyAsync(s->dnew, s->hnew, sizeof(JobDev) * nfresh, cudaMemcpyHostToDevice, s->stream),
             "copy new jobs");
    MLP_CUDA(launch_prepare(s->dnew, nfresh, s->wide, false, s->stream), "prepare kernel");
  }

  // 2. Iterations over every admitted search: searches whose merge fits
  //    shared memory first, the rest (global merge workspace) after them.
  const int smem_max = std::min(merge_smem_max_size(), solo_smem_max_size());
  std::stable_sort(s->active.begin(), s->active.end(), [smem_max](const Active& a, const Active& b) {
    return (a.job->size > smem_max) < (b.job->size > smem_max);
  });
  const int nact = (int)s->active.size();
  if (nact > 0 && iters > 0) {
    int ksmall = 0, max_small = 0, max_large = 0, max_size = 0;
    bool all_nb = true;  // every search evaluates all five neighbourhoods
    for (const Active& a : s->active) {
      const int sz = a.job->size;
      all_nb &= a.job->dev.nb_mask == 0x1f;
      max_size = std::max(max_size, sz);
      if (sz <= smem_max) {
        ksmall++;
        max_small = std::max(max_small, sz);
      } else {
        max_large = std::max(max_large, sz);
      }
    }
    const int shape = s->shape >= 0 ? s->shape : default_shape(max_size, nact);
    size_t ntiles = 0;
    for (int q = 0; q < nact; q++) {
      const int sz = s->active[q].job->size;
      ntiles += sweep_tiles(sz, kTileShapes[shape].tl, kTileShapes[shape].tr);
    }
    MLP_TRY(ensure_tiles(s, ntiles));
    size_t t = 0;
    for (int q = 0; q < nact; q++) {
      s->hjobs[q] = s->active[q].job->dev;
      job_tiles(s->active[q].job->size, shape, &s->job_tile_buf);
      for (SweepTile tile : s->job_tile_buf) {
        tile.job = q;
        s->htiles[t++] = tile;
      }
    }
    MLP_CUDA(cudaMemcpyAsync(s->djobs, s->hjobs, sizeof(JobDev) * nact, cudaMemcpyHostToDevice, s->stream),
             "copy jobs");
    MLP_CUDA(cudaMemcpyAsync(s->dtiles, s->htiles, sizeof(SweepTile) * t, cudaMemcpyHostToDevice, s->stream),
             "copy tiles");
    for (int it = 0; it < iters; it++) {
      if (!s->wide && all_nb)
        MLP_CUDA(launch_sweep_dvnd(s->dtiles, (int)t, s->djobs, shape, false, s->stream), "sweep kernel");
      else
        MLP_CUDA(launch_sweep(s->dtiles, (int)t, s->djobs, s->wide, shape, true, s->stream), "sweep kernel");
      if (nact >= kSoloMinJobs) {
        MLP_CUDA(launch_merge_solo(s->djobs, ksmall, s->wide, true, max_small, s->stream), "merge kernel");
        MLP_CUDA(launch_merge_solo(s->djobs + ksmall, nact - ksmall, s->wide, false, max_large, s->stream),
                 "merge kernel");
      } else {
        MLP_CUDA(launch_merge(s->djobs, ksmall, s->wide, true, max_small, s->stream), "merge kernel");
        MLP_CUDA(launch_merge(s->djobs + ksmall, nact - ksmall, s->wide, false, max_large, s->stream),
                 "merge kernel");
      }
    }
  }

  // 3. Statistics of every slot, then retirement of the finished searches.
  MLP_CUDA(cudaMemcpyAsync(s->hstats, s->dstats, sizeof(int64_t) * kStatWords * s->max_slots,
                           cudaMemcpyDeviceToHost, s->stream),
           "read stats");
  MLP_CUDA(cudaStreamSynchronize(s->stream), "step");
  std::vector<Active> keep, done;
  std::vector<int> done_status;
  for (Active& a : s->active) {
    const int64_t* row = s->hstats + (size_t)a.slot * kStatWords;
    const bool cancelled = std::find(cancels.begin(), cancels.end(), a.req->id) != cancels.end();
    if (cancelled || row[kStatError] || row[kStatConverged] || row[kStatSweeps] >= row[kStatLimit]) {
      done_status.push_back(cancelled ? (int)MLP_ERR_CANCELLED : row[kStatError] ? (int)kErrState : (int)kOk);
      done.push_back(std::move(a));
    } else {
      keep.push_back(std::move(a));
    }
  }
  s->active.swap(keep);
  if (done.empty()) {
    std::lock_guard<std::mutex> lock(s->mu);
    s->n_active = (int)s->active.size();
    return kOk;
  }
  std::vector<Result> res(done.size());
  for (size_t q = 0; q < done.size(); q++) {
    Result& r = res[q];
    const Active& a = done[q];
    const int64_t* row = s->hstats + (size_t)a.slot * kStatWords;
    r.status = done_status[q];
    r.n = a.req->n;
    r.cost = row[kStatCost];
    r.iterations = row[kStatIters];
    r.sweeps = row[kStatSweeps];
    r.moves = row[kStatMoves];
    r.evals = row[kStatSweeps] * evals_per_sweep(a.job->size, a.req->mask);
    r.converged = (int)row[kStatConverged];
    r.arrival = a.req->arrival;
    r.admitted = a.admitted;
    r.tour.resize(a.job->size);
    MLP_CUDA(cudaMemcpyAsync(r.tour.data(), a.job->dev.tour, sizeof(int32_t) * a.job->size, cudaMemcpyDeviceToHost,
                             s->stream),
             "read tour");
  }
  MLP_CUDA(cudaStreamSynchronize(s->stream), "read tours");
  const double t_done = s->now();
  size_t freed = 0;
  for (Active& a : done) {
    freed += a.req->footprint;
    s->free_slots.push_back(a.slot);
    a.job.reset();  // stream-ordered frees
    a.prob.reset();
  }
  std::lock_guard<std::mutex> lock(s->mu);
  s->in_use -= freed;
  s->n_active = (int)s->active.size();
  for (size_t q = 0; q < done.size(); q++) {
    res[q].finished = t_done;
    s->pending.erase(done[q].req->id);
    s->results[done[q].req->id] = std::move(res[q]);
    s->finished_ids.push_back(done[q].req->id);
  }
  return kOk;
}

// ---------------------------------------------------------------- C-ABI
extern "C" {

MLP_API int64_t mlp_server_footprint(int32_t n, int32_t wide) {
  if (n < 1 || n + 1 > kMaxSize) return -1;
  return (int64_t)server_footprint(n, wide != 0);
}

MLP_API int mlp_server_create(int64_t memory_budget, int32_t wide, int32_t max_active, mlp_server_t* out) {
  if (!out) return arg_error("null output handle");
  *out = nullptr;
  if (memory_budget <= 0) return arg_error("memory budget must be positive");
  if (max_active < 1 || max_active > 65536) return arg_error("max_active must lie in [1, 65536]");
  std::unique_ptr<mlp_server> s(new mlp_server());
  s->budget = (size_t)memory_budget;
  s->wide = wide != 0;
  s->max_slots = max_active;
  s->t0 = std::chrono::steady_clock::now();
  MLP_CUDA(cudaGetDevice(&s->device), "cudaGetDevice");
  MLP_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = s->device;
  MLP_CUDA(cudaMemPoolCreate(&s->pool, &props), "cudaMemPoolCreate");
  // Keep freed memory in the pool (up to the budget) for the next admissions.
  uint64_t keep = (uint64_t)memory_budget;
  MLP_CUDA(cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep), "pool threshold");
  const size_t slots = (size_t)max_active;
  MLP_CUDA(cudaMalloc(&s->djobs, sizeof(JobDev) * slots), "cudaMalloc(jobs)");
  MLP_CUDA(cudaMalloc(&s->dnew, sizeof(JobDev) * slots), "cudaMalloc(jobs)");
  MLP_CUDA(cudaMalloc(&s->dstats, sizeof(int64_t) * kStatWords * slots), "cudaMalloc(stats)");
  MLP_CUDA(cudaMemset(s->dstats, 0, sizeof(int64_t) * kStatWords * slots), "memset(stats)");
  MLP_CUDA(cudaMallocHost(&s->hjobs, sizeof(JobDev) * slots), "cudaMallocHost");
  MLP_CUDA(cudaMallocHost(&s->hnew, sizeof(JobDev) * slots), "cudaMallocHost");
  MLP_CUDA(cudaMallocHost(&s->hstats, sizeof(int64_t) * kStatWords * slots), "cudaMallocHost");
  MLP_CUDA(cudaMallocHost(&s->hinit, sizeof(int64_t) * kStatWords * slots), "cudaMallocHost");
  for (int q = max_active - 1; q >= 0; q--) s->free_slots.push_back(q);
  MLP_CUDA(configure_prepare(), "configure prepare kernel");
  MLP_CUDA(configure_merge(merge_smem_bytes(merge_smem_max_size())), "configure merge");
  *out = s.release();
  return kOk;
}

MLP_API void mlp_server_destroy(mlp_server_t s) { delete s; }

MLP_API double mlp_server_now(mlp_server_t s) { return s ? s->now() : 0.0; }

MLP_API int mlp_server_set_tile_shape(mlp_server_t s, int32_t shape) {
  if (!s) return arg_error("null server");
  if (shape < -1 || shape >= kNumTileShapes) return arg_error("tile shape out of range");
  s->shape = shape;
  return kOk;
}

MLP_API int mlp_server_submit(mlp_server_t s, int32_t n, const int32_t* x, const int32_t* y, int32_t dist_round,
                              const int32_t* tour, int32_t len, int32_t nb_mask, int32_t max_iters,
                              double arrival, int64_t* id) {
  MLP_RANGE("mlp_server_submit");
  if (!s || !x || !y || !tour) return arg_error("null argument");
  if (n < 5 || n + 1 > kMaxSize) {
    set_error("n must lie in [5, max size - 1]");
    return kErrRange;
  }
  if (nb_mask <= 0 || nb_mask > 0x1f) return arg_error("neighbourhood mask must be a nonzero subset of 0x1f");
  if (max_iters <= 0) return arg_error("max_iters must be positive");
  MLP_TRY(validate_tour(tour, len, n, n + 1));
  for (int q = 0; q < n; q++) {
    if (std::abs((int64_t)x[q] - x[0]) > 16383 || std::abs((int64_t)y[q] - y[0]) > 16383) {
      set_error("coordinate spans must not exceed 32767");
      return kErrRange;
    }
  }
  std::unique_ptr<Request> r(new Request());
  r->n = n;
  r->dist_round = dist_round ? 1 : 0;
  r->mask = nb_mask;
  r->max_iters = max_iters;
  r->x.assign(x, x + n);
  r->y.assign(y, y + n);
  r->tour.assign(tour, tour + len);
  r->arrival = arrival >= 0 ? arrival : s->now();
  r->footprint = server_footprint(n, s->wide);
  if (r->footprint > s->budget) {
    set_error("the request's device footprint exceeds the server's whole memory budget");
    return kErrNoMem;
  }
  std::lock_guard<std::mutex> lock(s->mu);
  r->id = s->next_id++;
  if (id) *id = r->id;
  s->pending.insert(r->id);
  s->queue.push_back(std::move(r));
  return kOk;
}

MLP_API int mlp_server_step(mlp_server_t s, int32_t iters, int32_t* active, int32_t* queued) {
  MLP_RANGE("mlp_server_step");
  if (!s) return arg_error("null server");
  if (iters < 0 || iters > 4096) return arg_error("iters must lie in [0, 4096]");
  const int st = server_step(s, iters);
  std::lock_guard<std::mutex> lock(s->mu);
  if (active) *active = s->n_active;
  if (queued) *queued = (int32_t)s->queue.size();
  return st;
}

MLP_API int mlp_server_finished(mlp_server_t s, int64_t* ids, int32_t cap, int32_t* count) {
  if (!s || !count || (cap > 0 && !ids)) return arg_error("null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  const int32_t k = (int32_t)std::min<size_t>(cap > 0 ? cap : 0, s->finished_ids.size());
  std::copy(s->finished_ids.begin(), s->finished_ids.begin() + k, ids);
  s->finished_ids.erase(s->finished_ids.begin(), s->finished_ids.begin() + k);
  *count = k;
  return kOk;
}

MLP_API int mlp_server_result(mlp_server_t s, int64_t id, int32_t* tour, int32_t len, mlp_dvnd_stats_t* stats,
                              mlp_serve_info_t* info) {
  if (!s) return arg_error("null server");
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->results.find(id);
  if (it == s->results.end()) {
    if (s->pending.count(id)) return MLP_PENDING;
    set_error("unknown request id (never submitted, or its result was already taken)");
    return kErrArg;
  }
  const Result& r = it->second;
  if (tour && r.status == kOk) {
    if (len != (int32_t)r.tour.size()) return arg_error("tour buffer length must equal n + 1");
    std::copy(r.tour.begin(), r.tour.end(), tour);
  }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->cost = r.cost;
    stats->iterations = r.iterations;
    stats->sweeps = r.sweeps;
    stats->moves = r.moves;
    stats->evals = r.evals;
    stats->converged = r.converged;
  }
  if (info) {
    info->arrival = r.arrival;
    info->admitted = r.admitted;
    info->finished = r.finished;
    info->status = r.status;
    info->n = r.n;
  }
  s->results.erase(it);
  return kOk;
}

MLP_API int mlp_server_cancel(mlp_server_t s, int64_t id) {
  if (!s) return arg_error("null server");
  std::unique_ptr<Request> r;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
      if ((*it)->id == id) {
        r = std::move(*it);
        s->queue.erase(it);
        break;
      }
    }
    if (!r) {
      if (!s->pending.count(id)) {
        set_error("unknown or finished request id");
        return kErrArg;
      }
      // Running (or being admitted): retired at the end of the next step.
      s->cancel_ids.push_back(id);
      return kOk;
    }
  }
  finish_without_search(s, std::move(r), MLP_ERR_CANCELLED, -1.0);
  return kOk;
}

MLP_API int mlp_server_status(mlp_server_t s, int64_t* mem_in_use, int32_t* active, int32_t* queued,
                              int32_t* finished) {
  if (!s) return arg_error("null server");
  std::lock_guard<std::mutex> lock(s->mu);
  if (mem_in_use) *mem_in_use = (int64_t)s->in_use;
  if (active) *active = s->n_active;
  if (queued) *queued = (int32_t)s->queue.size();
  if (finished) *finished = (int32_t)s->results.size();
  return kOk;
}

MLP_API int mlp_server_fail_next_admissions(mlp_server_t s, int32_t count) {
  if (!s) return arg_error("null server");
  if (count < 0) return arg_error("count must be non-negative");
  std::lock_guard<std::mutex> lock(s->mu);
  s->fail_next = count;
  return kOk;
}

}  // extern "C"
