// mlp_capi.cpp -- extern "C" API of libmlpgpu.so (declared in include/mlp_gpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <memory>
#include <vector>

#include "../../include/mlp_gpu.h"
#include "mlp_capi_internal.h"
#include "mlp_engine.h"
#include "mlp_kernels.cuh"

using namespace mlp;

#define MLP_CUDA(call, what)                        \
  do {                                              \
    int st_ = cuda_status((call), what);            \
    if (st_ != kOk) return st_;                     \
  } while (0)

#define MLP_TRY(expr)          \
  do {                         \
    int st_ = (expr);          \
    if (st_ != kOk) return st_; \
  } while (0)

static int arg_error(const char* msg) {
  set_error(msg);
  return kErrArg;
}

// ----------------------------------------------------------------------------
namespace mlp {

int validate_tour(const int32_t* tour, int len, int n, int size) {
  if (!tour) return arg_error("null tour");
  if (len != size) return arg_error("tour length must equal size = n + 1");
  if (tour[0] != 0 || tour[size - 1] != 0) return arg_error("the tour must start and end at depot 0");
  std::vector<uint8_t> seen(n, 0);
  for (int p = 1; p < size - 1; p++) {
    const int v = tour[p];
    if (v <= 0 || v >= n || seen[v]) return arg_error("tour positions 1..n-1 must hold a permutation of 1..n-1");
    seen[v] = 1;
  }
  return kOk;
}

int solver_init(mlp_solver* s, Problem* p, int wide) {
  s->prob = p;
  s->wide = wide != 0;
  MLP_CUDA(cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking), "cudaStreamCreate");
  Job* j = nullptr;
  MLP_TRY(job_create(p, s->wide, nb_blocks(2, p->size), &j));
  s->job.reset(j);
  s->set.reset(new JobSet({j}, s->wide, s->own_stream));
  MLP_TRY(s->set->init());
  // Start from the identity tour 0,1,...,n-1,0 so that every call is defined.
  std::vector<int32_t> t(p->size);
  for (int q = 0; q < p->n; q++) t[q] = q;
  t[p->size - 1] = 0;
  MLP_CUDA(cudaMemcpyAsync(j->dev.tour, t.data(), sizeof(int32_t) * p->size, cudaMemcpyHostToDevice,
                           s->set->stream()),
           "copy tour");
  MLP_TRY(s->set->prepare(true));
  MLP_CUDA(cudaStreamSynchronize(s->set->stream()), "prepare");
  return kOk;
}

int solver_stats(mlp_solver* s, mlp_dvnd_stats_t* out, int mask) {
  std::vector<std::array<int64_t, kStatWords>> st;
  MLP_TRY(s->set->read_stats(&st));
  if (out) {
    std::memset(out, 0, sizeof(*out));
    out->cost = st[0][kStatCost];
    out->iterations = st[0][kStatIters];
    out->sweeps = st[0][kStatSweeps];
    out->moves = st[0][kStatMoves];
    out->evals = st[0][kStatSweeps] * s->set->evals_per_sweep(0, mask);
    out->converged = (int32_t)st[0][kStatConverged];
  }
  return kOk;
}

}  // namespace mlp

mlp_solver::~mlp_solver() {
  set.reset();
  job.reset();
  if (dads) cudaFree(dads);
  if (dP) cudaFree(dP);
  if (own_stream) cudaStreamDestroy(own_stream);
}

// ----------------------------------------------------------------------------
extern "C" {

MLP_API int mlp_version(void) { return 10000; }

MLP_API const char* mlp_last_error(void) { return last_error(); }

MLP_API const char* mlp_status_string(int status) {
  switch (status) {
    case MLP_OK: return "ok";
    case MLP_ERR_ARG: return "invalid argument";
    case MLP_ERR_CUDA: return "CUDA error";
    case MLP_ERR_RANGE: return "value out of range";
    case MLP_ERR_IO: return "I/O error";
    case MLP_ERR_FORMAT: return "invalid format";
    case MLP_ERR_NOMEM: return "out of memory";
    case MLP_ERR_STATE: return "invalid state";
    case MLP_ERR_UNSUPPORTED: return "unsupported";
    case MLP_ERR_CANCELLED: return "cancelled";
    case MLP_PENDING: return "pending";
    default: return "unknown status";
  }
}

MLP_API int mlp_device_count(int32_t* count) {
  if (!count) return arg_error("null count");
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (e != cudaSuccess) {
    *count = 0;
    return cuda_status(e, "cudaGetDeviceCount");
  }
  *count = c;
  return kOk;
}

MLP_API int mlp_set_device(int32_t device) { return cuda_status(cudaSetDevice(device), "cudaSetDevice"); }

// ---------------------------------------------------------------- problem
MLP_API int mlp_problem_create_coords(int32_t n, const int32_t* x, const int32_t* y, int32_t cost_tour,
                                      int32_t dist_round, mlp_problem_t* out) {
  if (!out) return arg_error("null output handle");
  Problem* p = nullptr;
  MLP_TRY(problem_from_coords(n, x, y, cost_tour, dist_round, false, &p));
  *out = reinterpret_cast<mlp_problem_t>(p);
  return kOk;
}

MLP_API int mlp_problem_create_coords_device(int32_t n, const int32_t* x, const int32_t* y,
                                             int32_t cost_tour, int32_t dist_round, mlp_problem_t* out) {
  if (!out) return arg_error("null output handle");
  Problem* p = nullptr;
  MLP_TRY(problem_from_coords(n, x, y, cost_tour, dist_round, true, &p));
  *out = reinterpret_cast<mlp_problem_t>(p);
  return kOk;
}

MLP_API int mlp_problem_create_matrix(int32_t n, const int32_t* dist, int32_t cost_tour,
                                      mlp_problem_t* out) {
  if (!out) return arg_error("null output handle");
  Problem* p = nullptr;
  MLP_TRY(problem_from_matrix(n, dist, cost_tour, false, &p));
  *out = reinterpret_cast<mlp_problem_t>(p);
  return kOk;
}

MLP_API int mlp_problem_load_tsplib(const char* path, int32_t cost_tour, int32_t dist_round,
                                    mlp_problem_t* out) {
  if (!out || !path) return arg_error("null argument");
  Problem* p = nullptr;
  MLP_TRY(problem_from_tsplib(path, cost_tour, dist_round, &p));
  *out = reinterpret_cast<mlp_problem_t>(p);
  return kOk;
}

MLP_API int mlp_problem_info(mlp_problem_t h, int32_t* n, int32_t* size, int32_t* max_dist) {
  Problem* p = reinterpret_cast<Problem*>(h);
  if (!p) return arg_error("null problem");
  if (n) *n = p->n;
  if (size) *size = p->size;
  if (max_dist) *max_dist = p->dmax;
  return kOk;
}

MLP_API int mlp_problem_get_dist(mlp_problem_t h, int32_t* dist) {
  Problem* p = reinterpret_cast<Problem*>(h);
  if (!p || !dist) return arg_error("null argument");
  MLP_CUDA(cudaMemcpy(dist, p->dD, sizeof(int32_t) * (size_t)p->n * p->n, cudaMemcpyDeviceToHost), "copy D");
  return kOk;
}

MLP_API void mlp_problem_destroy(mlp_problem_t h) { delete reinterpret_cast<Problem*>(h); }

// ---------------------------------------------------------------- solver
MLP_API int mlp_solver_create(mlp_problem_t h, int32_t wide, mlp_solver_t* out) {
  Problem* p = reinterpret_cast<Problem*>(h);
  if (!p || !out) return arg_error("null argument");
  std::unique_ptr<mlp_solver> s(new mlp_solver());
  MLP_TRY(solver_init(s.get(), p, wide));
  *out = s.release();
  return kOk;
}

MLP_API void mlp_solver_destroy(mlp_solver_t s) {
  if (s) {
    cudaStreamSynchronize(s->set ? s->set->stream() : s->own_stream);
    delete s;
  }
}

MLP_API int mlp_solver_set_stream(mlp_solver_t s, void* stream) {
  if (!s) return arg_error("null solver");
  MLP_CUDA(cudaStreamSynchronize(s->set->stream()), "sync");
  return s->set->set_stream(stream ? static_cast<cudaStream_t>(stream) : s->own_stream);
}

MLP_API int mlp_solver_set_tile_shape(mlp_solver_t s, int32_t shape) {
  if (!s) return arg_error("null solver");
  return s->set->set_shape(shape);
}

MLP_API int mlp_solver_set_unroll(mlp_solver_t s, int32_t u) {
  if (!s) return arg_error("null solver");
  if (u == 0) {
    s->set->set_device_loop(true);
    return kOk;
  }
  s->set->set_device_loop(false);
  return s->set->set_unroll(u);
}

MLP_API int mlp_solver_set_merge_mode(mlp_solver_t s, int32_t mode) {
  if (!s) return arg_error("null solver");
  return s->set->set_merge_mode(mode);
}

MLP_API int mlp_solver_set_sweep_kernel(mlp_solver_t s, int32_t variant) {
  if (!s) return arg_error("null solver");
  return s->set->set_sweep_kernel(variant);
}

MLP_API int mlp_solver_set_total(mlp_solver_t s, int32_t on) {
  if (!s) return arg_error("null solver");
  return s->set->set_total(on != 0);
}

MLP_API int mlp_solver_set_tour(mlp_solver_t s, const int32_t* tour, int32_t len) {
  MLP_RANGE("mlp_solver_set_tour");
  if (!s) return arg_error("null solver");
  MLP_TRY(validate_tour(tour, len, s->prob->n, s->prob->size));
  MLP_CUDA(cudaMemcpyAsync(s->job->dev.tour, tour, sizeof(int32_t) * len, cudaMemcpyHostToDevice,
                           s->set->stream()),
           "copy tour");
  return s->set->prepare(true);
}

MLP_API int mlp_solver_random_tour_ties(mlp_solver_t s, uint32_t seed, float alpha, int32_t ties) {
  MLP_RANGE("mlp_solver_random_tour");
  if (!s) return arg_error("null solver");
  MLP_TRY(check_alpha(alpha));
  if (ties < 0 || ties > 1) return arg_error("ties must be 0 (client id) or 1 (the reference's sort)");
  const std::vector<GraspTask> task{GraspTask{s->prob->dD, s->job->dev.tour, s->prob->n, seed, alpha, ties, 0}};
  MLP_TRY(build_random_tours(task, s->set->stream()));
  return s->set->prepare(true);
}

MLP_API int mlp_solver_random_tour(mlp_solver_t s, uint32_t seed, float alpha) {
  return mlp_solver_random_tour_ties(s, seed, alpha, 0);
}

MLP_API int mlp_problem_random_tours_ties(mlp_problem_t h, int32_t count, const uint32_t* seeds, float alpha,
                                          int32_t ties, int32_t* tours) {
  MLP_RANGE("mlp_problem_random_tours");
  Problem* p = reinterpret_cast<Problem*>(h);
  if (!p) return arg_error("null problem");
  if (count < 0 || (count > 0 && (!seeds || !tours))) return arg_error("count must be >= 0 with seeds and tours");
  MLP_TRY(check_alpha(alpha));
  if (ties < 0 || ties > 1) return arg_error("ties must be 0 (client id) or 1 (the reference's sort)");
  if (count == 0) return kOk;
  const size_t sz = (size_t)p->size;
  struct Res {
    cudaStream_t st = nullptr;
    int32_t* d = nullptr;
    ~Res() {
      if (d) cudaFreeAsync(d, st);
      if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
      }
    }
  } r;
  MLP_CUDA(cudaStreamCreateWithFlags(&r.st, cudaStreamNonBlocking), "stream");
  MLP_CUDA(cudaMallocAsync(&r.d, sizeof(int32_t) * sz * (size_t)count, r.st), "cudaMallocAsync(tours)");
  std::vector<GraspTask> tasks;
  for (int32_t q = 0; q < count; q++)
    tasks.push_back(GraspTask{p->dD, r.d + q * sz, p->n, seeds[q], alpha, ties, 0});
  MLP_TRY(build_random_tours(tasks, r.st));
  MLP_CUDA(cudaMemcpyAsync(tours, r.d, sizeof(int32_t) * sz * (size_t)count, cudaMemcpyDeviceToHost, r.st),
           "copy tours");
  MLP_CUDA(cudaStreamSynchronize(r.st), "copy tours");
  return kOk;
}

MLP_API int mlp_problem_random_tours(mlp_problem_t h, int32_t count, const uint32_t* seeds, float alpha,
                                     int32_t* tours) {
  return mlp_problem_random_tours_ties(h, count, seeds, alpha, 0, tours);
}

MLP_API int mlp_solver_set_tour_device(mlp_solver_t s, const int32_t* tour, int32_t len) {
  if (!s || !tour) return arg_error("null argument");
  if (len != s->prob->size) return arg_error("tour length must equal size = n + 1");
  MLP_CUDA(cudaMemcpyAsync(s->job->dev.tour, tour, sizeof(int32_t) * len, cudaMemcpyDeviceToDevice,
                           s->set->stream()),
           "copy tour");
  return s->set->prepare(true);
}

MLP_API int mlp_solver_get_tour(mlp_solver_t s, int32_t* tour, int32_t len) {
  if (!s || !tour) return arg_error("null argument");
  if (len < s->prob->size) return arg_error("buffer shorter than size = n + 1");
  MLP_CUDA(cudaMemcpyAsync(tour, s->job->dev.tour, sizeof(int32_t) * s->prob->size, cudaMemcpyDeviceToHost,
                           s->set->stream()),
           "copy tour");
  MLP_CUDA(cudaStreamSynchronize(s->set->stream()), "sync");
  return kOk;
}

// Checkpoint text format of MLSolution::save / load (source/mlsolution.cpp:685-751):
// the tour length, the cost, then the tour on one line.
MLP_API int mlp_solver_save(mlp_solver_t s, const char* path) {
  if (!s || !path) return arg_error("null argument");
  std::vector<int32_t> t(s->prob->size);
  MLP_TRY(mlp_solver_get_tour(s, t.data(), (int32_t)t.size()));
  int64_t cost = 0;
  MLP_TRY(mlp_solver_cost(s, &cost));
  FILE* f = std::fopen(path, "w");
  if (!f) {
    set_error(std::string("cannot write solution file: ") + path);
    return kErrIo;
  }
  std::fprintf(f, "%d\n%lld\n", (int)t.size(), (long long)cost);
  for (size_t q = 0; q < t.size(); q++) std::fprintf(f, q + 1 < t.size() ? "%d " : "%d\n", t[q]);
  const bool ok = std::fclose(f) == 0;
  if (!ok) {
    set_error(std::string("error writing solution file: ") + path);
    return kErrIo;
  }
  return kOk;
}

MLP_API int mlp_solver_load(mlp_solver_t s, const char* path) {
  if (!s || !path) return arg_error("null argument");
  FILE* f = std::fopen(path, "r");
  if (!f) {
    set_error(std::string("cannot open solution file: ") + path);
    return kErrIo;
  }
  const int size = s->prob->size;
  long long v = 0, cost = 0;
  std::vector<int32_t> t(size);
  bool ok = std::fscanf(f, "%lld", &v) == 1;
  // Like MLSolution::load: the stored length may be size or size - 1 (a file
  // written for the other costTour setting); size entries follow the cost,
  // which is recomputed rather than trusted.
  if (ok && v != size && v != size - 1) {
    std::fclose(f);
    set_error("invalid solution file: tour length does not match the problem");
    return kErrFormat;
  }
  ok = ok && std::fscanf(f, "%lld", &cost) == 1;
  for (int q = 0; ok && q < size; q++) {
    long long x = 0;
    ok = std::fscanf(f, "%lld", &x) == 1 && x >= 0 && x < 65536;
    t[q] = (int32_t)x;
  }
  std::fclose(f);
  if (!ok) {
    set_error("invalid solution file: truncated or malformed");
    return kErrFormat;
  }
  return mlp_solver_set_tour(s, t.data(), size);
}

MLP_API int mlp_solver_tour_device(mlp_solver_t s, int32_t** tour) {
  if (!s || !tour) return arg_error("null argument");
  *tour = s->job->dev.tour;
  return kOk;
}

MLP_API int mlp_solver_cost(mlp_solver_t s, int64_t* cost) {
  if (!s || !cost) return arg_error("null argument");
  mlp_dvnd_stats_t st;
  MLP_TRY(solver_stats(s, &st, MLP_NB_ALL));
  *cost = st.cost;
  return kOk;
}

MLP_API int mlp_solver_weights(mlp_solver_t s, int32_t* w, int32_t len) {
  if (!s || !w) return arg_error("null argument");
  if (len < s->prob->size) return arg_error("buffer shorter than size");
  MLP_CUDA(cudaMemcpyAsync(w, s->job->dev.w, sizeof(int32_t) * s->prob->size, cudaMemcpyDeviceToHost,
                           s->set->stream()),
           "copy w");
  MLP_CUDA(cudaStreamSynchronize(s->set->stream()), "sync");
  return kOk;
}

MLP_API int mlp_solver_ads(mlp_solver_t s, uint32_t* ads, int64_t words) {
  MLP_RANGE("mlp_solver_ads");
  if (!s || !ads) return arg_error("null argument");
  const int sz = s->prob->size;
  const size_t need = 32 + (size_t)sz * (sz + 3);
  if ((size_t)words < need) return arg_error("ADS buffer needs 32 + size*(size+3) words");
  if (!s->dads) {
    MLP_CUDA(cudaMalloc(&s->dads, need * 4), "cudaMalloc(ads)");
    MLP_CUDA(cudaMalloc(&s->dP, (size_t)sz * 4), "cudaMalloc(ads)");
  }
  int32_t* cx = s->prob->dX;
  int32_t* cy = s->prob->dY;
  std::unique_ptr<int32_t, decltype(&cudaFree)> zeros(nullptr, &cudaFree);
  if (!cx) {
    int32_t* z = nullptr;
    MLP_CUDA(cudaMalloc(&z, sizeof(int32_t) * s->prob->n), "cudaMalloc");
    MLP_CUDA(cudaMemset(z, 0, sizeof(int32_t) * s->prob->n), "memset");
    zeros.reset(z);
    cx = cy = z;
  }
  MLP_CUDA(launch_ads(s->set->device_jobs(), cx, cy, s->dads, s->prob->cost_tour, s->prob->dist_round,
                      s->set->stream(), s->dP, sz),
           "ads kernel");
  MLP_CUDA(cudaMemcpyAsync(ads, s->dads, need * 4, cudaMemcpyDeviceToHost, s->set->stream()), "copy ads");
  MLP_CUDA(cudaStreamSynchronize(s->set->stream()), "sync");
  return kOk;
}

MLP_API int mlp_solver_num_candidates(mlp_solver_t s, int32_t nb, int32_t* count) {
  if (!s || !count) return arg_error("null argument");
  if (nb < 0 || nb >= kNumNb) return arg_error("neighbourhood out of range");
  *count = nb_blocks(nb, s->prob->size);
  return kOk;
}

MLP_API int mlp_solver_eval(mlp_solver_t s, int32_t nb, int64_t* cost, int32_t* oi, int32_t* oj) {
  MLP_RANGE("mlp_solver_eval");
  if (!s || !cost || !oi || !oj) return arg_error("null argument");
  if (nb < 0 || nb >= kNumNb) return arg_error("neighbourhood out of range");
  const int sz = s->prob->size;
  const int m = nb_blocks(nb, sz), off = nb_offset(nb, sz);
  MLP_TRY(s->set->set_mask(1 << nb));
  MLP_TRY(s->set->prepare(false));
  MLP_TRY(s->set->sweep_only());
  std::vector<uint64_t> keys(m);
  MLP_CUDA(cudaMemcpyAsync(keys.data(), s->job->dev.keys + off, sizeof(uint64_t) * m, cudaMemcpyDeviceToHost,
                           s->set->stream()),
           "copy keys");
  MLP_TRY(s->set->prepare(false));
  MLP_CUDA(cudaStreamSynchronize(s->set->stream()), "sync");
  const int64_t sentinel = s->wide ? INT64_MAX : (int64_t)kCostInfty32;
  for (int b = 0; b < m; b++) {
    if (keys[b] == kKeyNone) {
      cost[b] = sentinel;
      oi[b] = oj[b] = 0;
      continue;
    }
    int i, j;
    map_move(nb, sz, b, (int)(keys[b] & ((1u << kCtxBits) - 1)), i, j);
    cost[b] = key_cost(keys[b], kCtxBits);
    oi[b] = i;
    oj[b] = j;
  }
  return kOk;
}

static int oropt_k_check(mlp_solver_t s, int32_t k) {
  if (!s) return arg_error("null solver");
  if (k < 1 || k > kMaxOroptK) return arg_error("Or-opt k must lie in [1, 28]");
  if (oropt_blocks(k, s->prob->size) < 1) return arg_error("Or-opt k too large for this instance");
  return kOk;
}

// Per-block candidates of Or-opt-k into the job's key array (keys reset by
// the caller's prepare afterwards).
static int oropt_eval_keys(mlp_solver_t s, int32_t k) {
  MLP_TRY(s->set->prepare(false));
  MLP_CUDA(launch_oropt_eval(s->set->device_jobs(), k, s->prob->size, s->wide, s->job->dev.keys, s->set->stream()),
           "Or-opt-k kernel");
  return kOk;
}

MLP_API int mlp_solver_eval_oropt(mlp_solver_t s, int32_t k, int64_t* cost, int32_t* oi, int32_t* oj) {
  MLP_RANGE("mlp_solver_eval_oropt");
  MLP_TRY(oropt_k_check(s, k));
  if (!cost || !oi || !oj) return arg_error("null argument");
  const int sz = s->prob->size, m = oropt_blocks(k, sz);
  MLP_TRY(oropt_eval_keys(s, k));
  std::vector<uint64_t> keys(m);
  MLP_CUDA(cudaMemcpyAsync(keys.data(), s->job->dev.keys, sizeof(uint64_t) * m, cudaMemcpyDeviceToHost,
                           s->set->stream()),
           "copy keys");
  MLP_TRY(s->set->prepare(false));
  MLP_CUDA(cudaStreamSynchronize(s->set->stream()), "sync");
  const int64_t sentinel = s->wide ? INT64_MAX : (int64_t)kCostInfty32;
  for (int b = 0; b < m; b++) {
    if (keys[b] == kKeyNone) {
      cost[b] = sentinel;
      oi[b] = oj[b] = 0;
      continue;
    }
    int i, j;
    map_oropt(k, sz, b, (int)(keys[b] & ((1u << kCtxBits) - 1)), i, j);
    cost[b] = key_cost(keys[b], kCtxBits);
    oi[b] = i;
    oj[b] = j;
  }
  return kOk;
}

MLP_API int mlp_solver_pass_oropt(mlp_solver_t s, int32_t k, int32_t max_moves, int32_t* is, int32_t* js,
                                  int64_t* costs, int32_t* count, int64_t* new_cost) {
  MLP_RANGE("mlp_solver_pass_oropt");
  MLP_TRY(oropt_k_check(s, k));
  if (max_moves > 0 && (!is || !js || !costs)) return arg_error("null move arrays");
  const int sz = s->prob->size, m = oropt_blocks(k, sz);
  struct Scratch {  // stream-ordered: no device-wide synchronisation
    cudaStream_t st;
    uint8_t* p = nullptr;
    ~Scratch() {
      if (p) cudaFreeAsync(p, st);
    }
  } sc{s->set->stream()};
  const size_t body = oropt_pass_scratch_bytes(sz, k);
  const size_t o_ij = (body + 255) / 256 * 256, o_cost = o_ij + ((size_t)m * 4 + 255) / 256 * 256;
  const size_t o_cnt = o_cost + (size_t)m * 8, bytes = o_cnt + 256;
  MLP_CUDA(cudaMallocAsync(&sc.p, bytes, s->set->stream()), "cudaMallocAsync(Or-opt-k pass)");
  MLP_TRY(oropt_eval_keys(s, k));
  uint32_t* dij = (uint32_t*)(sc.p + o_ij);
  int64_t* dcost = (int64_t*)(sc.p + o_cost);
  int* dcnt = (int*)(sc.p + o_cnt);
  MLP_CUDA(launch_oropt_pass(s->set->device_jobs(), k, s->wide, s->job->dev.keys, sc.p, dij, dcost, dcnt,
                             s->set->stream()),
           "Or-opt-k pass kernel");
  MLP_TRY(s->set->prepare(false));  // w, prefix arrays and cost of the new tour; keys reset
  int applied = 0;
  MLP_CUDA(cudaMemcpyAsync(&applied, dcnt, sizeof(int), cudaMemcpyDeviceToHost, s->set->stream()), "copy count");
  MLP_CUDA(cudaStreamSynchronize(s->set->stream()), "sync");
  const int take = std::min(applied, std::max(0, (int)max_moves));
  if (take > 0) {
    std::vector<uint32_t> mv(take);
    MLP_CUDA(cudaMemcpyAsync(mv.data(), dij, 4 * take, cudaMemcpyDeviceToHost, s->set->stream()), "copy moves");
    MLP_CUDA(cudaMemcpyAsync(costs, dcost, 8 * take, cudaMemcpyDeviceToHost, s->set->stream()), "copy moves");
    MLP_CUDA(cudaStreamSynchronize(s->set->stream()), "sync");
    for (int q = 0; q < take; q++) {
      is[q] = (int32_t)(mv[q] & 0x3fff);
      js[q] = (int32_t)(mv[q] >> 14);
    }
  }
  if (count) *count = applied;
  if (new_cost) MLP_TRY(mlp_solver_cost(s, new_cost));
  return kOk;
}

MLP_API int mlp_solver_pass(mlp_solver_t s, int32_t nb, int32_t max_moves, int32_t* ids, int32_t* is,
                            int32_t* js, int64_t* costs, int32_t* count, int64_t* new_cost) {
  MLP_RANGE("mlp_solver_pass");
  if (!s) return arg_error("null solver");
  if (nb < 0 || nb >= kNumNb) return arg_error("neighbourhood out of range");
  if (max_moves > 0 && (!ids || !is || !js || !costs)) return arg_error("null move arrays");
  MLP_TRY(s->set->set_mask(1 << nb));
  MLP_TRY(s->set->set_record_moves(true));
  const int rs = s->set->run(1, true);
  MLP_TRY(s->set->set_record_moves(false));
  MLP_TRY(rs);
  mlp_dvnd_stats_t st;
  std::vector<std::array<int64_t, kStatWords>> raw;
  MLP_TRY(s->set->read_stats(&raw));
  MLP_TRY(solver_stats(s, &st, 1 << nb));
  const int applied = (int)raw[0][kStatLastMoves];
  const int take = std::min(std::min(applied, (int)std::max(0, max_moves)), s->job->moves_cap);
  if (take > 0) {
    std::vector<uint32_t> mv(take);
    std::vector<int64_t> mc(take);
    MLP_CUDA(cudaMemcpyAsync(mv.data(), s->job->dev.moves_out, 4 * take, cudaMemcpyDeviceToHost,
                             s->set->stream()),
             "copy moves");
    MLP_CUDA(cudaMemcpyAsync(mc.data(), s->job->dev.moves_cost, 8 * take, cudaMemcpyDeviceToHost,
                             s->set->stream()),
             "copy moves");
    MLP_CUDA(cudaStreamSynchronize(s->set->stream()), "sync");
    for (int q = 0; q < take; q++) {
      ids[q] = (int32_t)(mv[q] & 0xf);
      is[q] = (int32_t)((mv[q] >> 4) & 0x3fff);
      js[q] = (int32_t)(mv[q] >> 18);
      costs[q] = mc[q];
    }
  }
  if (count) *count = applied;
  if (new_cost) *new_cost = st.cost;
  return kOk;
}

MLP_API int mlp_solver_dvnd(mlp_solver_t s, int32_t nb_mask, int32_t max_iters, mlp_dvnd_stats_t* stats) {
  MLP_RANGE("mlp_solver_dvnd");
  if (!s) return arg_error("null solver");
  MLP_TRY(s->set->set_mask(nb_mask));
  MLP_TRY(s->set->run(max_iters, true));
  return solver_stats(s, stats, nb_mask);
}

MLP_API int mlp_solver_dvnd_async(mlp_solver_t s, int32_t nb_mask, int32_t max_iters) {
  MLP_RANGE("mlp_solver_dvnd_async");
  if (!s) return arg_error("null solver");
  MLP_TRY(s->set->set_mask(nb_mask));
  return s->set->enqueue_device_loop(max_iters);
}

MLP_API int mlp_solver_begin(mlp_solver_t s, int32_t nb_mask, int32_t max_iters) {
  if (!s) return arg_error("null solver");
  if (max_iters <= 0) return arg_error("max_iters must be positive");
  MLP_TRY(s->set->set_mask(nb_mask));
  MLP_CUDA(launch_stats_begin(s->set->device_jobs(), 1, max_iters, s->set->stream()), "stats kernel");
  return kOk;
}

MLP_API int mlp_solver_enqueue(mlp_solver_t s, int32_t iterations) {
  MLP_RANGE("mlp_solver_enqueue");
  if (!s) return arg_error("null solver");
  if (iterations <= 0) return arg_error("iterations must be positive");
  return s->set->enqueue_iterations(iterations);
}

MLP_API int mlp_solver_stats(mlp_solver_t s, mlp_dvnd_stats_t* stats) {
  if (!s || !stats) return arg_error("null argument");
  return solver_stats(s, stats, s->job->dev.nb_mask);
}

MLP_API int mlp_solver_sweep(mlp_solver_t s, int32_t nb_mask, int32_t repeats, int64_t* evals_per_sweep) {
  MLP_RANGE("mlp_solver_sweep");
  if (!s) return arg_error("null solver");
  if (repeats < 0) return arg_error("repeats must be >= 0");
  MLP_TRY(s->set->set_mask(nb_mask));
  MLP_CUDA(launch_stats_begin(s->set->device_jobs(), 1, 1, s->set->stream()), "stats kernel");
  for (int r = 0; r < repeats; r++) MLP_TRY(s->set->sweep_kernel());
  MLP_TRY(s->set->prepare(false));
  if (evals_per_sweep) *evals_per_sweep = s->set->evals_per_sweep(0, nb_mask);
  return kOk;
}

MLP_API int mlp_tuning_set(const int32_t* max_size, const int32_t* shape_one, const int32_t* shape_many,
                           int32_t count) {
  return tuning_set(max_size, shape_one, shape_many, count);
}

MLP_API int mlp_tuning_get(int32_t* max_size, int32_t* shape_one, int32_t* shape_many, int32_t cap,
                           int32_t* count) {
  int c = 0;
  const int st = tuning_get(max_size, shape_one, shape_many, cap, &c);
  if (count) *count = c;
  return st;
}

MLP_API int mlp_tuning_load(const char* path) { return tuning_load(path); }

MLP_API int mlp_solver_autotune(mlp_solver_t s, int32_t* shape) {
  if (!s) return arg_error("null solver");
  cudaStream_t st = s->set->stream();
  cudaEvent_t a, b;
  MLP_CUDA(cudaEventCreate(&a), "event");
  MLP_CUDA(cudaEventCreate(&b), "event");
  const int old_mask = s->job->dev.nb_mask;
  MLP_TRY(s->set->set_mask(MLP_NB_ALL));
  float best = 1e30f;
  int best_shape = s->set->shape();
  for (int sh = 0; sh < kNumTileShapes; sh++) {
    MLP_TRY(s->set->set_shape(sh));
    MLP_CUDA(launch_stats_begin(s->set->device_jobs(), 1, 1, st), "stats kernel");
    for (int r = 0; r < 3; r++) MLP_TRY(s->set->sweep_kernel());
    MLP_CUDA(cudaEventRecord(a, st), "event");
    for (int r = 0; r < 20; r++) MLP_TRY(s->set->sweep_kernel());
    MLP_CUDA(cudaEventRecord(b, st), "event");
    MLP_CUDA(cudaEventSynchronize(b), "event");
    float ms = 0;
    MLP_CUDA(cudaEventElapsedTime(&ms, a, b), "event");
    if (ms < best) {
      best = ms;
      best_shape = sh;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  MLP_TRY(s->set->set_shape(best_shape));
  MLP_TRY(s->set->prepare(false));
  MLP_TRY(s->set->set_mask(old_mask));
  MLP_CUDA(cudaStreamSynchronize(st), "sync");
  if (shape) *shape = best_shape;
  return kOk;
}

MLP_API int mlp_solver_time_sweep(mlp_solver_t s, int32_t nb_mask, int32_t repeats, void* flush, int64_t flush_bytes,
                                  float* ms) {
  MLP_RANGE("mlp_solver_time_sweep");
  if (!s || !ms) return arg_error("null argument");
  if (repeats <= 0 || repeats > 4096) return arg_error("repeats must be in 1 .. 4096");
  if (flush != nullptr && flush_bytes <= 0) return arg_error("flush_bytes must be positive");
  cudaStream_t st = s->set->stream();
  MLP_TRY(s->set->set_mask(nb_mask));
  MLP_CUDA(launch_stats_begin(s->set->device_jobs(), 1, 1, st), "stats kernel");
  for (int r = 0; r < 3; r++) MLP_TRY(s->set->sweep_kernel());
  std::vector<cudaEvent_t> ev;
  int rc = kOk;
  for (int q = 0; rc == kOk && q < 2 * repeats; q++) {
    cudaEvent_t e = nullptr;
    rc = cuda_status(cudaEventCreate(&e), "event");
    if (rc == kOk) ev.push_back(e);
  }
  std::vector<float> t;
  if (flush != nullptr) {
    // Cold: every launch after the flush, between its own two events.
    for (int r = 0; rc == kOk && r < repeats; r++) {
      rc = cuda_status(cudaMemsetAsync(flush, r & 0xff, (size_t)flush_bytes, st), "L2 flush");
      if (rc == kOk) rc = cuda_status(cudaEventRecord(ev[2 * r], st), "event");
      if (rc == kOk) rc = s->set->sweep_kernel();
      if (rc == kOk) rc = cuda_status(cudaEventRecord(ev[2 * r + 1], st), "event");
    }
    if (rc == kOk) rc = cuda_status(cudaStreamSynchronize(st), "sync");
    for (int r = 0; rc == kOk && r < repeats; r++) {
      float x = 0;
      rc = cuda_status(cudaEventElapsedTime(&x, ev[2 * r], ev[2 * r + 1]), "event");
      t.push_back(x);
    }
  } else {
    // Warm: the launches back to back between two events (each launch's
    // set-up overlaps the previous one's run, as in a DVND), per launch.
    rc = cuda_status(cudaEventRecord(ev[0], st), "event");
    for (int r = 0; rc == kOk && r < repeats; r++) rc = s->set->sweep_kernel();
    if (rc == kOk) rc = cuda_status(cudaEventRecord(ev[1], st), "event");
    if (rc == kOk) rc = cuda_status(cudaStreamSynchronize(st), "sync");
    float x = 0;
    if (rc == kOk) rc = cuda_status(cudaEventElapsedTime(&x, ev[0], ev[1]), "event");
    t.push_back(x / (float)repeats);
  }
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  MLP_TRY(rc);
  std::sort(t.begin(), t.end());
  *ms = t[t.size() / 2];
  MLP_TRY(s->set->prepare(false));
  MLP_CUDA(cudaStreamSynchronize(st), "sync");
  return kOk;
}

// ---------------------------------------------------------------- batch
MLP_API int mlp_batch_create(int32_t wide, mlp_batch_t* out) {
  if (!out) return arg_error("null output handle");
  mlp_batch* b = new mlp_batch();
  b->wide = wide != 0;
  cudaError_t e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete b;
    return cuda_status(e, "cudaStreamCreate");
  }
  b->stream = b->own_stream;
  *out = b;
  return kOk;
}

MLP_API void mlp_batch_destroy(mlp_batch_t b) {
  if (!b) return;
  cudaStreamSynchronize(b->stream);
  delete b;
}

mlp_batch::~mlp_batch() {
  set.reset();
  jobs.clear();
  if (own_stream) cudaStreamDestroy(own_stream);
}

MLP_API int mlp_batch_set_stream(mlp_batch_t b, void* stream) {
  if (!b) return arg_error("null batch");
  b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
  if (b->set) return b->set->set_stream(b->stream);
  return kOk;
}

MLP_API int mlp_batch_set_tile_shape(mlp_batch_t b, int32_t shape) {
  if (!b) return arg_error("null batch");
  if (shape < -1 || shape >= kNumTileShapes) return arg_error("tile shape out of range");
  b->shape = shape;
  if (b->set && shape >= 0) return b->set->set_shape(shape);
  return kOk;
}

MLP_API int mlp_batch_set_check_interval(mlp_batch_t b, int32_t iterations) {
  if (!b) return arg_error("null batch");
  if (iterations < 1 || iterations > 256) return arg_error("check interval must lie in [1, 256]");
  b->check_interval = iterations;
  if (b->set) return b->set->set_unroll(iterations);
  return kOk;
}

MLP_API int mlp_batch_set_merge_mode(mlp_batch_t b, int32_t mode) {
  if (!b) return arg_error("null batch");
  if (mode < kMergeAuto || mode > kMergeSolo) return arg_error("merge mode must be 0, 1 or 2");
  b->merge_mode = mode;
  if (b->set) return b->set->set_merge_mode(mode);
  return kOk;
}

MLP_API int mlp_batch_set_sweep_kernel(mlp_batch_t b, int32_t variant) {
  if (!b) return arg_error("null batch");
  if (variant < 0 || variant > 1) return arg_error("sweep kernel must be 0 or 1");
  b->sweep_kernel = variant;
  if (b->set) return b->set->set_sweep_kernel(variant);
  return kOk;
}

MLP_API int mlp_batch_set_total(mlp_batch_t b, int32_t on) {
  if (!b) return arg_error("null batch");
  b->total = on != 0;
  if (b->set) return b->set->set_total(b->total);
  return kOk;
}

MLP_API int mlp_batch_add(mlp_batch_t b, mlp_problem_t h, const int32_t* tour, int32_t len, int32_t* job) {
  Problem* p = reinterpret_cast<Problem*>(h);
  if (!b || !p) return arg_error("null argument");
  MLP_TRY(validate_tour(tour, len, p->n, p->size));
  Job* j = nullptr;
  MLP_TRY(job_create(p, b->wide, 0, &j));
  b->jobs.emplace_back(j);
  b->tours.emplace_back(tour, tour + len);
  b->random_start.emplace_back();
  b->set.reset();
  if (job) *job = (int32_t)b->jobs.size() - 1;
  return kOk;
}

MLP_API int mlp_batch_add_random_ties(mlp_batch_t b, mlp_problem_t h, uint32_t seed, float alpha, int32_t ties,
                                      int32_t* job) {
  Problem* p = reinterpret_cast<Problem*>(h);
  if (!b || !p) return arg_error("null argument");
  MLP_TRY(check_alpha(alpha));
  if (ties < 0 || ties > 1) return arg_error("ties must be 0 (client id) or 1 (the reference's sort)");
  Job* j = nullptr;
  MLP_TRY(job_create(p, b->wide, 0, &j));
  b->jobs.emplace_back(j);
  b->tours.emplace_back();
  mlp_batch::RandomStart rs;
  rs.seed = seed;
  rs.alpha = alpha;
  rs.ties = ties;
  b->random_start.push_back(rs);
  b->set.reset();
  if (job) *job = (int32_t)b->jobs.size() - 1;
  return kOk;
}

MLP_API int mlp_batch_add_random(mlp_batch_t b, mlp_problem_t h, uint32_t seed, float alpha, int32_t* job) {
  return mlp_batch_add_random_ties(b, h, seed, alpha, 0, job);
}

static int batch_upload(mlp_batch* b) {
  std::vector<GraspTask> tasks;
  for (size_t q = 0; q < b->jobs.size(); q++) {
    Job* j = b->jobs[q].get();
    if (b->tours[q].empty()) {
      const mlp_batch::RandomStart& rs = b->random_start[q];
      tasks.push_back(GraspTask{j->prob->dD, j->dev.tour, j->prob->n, rs.seed, rs.alpha, rs.ties, 0});
      continue;
    }
    MLP_CUDA(cudaMemcpyAsync(j->dev.tour, b->tours[q].data(), sizeof(int32_t) * b->tours[q].size(),
                             cudaMemcpyHostToDevice, b->stream),
             "copy tour");
  }
  MLP_TRY(build_random_tours(tasks, b->stream));
  return b->set->prepare(true);
}

static int batch_build(mlp_batch* b) {
  if (b->set) return kOk;
  if (b->jobs.empty()) return arg_error("empty batch");
  std::vector<Job*> js;
  for (auto& j : b->jobs) js.push_back(j.get());
  b->set.reset(new JobSet(js, b->wide, b->stream));
  if (b->shape >= 0) MLP_TRY(b->set->set_shape(b->shape));
  MLP_TRY(b->set->set_merge_mode(b->merge_mode));
  MLP_TRY(b->set->set_sweep_kernel(b->sweep_kernel));
  MLP_TRY(b->set->set_unroll(b->check_interval));
  MLP_TRY(b->set->init());
  MLP_TRY(b->set->set_total(b->total));
  return batch_upload(b);
}

MLP_API int mlp_batch_reset(mlp_batch_t b) {
  if (!b) return arg_error("null batch");
  if (!b->set) return batch_build(b);
  return batch_upload(b);
}

MLP_API int mlp_batch_run(mlp_batch_t b, int32_t nb_mask, int32_t max_iters) {
  MLP_RANGE("mlp_batch_run");
  if (!b) return arg_error("null batch");
  MLP_TRY(batch_build(b));
  MLP_TRY(b->set->set_mask(nb_mask));
  b->mask = nb_mask;
  return b->set->run(max_iters, true);
}

MLP_API int mlp_batch_run_async(mlp_batch_t b, int32_t nb_mask, int32_t max_iters) {
  MLP_RANGE("mlp_batch_run_async");
  if (!b) return arg_error("null batch");
  MLP_TRY(batch_build(b));
  MLP_TRY(b->set->set_mask(nb_mask));
  b->mask = nb_mask;
  return b->set->enqueue_device_loop(max_iters);
}

MLP_API int mlp_batch_result(mlp_batch_t b, int32_t job, int32_t* tour, int32_t len, mlp_dvnd_stats_t* stats) {
  if (!b) return arg_error("null batch");
  if (job < 0 || job >= (int)b->jobs.size()) return arg_error("job index out of range");
  MLP_TRY(batch_build(b));
  Job* j = b->jobs[job].get();
  if (tour) {
    if (len < j->size) return arg_error("buffer shorter than size");
    MLP_CUDA(cudaMemcpyAsync(tour, j->dev.tour, sizeof(int32_t) * j->size, cudaMemcpyDeviceToHost, b->stream),
             "copy tour");
  }
  if (stats) {
    std::vector<std::array<int64_t, kStatWords>> st;
    MLP_TRY(b->set->read_stats(&st));
    std::memset(stats, 0, sizeof(*stats));
    stats->cost = st[job][kStatCost];
    stats->iterations = st[job][kStatIters];
    stats->sweeps = st[job][kStatSweeps];
    stats->moves = st[job][kStatMoves];
    stats->evals = st[job][kStatSweeps] * b->set->evals_per_sweep(job, b->mask);
    stats->converged = (int32_t)st[job][kStatConverged];
  }
  MLP_CUDA(cudaStreamSynchronize(b->stream), "sync");
  return kOk;
}

}  // extern "C"
