// mlp_engine.h -- host side of the GB300 MLP local-search engine (internal C++).
//
// The reference's task objects map onto this engine as follows:
//   MLProblem   (source/mlproblem.h:61-151)   -> mlp::Problem: n x n int32 distance
//               matrix resident in HBM, built on the device from coordinates or
//               uploaded from the host.
//   MLSolution  (source/mlsolution.h:62-434)  -> the tour + ADS prefix arrays of a Job.
//   MLKernel*   (source/mlkernel.h:104-318)   -> mlp::JobSet: the fused sweep over the
//               five neighbourhoods, the device merge/apply and the ADS rebuild,
//               launched on one stream and captured into CUDA graphs.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "mlp_common.cuh"
#include "mlp_kernels.cuh"

namespace mlp {

// Status codes of the C-ABI (mirrored in include/mlp_gpu.h).
enum Status : int {
  kOk = 0,
  kErrArg = 1,
  kErrCuda = 2,
  kErrRange = 3,
  kErrIo = 4,
  kErrFormat = 5,
  kErrNoMem = 6,
  kErrState = 7,
  kErrUnsupported = 8,
};

void set_error(const std::string& msg);
const char* last_error();
int cuda_status(cudaError_t e, const char* what);

struct Problem {
  int n = 0;
  int size = 0;
  int cost_tour = 1;
  int dist_round = 0;
  int device = 0;
  int32_t dmax = 0;
  int32_t* dD = nullptr;  // n x n
  int32_t* dX = nullptr;  // node coordinates (optional)
  int32_t* dY = nullptr;
  std::vector<int32_t> hx, hy;
  std::string name;
  cudaStream_t alloc_stream = nullptr;  // non-null: stream-ordered allocation
  bool async_alloc = false;
  ~Problem();
};

int problem_from_coords(int n, const int32_t* x, const int32_t* y, int cost_tour, int dist_round,
                        bool x_on_device, Problem** out);
// Same with stream-ordered allocation from `pool` and no host
// synchronisation (the coordinates are staged before the call returns).
int problem_from_coords_async(int n, const int32_t* x, const int32_t* y, int dist_round, cudaMemPool_t pool,
                              cudaStream_t stream, Problem** out);
int problem_from_matrix(int n, const int32_t* D, int cost_tour, bool on_device, Problem** out);
int problem_from_tsplib(const char* path, int cost_tour, int dist_round, Problem** out);
// TSPLIB EUC_2D reader (coordinates rounded with TSPLIB nint, source/tsplib.cpp:237-240).
int read_tsplib_euc2d(const char* path, std::vector<int32_t>& x, std::vector<int32_t>& y,
                      std::string& name);

// One local-search job: a problem plus its device-resident tour and ADS arrays.
struct Job {
  Problem* prob = nullptr;
  bool wide = false;
  int size = 0;
  void* arena = nullptr;  // single device allocation holding every array
  size_t arena_bytes = 0;
  JobDev dev{};           // host copy of the descriptor
  int moves_cap = 0;
  cudaStream_t alloc_stream = nullptr;
  bool async_alloc = false;
  void* total = nullptr;  // TOTAL lists (allocated when a job set first enters TOTAL mode)
  size_t total_bytes = 0;
  int32_t* rt_mem = nullptr;  // the arena's term tables (32-bit jobs); dev.RT/CT point
  int32_t* ct_mem = nullptr;  // at them unless the job's set computes terms per tile
  ~Job();
};

int job_create(Problem* p, bool wide, int moves_cap, Job** out);
// Stream-ordered variant (memory from `pool`).
int job_create_async(Problem* p, bool wide, cudaMemPool_t pool, cudaStream_t stream, Job** out);
// Per-job sweep tiles of one tile shape (job index 0).
void job_tiles(int size, int shape, std::vector<SweepTile>* out);
size_t job_bytes(int size, bool wide, int moves_cap);
// Device bytes of a job's TOTAL lists (every improving move of each
// neighbourhood, the per-neighbourhood greedy output and counters).
size_t job_total_bytes(int size, bool wide);
// Allocates the TOTAL lists once and points the descriptor at them.
int job_enable_total(Job* j);

enum MergeMode : int { kMergeAuto = 0, kMergeCluster = 1, kMergeSolo = 2 };
constexpr int kSoloMinJobs = 16;

struct DvndResult {
  int64_t cost = 0;
  int64_t iterations = 0;   // iterations that applied moves
  int64_t sweeps = 0;       // neighbourhood sweeps run
  int64_t moves = 0;        // moves applied
  int64_t evals = 0;        // move evaluations
  int converged = 0;
};

// A set of jobs processed by the same launches (one job for the plain form,
// many for the batched form).
class JobSet {
 public:
  JobSet(std::vector<Job*> jobs, bool wide, cudaStream_t stream);
  ~JobSet();
  int init();
  int set_stream(cudaStream_t s);
  cudaStream_t stream() const { return stream_; }
  int set_shape(int shape);
  int shape() const { return shape_; }
  int set_unroll(int u);
  // true (the default): a one-search set on a stream loops on the device
  // (graph while node); false: the host checks convergence after every
  // `unroll` graph-replayed iterations.  A batch always checks on the host,
  // every `unroll` iterations, one check late (converged jobs then leave the
  // launches).
  void set_device_loop(bool on) { device_loop_ = on; }
  // Rebuild the ADS arrays and reset statistics (after new tours).
  int prepare(bool reset_stats);
  // Set the neighbourhood mask of every job (bit nb = neighbourhood nb).
  int set_mask(int mask);
  // Record the applied moves of each iteration (for the legacy move vectors).
  int set_record_moves(bool on);
  // One sweep only (keys left on the device; call prepare() afterwards).
  int sweep_only();
  // The sweep kernel of a DVND iteration alone (improving candidates only;
  // after a statistics reset).
  int sweep_kernel();
  // DVND iterations until every job converged or max_iters sweeps ran.
  int run(int max_iters, bool sync);
  // Enqueue `iters` iterations without host synchronisation (graph replay).
  int enqueue_iterations(int iters);
  // Enqueue a whole DVND (at most max_iters sweeps per job) as one CUDA graph
  // whose while-node loops on the device until every job converged; no host
  // synchronisation.  Read the results with read_stats().
  int enqueue_device_loop(int max_iters);
  int read_stats(std::vector<std::array<int64_t, kStatWords>>* out);
  int64_t evals_per_sweep(int job, int mask) const;
  const std::vector<Job*>& jobs() const { return all_jobs_; }
  // Launch only the listed jobs (indices into jobs()); converged jobs are
  // dropped this way between graph replays of a batch.
  // sync = false: the copies of the new job and tile arrays are left in the
  // stream, staged in pinned buffer `buf` (0 or 1), which must not be staged
  // into again before work enqueued after them has completed.
  int set_active(const std::vector<int>& idx, int buf = 0, bool sync = true);
  int ensure_all_active();
  JobDev* device_jobs() const { return djobs_; }
  int ntiles() const { return ntiles_; }
  // One DVND iteration over the current jobs (no statistics reset).
  int launch_iteration();
  // Merge kernel: kMergeAuto (one CTA per job for sets of kSoloMinJobs jobs
  // or more, a six-CTA cluster per job otherwise), kMergeCluster, kMergeSolo.
  int set_merge_mode(int mode);
  bool solo_merge() const;
  // TOTAL candidate mode: every move the sweep evaluates is a merge
  // candidate (the reference's isTotal kernels), not only each block's best.
  int set_total(bool on);
  bool total() const { return total_; }
  // DVND sweep kernel: 1 (default) the term-table kernel for 32-bit job sets
  // that evaluate all five neighbourhoods (k_sweep_dvnd), 0 the general
  // kernel everywhere.  Both give identical candidates.
  int set_sweep_kernel(int variant);
  int sweep_kernel_variant() const { return sweep_variant_; }

 private:
  int build_tiles(int buf = 0, bool sync = true);
  int check_stats(const int64_t* hst);  // the statistics' internal error words
  void drop_graphs();
  bool dvnd_sweep() const { return sweep_variant_ == 1 && !wide_ && mask_ == 0x1f; }
  // A set of one search computes the DVND sweep's row and column terms in
  // every tile instead of having the ADS rebuild (one CTA, on the merge's
  // critical path) write term tables.
  bool local_terms() const { return all_jobs_.size() == 1; }
  int graph_for(int iters, cudaGraphExec_t* out);
  std::vector<Job*> all_jobs_;  // every job of the set (statistics order)
  std::vector<Job*> jobs_;      // the jobs the launches cover
  bool wide_;
  cudaStream_t stream_;
  int shape_ = -1;
  int unroll_ = 16;  // iterations between host checks (a batch's check interval)
  bool device_loop_ = true;  // a one-search set on a stream loops on the device
  int mask_ = 0x1f;
  int max_size_ = 0;
  bool merge_smem_ = true;
  bool solo_smem_ = true;
  int merge_mode_ = 0;
  bool total_ = false;
  int sweep_variant_ = 1;
  int shape_user_ = -1;  // tile shape to restore when TOTAL mode ends
  JobDev* djobs_ = nullptr;
  SweepTile* dtiles_ = nullptr;
  int ntiles_ = 0;
  int64_t* hstats_ = nullptr;  // pinned, kStatWords per job
  int64_t* hstats2_ = nullptr;  // a second one (the batch loop reads one while the other fills)
  cudaEvent_t stats_ev_[2] = {nullptr, nullptr};
  size_t tiles_cap_ = 0;                        // tiles dtiles_ and each staging buffer hold
  SweepTile* htiles_[2] = {nullptr, nullptr};  // pinned staging of the tile list
  JobDev* hjobs_[2] = {nullptr, nullptr};      // pinned staging of the job descriptors
  int64_t* dstats_ = nullptr;  // device, kStatWords per job (jobs' stats live here)
  std::vector<void*> extra_ws_;  // merge workspaces allocated for jobs of mixed-size sets
  std::map<int, cudaGraphExec_t> graphs_;
  cudaGraphExec_t loop_graph_ = nullptr;
  int loop_unroll_ = 0;
};

// Start tours of MLSolution::random built on the device (mlp_grasp.cu), one
// per task, written to the tasks' device tours; waits for the stream and
// reports a failed internal check.
int build_random_tours(const std::vector<GraspTask>& tasks, cudaStream_t stream);
// alpha of the constructor must lie in [0, 1].
int check_alpha(float alpha);

// Sweep tile shape for a job set whose largest tour has `size` positions:
// the autotuner's table when one is set, else a built-in rule.
int default_shape(int size, int njobs);
constexpr int kManyJobs = 8;  // job sets this large use the "many jobs" shape
int tuning_set(const int32_t* max_size, const int32_t* one, const int32_t* many, int count);
int tuning_get(int32_t* max_size, int32_t* one, int32_t* many, int cap, int* count);
int tuning_load(const char* path);

}  // namespace mlp
