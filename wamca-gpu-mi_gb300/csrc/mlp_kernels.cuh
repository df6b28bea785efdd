// mlp_kernels.cuh -- launch entry points of the engine's CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include "mlp_common.cuh"

namespace mlp {

// Sweep tile shapes (diagonals x rows) compiled into the library.  per = 2:
// the DVND sweep gives each thread two adjacent diagonals (k_sweep_dvnd2);
// every other sweep kernel runs such a shape with one diagonal per thread.
struct TileShape {
  int tl;   // diagonals per tile
  int tr;   // rows per tile
  int per;  // diagonals per thread of the DVND sweep
};
constexpr TileShape kTileShapes[] = {{32, 4, 1},  {32, 8, 1},  {32, 16, 1}, {64, 4, 1},  {64, 8, 1},
                                       {64, 16, 1}, {128, 8, 1}, {128, 16, 1}, {32, 32, 1}, {64, 32, 1},
                                       {64, 8, 2},  {64, 16, 2}, {64, 32, 2},  {128, 16, 2}};
constexpr int kNumTileShapes = sizeof(kTileShapes) / sizeof(kTileShapes[0]);

// Launches `kernel` with programmatic stream serialization on a created
// stream (an ordinary launch on the legacy default stream): it may start
// while its predecessor runs, once that predecessor calls
// pdl_launch_dependents, and must call pdl_wait before it reads anything the
// predecessor writes.  In a captured graph the dependency becomes a
// programmatic edge.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = s != 0 ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// Bytes of dynamic shared memory the merge kernel needs for `size`
// (0 if the job must use its global workspace instead).
size_t merge_smem_bytes(int size);
// Bytes of global workspace a job of `size` needs when the merge cannot run
// from shared memory.
size_t merge_ws_bytes(int size);
// Largest size whose merge workspace fits in shared memory.
int merge_smem_max_size();
// The same for the one-CTA-per-job merge (launch_merge_solo).
size_t solo_smem_bytes(int size);
int solo_smem_max_size();
// A job of `size` needs a global merge workspace (some merge kernel cannot
// run it from shared memory).
inline bool merge_needs_ws(int size) {
  return size > merge_smem_max_size() || size > solo_smem_max_size();
}

// Opt the merge kernels into `bytes` of dynamic shared memory (call before
// launching or capturing merges that use shared memory).
cudaError_t configure_merge(size_t bytes);
// Sets the CUDA-graph while-condition: 1 while some job is neither converged
// nor at its sweep limit (the device-side DVND loop).
cudaError_t launch_loop_condition(const JobDev* jobs, int njobs, cudaGraphConditionalHandle h,
                                  cudaStream_t s);
// Opt the ADS-rebuild kernel alone into its dynamic shared memory.
cudaError_t configure_prepare();
// Zero the run counters of every job and set its sweep limit.
cudaError_t launch_stats_begin(const JobDev* jobs, int njobs, int64_t limit, cudaStream_t s);
cudaError_t launch_prepare(const JobDev* jobs, int njobs, bool wide, bool reset_stats,
                           cudaStream_t s);
// improve_only: publish only improving candidates (DVND iterations; the
// merge ignores the others); false publishes every block's best (evaluation).
cudaError_t launch_sweep(const SweepTile* tiles, int ntiles, const JobDev* jobs, bool wide,
                         int shape, bool improve_only, cudaStream_t s);
// One six-CTA cluster per job (latency: a single job or a few).
cudaError_t launch_merge(const JobDev* jobs, int njobs, bool wide, bool use_smem, int max_size,
                         cudaStream_t s);
// One CTA per job (throughput: sets of many jobs).  Identical results.
cudaError_t launch_merge_solo(const JobDev* jobs, int njobs, bool wide, bool use_smem, int max_size,
                              cudaStream_t s);
// TOTAL candidate mode (every evaluated move is a merge candidate).
// The collecting sweep appends each job's improving moves to its TOTAL lists
// (compiled for the tile shapes total_shape() picks); the TOTAL greedy selects
// per neighbourhood (mlp_total.cu); the finish runs the cross-neighbourhood
// greedy, apply and ADS rebuild (one CTA per job, the k_merge_solo workspace).
constexpr int kTotalShapeSmall = 3;  // 64 diagonals x 4 rows: sets whose tours have <= 2000 positions
constexpr int kTotalShapeLarge = 7;  // 128 diagonals x 16 rows
inline int total_shape(int max_size) { return max_size <= 2000 ? kTotalShapeSmall : kTotalShapeLarge; }
// DVND sweep of 32-bit jobs over all five neighbourhoods (mlp_sweep.cu): the
// same keys as launch_sweep with improve_only for jobs whose mask is all five
// neighbourhoods.  local = false: the terms come from the jobs' term tables
// (written by the ADS rebuild); local = true: every tile computes its own from
// the prefix arrays (jobs whose descriptors carry no tables).
cudaError_t launch_sweep_dvnd(const SweepTile* tiles, int ntiles, const JobDev* jobs, int shape, bool local,
                              cudaStream_t s);
cudaError_t launch_sweep_collect(const SweepTile* tiles, int ntiles, const JobDev* jobs, bool wide, int shape,
                                 cudaStream_t s);
cudaError_t launch_total_select(const JobDev* jobs, int njobs, bool wide, cudaStream_t s);
cudaError_t launch_total_finish(const JobDev* jobs, int njobs, bool wide, bool use_smem, int max_size,
                                cudaStream_t s);
// Opt the TOTAL greedy into its dynamic shared memory (configure_merge calls it).
cudaError_t configure_total();
// MLSolution::random on the device (mlp_grasp.cu): one start per task, its
// n + 1 entries written to `tour` (device), MTRandom seeded with `seed`;
// alpha in [0, 1].  ties = 0: equal distances ordered by client id (one warp
// per start, a rank selection per step); ties = 1: the reference's own order,
// its std::sort of the persistent candidate array restated step for step
// (mlp_refsort.cuh; one warp per start, the sort on one lane).  *err (device)
// counts starts that failed an internal check (none expected).
struct GraspTask {
  const int32_t* D;  // n x n distances
  int32_t* tour;     // n + 1 entries
  int32_t n;
  uint32_t seed;
  float alpha;
  int32_t ties;
  int64_t scratch;   // ties = 1 and n > kGraspRefSmemN: word offset of 2n words in the scratch buffer
};
constexpr int kGraspRefSmemN = 2048;  // ties = 1: up to this n the candidate arrays stay in shared memory
cudaError_t configure_grasp();
// tasks holds `count` tasks of one ties mode; scratch: see GraspTask::scratch.
cudaError_t launch_grasp(const GraspTask* tasks, int count, int ties, uint32_t* scratch, int* err, cudaStream_t s);
// Or-opt-k for any k in [1, kMaxOroptK] on one job: the per-block candidates
// (oropt_blocks(k, size) keys, (delta, ctx) as the sweep's) and the pass over
// them (greedy, apply; rebuild the ADS afterwards with launch_prepare).
size_t oropt_pass_scratch_bytes(int size, int k);
cudaError_t launch_oropt_eval(const JobDev* job, int k, int size, bool wide, uint64_t* keys, cudaStream_t s);
cudaError_t launch_oropt_pass(const JobDev* job, int k, bool wide, const uint64_t* keys, uint8_t* scratch,
                              uint32_t* out_ij, int64_t* out_cost, int* out_count, cudaStream_t s);
// Reference ADS buffer (source/mlads.h:38-74) of each job's current tour.
cudaError_t launch_ads(const JobDev* job, const int32_t* cx, const int32_t* cy, uint32_t* ads,
                       int cost_tour, int dist_round, cudaStream_t s, uint32_t* Pbuf, int size);
// D[a][b] = int(sqrtf(float(dx^2 + dy^2)) + dr)  (source/mlproblem.cpp:153-166)
cudaError_t launch_dist(const int32_t* x, const int32_t* y, int n, int dist_round, int32_t* D,
                        int32_t* dmax, cudaStream_t s);
// Sequential application of legacy moves (source/dvnd.cpp:16-145).
// `moves` holds m (id, i, j) int32 triples.
cudaError_t launch_legacy_apply(const JobDev* job, const int32_t* moves, int m, cudaStream_t s);

}  // namespace mlp
