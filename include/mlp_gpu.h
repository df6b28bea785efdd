/*
 * mlp_gpu.h -- C-ABI of the GB300 MLP local-search engine (libmlpgpu.so).
 *
 * Plain C types only: pointers, sizes and status codes; no CUDA or C++ types
 * in any signature (a CUDA stream is passed as `void*`).  Every function
 * returns MLP_OK (0) or a nonzero MLP_ERR_* code; mlp_last_error() gives the
 * message of the calling thread's last failure.  Handles are not thread-safe:
 * use one handle per thread, or serialise calls on a handle.
 *
 * Mapping to the reference (LabIC-UFF/wamca-gpu-mi):
 *   mlp_problem_*   MLProblem(costTour, distRound, coordShift) + load()
 *                   (source/mlproblem.h:61-151, source/mlproblem.cpp:78-207)
 *   mlp_solver_*    MLSolution (tour, update/costCalc/ldsUpdate, ADS buffer;
 *                   source/mlsolution.h:62-434) together with the
 *                   MLKernelSwap / MLKernel2Opt / MLKernelOrOpt tasks
 *                   (source/mlkernel.h:104-318) and the runKernel/runGpuGpu
 *                   glue of WAMCAExperiment (source/WamcaExperiment.hpp:229-365)
 *   mlp_batch_*     many independent DVND searches in shared launches (no
 *                   counterpart in the reference; the batched form)
 *   mlp_server_*    continuous-batching request loop (no counterpart; the
 *                   serving form)
 * The reference's own extern "C" DVND entry points are in wamca_dvnd.h.
 *
 * Conventions: n = number of nodes (node ids 0..n-1, depot 0); size = n + 1 is
 * the tour length (costTour: the tour starts and ends at depot 0, as in every
 * reference entry point).  Neighbourhoods: 0 SWAP, 1 2OPT, 2 OROPT1,
 * 3 OROPT2, 4 OROPT3 (move id = neighbourhood, source/mlads.h:150-181).
 * `wide` = 0 computes costs and deltas in 32 bits with the reference's
 * wrap-around arithmetic; `wide` = 1 computes them exactly in 64 bits.
 */
#ifndef MLP_GPU_H
#define MLP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MLP_API __attribute__((visibility("default")))
#else
#define MLP_API
#endif

enum {
  MLP_OK = 0,
  MLP_ERR_ARG = 1,         /* invalid argument */
  MLP_ERR_CUDA = 2,        /* CUDA runtime error (message in mlp_last_error) */
  MLP_ERR_RANGE = 3,       /* size, distance or coordinate out of range */
  MLP_ERR_IO = 4,          /* file cannot be read */
  MLP_ERR_FORMAT = 5,      /* malformed or unsupported instance file */
  MLP_ERR_NOMEM = 6,       /* device or host allocation failed / over budget */
  MLP_ERR_STATE = 7,       /* call not valid in the handle's current state */
  MLP_ERR_UNSUPPORTED = 8, /* feature the reference does not support */
  MLP_ERR_CANCELLED = 9,   /* served request cancelled before it finished */
  MLP_PENDING = 10         /* served request not finished yet (not an error) */
};

enum { MLP_NB_SWAP = 0, MLP_NB_2OPT = 1, MLP_NB_OROPT1 = 2, MLP_NB_OROPT2 = 3, MLP_NB_OROPT3 = 4 };
#define MLP_NB_ALL 0x1f

typedef struct mlp_problem* mlp_problem_t;
typedef struct mlp_solver* mlp_solver_t;
typedef struct mlp_batch* mlp_batch_t;
typedef struct mlp_server* mlp_server_t;

typedef struct {
  int64_t cost;        /* latency of the final tour */
  int64_t iterations;  /* DVND iterations that applied at least one move */
  int64_t sweeps;      /* full neighbourhood evaluations run */
  int64_t moves;       /* moves applied */
  int64_t evals;       /* move evaluations performed */
  int32_t converged;   /* 1 if a local optimum was reached */
  int32_t reserved;
} mlp_dvnd_stats_t;

/* ---- library ---- */
MLP_API int mlp_version(void);
MLP_API const char* mlp_last_error(void);
MLP_API const char* mlp_status_string(int status);
MLP_API int mlp_device_count(int32_t* count);
MLP_API int mlp_set_device(int32_t device);

/* ---- problem (MLProblem) ---- */
/* Distances D[a][b] = int(sqrtf(float(dx^2+dy^2)) + 0.5*dist_round), built on
 * the device (source/mlproblem.cpp:153-166).  cost_tour must be 1. */
MLP_API int mlp_problem_create_coords(int32_t n, const int32_t* x, const int32_t* y,
                                      int32_t cost_tour, int32_t dist_round, mlp_problem_t* out);
/* Same with x, y already in device memory. */
MLP_API int mlp_problem_create_coords_device(int32_t n, const int32_t* x_dev, const int32_t* y_dev,
                                             int32_t cost_tour, int32_t dist_round,
                                             mlp_problem_t* out);
/* Symmetric n x n row-major matrix, entries in [0, 65535]. */
MLP_API int mlp_problem_create_matrix(int32_t n, const int32_t* dist, int32_t cost_tour,
                                      mlp_problem_t* out);
/* TSPLIB EUC_2D file (MLProblem::load). */
MLP_API int mlp_problem_load_tsplib(const char* path, int32_t cost_tour, int32_t dist_round,
                                    mlp_problem_t* out);
MLP_API int mlp_problem_info(mlp_problem_t p, int32_t* n, int32_t* size, int32_t* max_dist);
/* `count` starts of MLSolution::random (as mlp_solver_random_tour), start q
 * from seeds[q], built on the device in parallel (one warp each) and copied to
 * `tours` (count x size entries, host memory). */
MLP_API int mlp_problem_random_tours(mlp_problem_t p, int32_t count, const uint32_t* seeds, float alpha,
                                     int32_t* tours);
/* The same with the tie order chosen: ties = 0 as above (client id, one warp
 * per start, a rank selection per step); ties = 1 the reference's own order,
 * equal to MLSolution::random built with GCC's libstdc++: the persistent
 * candidate array is re-sorted each step by a restatement of that library's
 * std::sort (one warp per start, the sort on one lane; slower, for parity). */
MLP_API int mlp_problem_random_tours_ties(mlp_problem_t p, int32_t count, const uint32_t* seeds, float alpha,
                                          int32_t ties, int32_t* tours);
/* Copies the n x n distance matrix to host memory. */
MLP_API int mlp_problem_get_dist(mlp_problem_t p, int32_t* dist);
MLP_API void mlp_problem_destroy(mlp_problem_t p);

/* ---- solver (MLSolution + MLKernel tasks of one instance) ---- */
MLP_API int mlp_solver_create(mlp_problem_t p, int32_t wide, mlp_solver_t* out);
MLP_API void mlp_solver_destroy(mlp_solver_t s);
/* Stream on which every later call of this solver runs (NULL: the solver's own). */
MLP_API int mlp_solver_set_stream(mlp_solver_t s, void* cuda_stream);
/* Sweep tile shape index (0..13: diagonals x rows = 32x4, 32x8, 32x16, 64x4, 64x8,
 * 64x16, 128x8, 128x16, 32x32, 64x32, then 64x8, 64x16, 64x32, 128x16 where the
 * DVND sweep gives each thread two adjacent diagonals).  Loop mode of mlp_solver_dvnd: iterations = 0
 * (the default) runs the whole loop on the device (a CUDA-graph while node
 * over 16 iterations at a time, no host round trips; always the mode of
 * mlp_solver_dvnd_async; a solver without a stream of its own checks on the
 * host after every iteration); iterations >= 1 replays CUDA graphs of that
 * many iterations and checks convergence on the host in between. */
MLP_API int mlp_solver_set_tile_shape(mlp_solver_t s, int32_t shape);
MLP_API int mlp_solver_set_unroll(mlp_solver_t s, int32_t iterations);
/* DVND sweep kernel (no counterpart in the reference): 1 (default) the
 * kernel that reads per-position row and column terms (32-bit solvers that
 * evaluate all five neighbourhoods), 0 the general fused sweep.  Results are
 * identical; the switch exists for measurement and testing. */
MLP_API int mlp_solver_set_sweep_kernel(mlp_solver_t s, int32_t variant);
/* Merge kernel of the solver's iterations (as mlp_batch_set_merge_mode; the
 * default for one search is the six-CTA cluster).  Every mode gives the same
 * results. */
MLP_API int mlp_solver_set_merge_mode(mlp_solver_t s, int32_t mode);
/* Candidate mode of every later pass / DVND of this solver.  0 (default): one
 * candidate per reference block (the ODC kernels).  1: TOTAL multi-improvement
 * (the reference's isTotal kernels, source/mlkernel.h:150-163,
 * mlkswap.cu:334-526, mlk2opt.cu:270-447, mlkoropt.cu:368-612, merged by
 * mlkernel.cu:183-250): every move the neighbourhood evaluates is a candidate;
 * per neighbourhood the improving ones are taken greedily in (delta, i, j)
 * order, skipping any that conflicts with one taken before; a DVND iteration
 * then merges the neighbourhoods' selections as usual.  The first switch to 1
 * allocates the TOTAL lists: about 32 * size^2 bytes (64 * size^2 with 64-bit
 * costs). */
MLP_API int mlp_solver_set_total(mlp_solver_t s, int32_t on);
/* Tour of `len` = size entries: tour[0] = tour[size-1] = 0 and a permutation of
 * 1..n-1 in between.  Rebuilds the ADS (update() + ldsUpdate()). */
MLP_API int mlp_solver_set_tour(mlp_solver_t s, const int32_t* tour, int32_t len);
/* Same with the tour already in device memory (enqueued, no host sync). */
MLP_API int mlp_solver_set_tour_device(mlp_solver_t s, const int32_t* tour_dev, int32_t len);
/* The tour becomes a start of MLSolution::random(rng, alpha) (source/mlsolution.cpp:754-874)
 * built on the device: MTRandom seeded with `seed`; each step appends the
 * candidate of rank rng.rand(ceil(alpha * count) - 1) in ascending distance to
 * the client added last.  Equal distances are taken in client-id order (the
 * reference's std::sort leaves their order to the library).  alpha in [0, 1].
 * Rebuilds the ADS. */
MLP_API int mlp_solver_random_tour(mlp_solver_t s, uint32_t seed, float alpha);
/* As mlp_solver_random_tour with the tie order chosen (see
 * mlp_problem_random_tours_ties; ties = 1 reproduces MLSolution::random). */
MLP_API int mlp_solver_random_tour_ties(mlp_solver_t s, uint32_t seed, float alpha, int32_t ties);
MLP_API int mlp_solver_get_tour(mlp_solver_t s, int32_t* tour, int32_t len);
/* Checkpoint / resume in the text format of MLSolution::save / load
 * (source/mlsolution.cpp:685-751): tour length, cost, the tour.  Loading
 * accepts a stored length of size or size - 1 as the reference does, reads
 * size entries, validates the tour and recomputes the cost and ADS. */
MLP_API int mlp_solver_save(mlp_solver_t s, const char* path);
MLP_API int mlp_solver_load(mlp_solver_t s, const char* path);
/* Device pointer to the solver's current tour (valid until destroy). */
MLP_API int mlp_solver_tour_device(mlp_solver_t s, int32_t** tour_dev);
/* Latency cost of the current tour (MLSolution::costCalc after update). */
MLP_API int mlp_solver_cost(mlp_solver_t s, int64_t* cost);
/* Adjacent weights w[p] (MLSolution::weights), `len` = size. */
MLP_API int mlp_solver_weights(mlp_solver_t s, int32_t* w, int32_t len);
/* Reference ADS buffer (MLSolution::adsData after ldsUpdate, source/mlads.h:38-74):
 * 32 + size*(size+3) uint32 words.  Header words 6..31 are zero. */
MLP_API int mlp_solver_ads(mlp_solver_t s, uint32_t* ads, int64_t words);
/* Per-block candidates of one neighbourhood on the current tour (the move buffer
 * an ODC kernel writes, one per reference block), without merging.  Arrays of
 * mlp_solver_num_candidates(nb) entries; a block without a selectable move gets
 * cost = INT32_MAX (wide: INT64_MAX) and i = j = 0. */
MLP_API int mlp_solver_num_candidates(mlp_solver_t s, int32_t nb, int32_t* count);
MLP_API int mlp_solver_eval(mlp_solver_t s, int32_t nb, int64_t* cost, int32_t* i, int32_t* j);
/* One reference neighbourhood pass (runKernel: evaluate nb, GPU merge, apply the
 * kept improving moves, update).  Writes up to max_moves applied moves in
 * application order; *count = moves applied; *new_cost = resulting cost. */
MLP_API int mlp_solver_pass(mlp_solver_t s, int32_t nb, int32_t max_moves, int32_t* ids,
                            int32_t* is, int32_t* js, int64_t* costs, int32_t* count,
                            int64_t* new_cost);
/* Or-opt-k for any k in [1, 28] (MLKernelOrOpt(problem, k): the ODC
 * kernelOrOpt with tag = k, source/mlkoropt.cu:620-794, move id k + 1).
 * eval: the per-block candidates, size - k - 2 entries (as mlp_solver_eval).
 * pass: evaluate, merge the improving candidates greedily in (delta, block)
 * order with f_canOrOptMerge, apply them and rebuild the ADS (as
 * mlp_solver_pass); moves are written in application order, their id is
 * k + 1.  The DVND's three Or-opt neighbourhoods are k = 1, 2, 3. */
MLP_API int mlp_solver_eval_oropt(mlp_solver_t s, int32_t k, int64_t* cost, int32_t* i, int32_t* j);
MLP_API int mlp_solver_pass_oropt(mlp_solver_t s, int32_t k, int32_t max_moves, int32_t* is, int32_t* js,
                                  int64_t* costs, int32_t* count, int64_t* new_cost);
/* Multi-improvement DVND to a local optimum over the neighbourhoods of nb_mask
 * (at most max_iters sweeps).  Synchronous. */
MLP_API int mlp_solver_dvnd(mlp_solver_t s, int32_t nb_mask, int32_t max_iters,
                            mlp_dvnd_stats_t* stats);
/* Enqueue a whole DVND (device-side loop) on the solver's stream and return
 * without waiting; read the result with mlp_solver_stats / get_tour. */
MLP_API int mlp_solver_dvnd_async(mlp_solver_t s, int32_t nb_mask, int32_t max_iters);
/* Enqueue `iterations` DVND iterations on the solver's stream without waiting
 * (call mlp_solver_begin first; read results with mlp_solver_stats). */
MLP_API int mlp_solver_begin(mlp_solver_t s, int32_t nb_mask, int32_t max_iters);
MLP_API int mlp_solver_enqueue(mlp_solver_t s, int32_t iterations);
MLP_API int mlp_solver_stats(mlp_solver_t s, mlp_dvnd_stats_t* stats);
/* Enqueue `repeats` sweeps of nb_mask as the solver's DVND iterations run them
 * (the same kernel, improving candidates only; a timing helper: the tour is
 * not changed): one tiny counter-reset kernel, `repeats` sweep kernels and one
 * ADS rebuild.  *evals_per_sweep = move evaluations of one sweep. */
MLP_API int mlp_solver_sweep(mlp_solver_t s, int32_t nb_mask, int32_t repeats,
                             int64_t* evals_per_sweep);
/* Tile-shape table (no counterpart in the reference; chosen by the
 * autotuner wamca-gpu-mi_gb300/mlpgpu/autotune.py).  Row q applies to job
 * sets whose largest tour has at most max_size[q] positions: shape_one[q] for
 * fewer than 8 jobs, shape_many[q] for 8 or more; sizes strictly increasing,
 * count <= 64 (0 clears the table; without a table a built-in rule applies).
 * Process-wide; used by solvers, batches and servers created afterwards (an
 * explicit set_tile_shape wins).  The shape never changes results. */
MLP_API int mlp_tuning_set(const int32_t* max_size, const int32_t* shape_one, const int32_t* shape_many,
                           int32_t count);
MLP_API int mlp_tuning_get(int32_t* max_size, int32_t* shape_one, int32_t* shape_many, int32_t cap,
                           int32_t* count);
/* Loads the table from the autotuner's JSON file ("table": [[size, one, many], ...]). */
MLP_API int mlp_tuning_load(const char* path);
/* Autotune the sweep tile shape on the current tour; returns the chosen index. */
MLP_API int mlp_solver_autotune(mlp_solver_t s, int32_t* shape);
/* Timing helper: `repeats` launches of the solver's sweep kernel for nb_mask
 * on the current tour (improving candidates only, as its DVND iterations run
 * it), timed with CUDA events on the solver's stream.  Without flush (null):
 * the launches back to back between two events, *ms = the time per launch in
 * milliseconds.  With flush (a device buffer of flush_bytes): the buffer is
 * overwritten before every launch, so one larger than L2 makes each launch
 * start cold, and each launch sits between its own two events; *ms = the
 * median.  The candidate keys are reset and the ADS rebuilt afterwards; the
 * tour is not changed. */
MLP_API int mlp_solver_time_sweep(mlp_solver_t s, int32_t nb_mask, int32_t repeats, void* flush, int64_t flush_bytes,
                                  float* ms);

/* Evaluation without any allocation (no counterpart in the reference).
 * For callers that cannot allocate device memory -- code running inside
 * another framework's memory pool or budget, services whose device memory is
 * partitioned ahead of time, hosts that must not call cudaMalloc/cudaFree
 * (they synchronise the whole device).  Computes the per-block candidates of
 * neighbourhood nb (as mlp_solver_eval) for `tour_dev` (n + 1 entries) over
 * the n x n distances `dist_dev`, writing nb's candidate count of entries to
 * cost_dev / i_dev / j_dev; every pointer is device memory owned by the
 * caller.  With size = n + 1 the candidate count is (size + 1) / 2 - 1 for
 * swap (nb 0), (size + 1) / 2 for 2-opt (nb 1) and size - k - 2 for Or-opt-k
 * (nb = k + 1).  The tour must hold depot 0 at both ends and every client
 * 1..n-1 once; it is checked on the device before any distance is read
 * through it, and a tour that fails yields cost INT64_MIN and i = j = -1 in
 * every output entry (nothing else is read or written).  Distances are used
 * only as values: they must be symmetric and in [0, 65535] (as
 * mlp_problem_from_matrix requires), otherwise the candidates are
 * meaningless.  All intermediate data lives in one fixed 256 KB device array that
 * the library holds on each GPU it is loaded on until the process exits:
 * n + 1 <= 2048, larger instances are rejected with MLP_ERR_RANGE.  The first
 * call on a device looks up that array's address (make it before any stream
 * capture).  Every call shares the array: calls that overlap on the GPU race,
 * so serialise them.  Enqueued on `stream` (NULL: legacy default stream). */
MLP_API int mlp_eval_noalloc(const int32_t* dist_dev, int32_t n, const int32_t* tour_dev, int32_t nb,
                             int32_t wide, int64_t* cost_dev, int32_t* i_dev, int32_t* j_dev,
                             void* stream);

/* ---- batched form ---- */
MLP_API int mlp_batch_create(int32_t wide, mlp_batch_t* out);
MLP_API void mlp_batch_destroy(mlp_batch_t b);
MLP_API int mlp_batch_set_stream(mlp_batch_t b, void* cuda_stream);
/* Adds a search of problem p from `tour` (size entries).  The problem must
 * outlive the batch.  Returns the job index in *job. */
MLP_API int mlp_batch_add(mlp_batch_t b, mlp_problem_t p, const int32_t* tour, int32_t len,
                          int32_t* job);
/* Runs every job's DVND to a local optimum (at most max_iters sweeps each). */
MLP_API int mlp_batch_run(mlp_batch_t b, int32_t nb_mask, int32_t max_iters);
/* Same, enqueued on the batch's stream without waiting (device-side loop). */
MLP_API int mlp_batch_run_async(mlp_batch_t b, int32_t nb_mask, int32_t max_iters);
/* Resets every job to the tour it was added with (for repeated runs). */
MLP_API int mlp_batch_reset(mlp_batch_t b);
MLP_API int mlp_batch_result(mlp_batch_t b, int32_t job, int32_t* tour, int32_t len,
                             mlp_dvnd_stats_t* stats);
MLP_API int mlp_batch_set_tile_shape(mlp_batch_t b, int32_t shape);
/* Merge kernel of the batch's iterations: 0 = automatic (one CTA per job for
 * 16 jobs or more, otherwise a six-CTA cluster per job), 1 = cluster, 2 = one
 * CTA per job.  Every mode gives the same results. */
MLP_API int mlp_batch_set_merge_mode(mlp_batch_t b, int32_t mode);
/* DVND sweep kernel of the batch's iterations (as mlp_solver_set_sweep_kernel). */
MLP_API int mlp_batch_set_sweep_kernel(mlp_batch_t b, int32_t variant);
/* Adds a search whose start is MLSolution::random(seed, alpha), built on the
 * device when the batch is (re)started (as mlp_solver_random_tour). */
MLP_API int mlp_batch_add_random(mlp_batch_t b, mlp_problem_t p, uint32_t seed, float alpha, int32_t* job);
/* As mlp_batch_add_random with the tie order chosen (see mlp_problem_random_tours_ties). */
MLP_API int mlp_batch_add_random_ties(mlp_batch_t b, mlp_problem_t p, uint32_t seed, float alpha, int32_t ties,
                                      int32_t* job);
/* Candidate mode of the batch's searches (as mlp_solver_set_total). */
MLP_API int mlp_batch_set_total(mlp_batch_t b, int32_t on);
/* Iterations between the host's convergence checks (default 4); after each
 * check the jobs that converged leave the launches.  The host reads each
 * check's statistics while the next interval runs, so a job that converged
 * stays in the launches for one more interval (its kernels return at once). */
MLP_API int mlp_batch_set_check_interval(mlp_batch_t b, int32_t iterations);

/* ---- serving form: continuous batching of arriving searches ----
 * A server owns a CUDA stream and a device memory pool.  Requests (instance
 * coordinates, start tour, neighbourhood mask, sweep limit) are queued by
 * mlp_server_submit; each mlp_server_step admits queued requests in arrival
 * order while a slot is free and their footprint (mlp_server_footprint: the
 * n x n int32 distances, coordinates, tour and ADS arrays) fits the memory
 * budget, runs `iters` DVND iterations over every admitted search in shared
 * launches and retires the searches that converged or used their sweep limit.
 * A search's result is the same as mlp_solver_dvnd's on the same input, alone
 * or in any mix.  submit / finished / result / cancel / status may be called
 * from other threads while one thread calls step. */
typedef struct {
  double arrival;   /* seconds on the server clock (mlp_server_now) */
  double admitted;  /* admission time (-1 if never admitted) */
  double finished;  /* time the result became available */
  int32_t status;   /* MLP_OK, MLP_ERR_CANCELLED or the error that ended it */
  int32_t n;
} mlp_serve_info_t;

/* memory_budget: device bytes for admitted searches; max_active: slots. */
MLP_API int mlp_server_create(int64_t memory_budget, int32_t wide, int32_t max_active, mlp_server_t* out);
MLP_API void mlp_server_destroy(mlp_server_t s);
/* Seconds since the server was created (the clock of arrival/finish times). */
MLP_API double mlp_server_now(mlp_server_t s);
/* Device bytes one search of n nodes is admitted against (-1: n invalid). */
MLP_API int64_t mlp_server_footprint(int32_t n, int32_t wide);
/* Fixed tile shape for the sweeps (-1: chosen per step). */
MLP_API int mlp_server_set_tile_shape(mlp_server_t s, int32_t shape);
/* Queues a search of the EUC_2D instance (x, y) from `tour` (n + 1 entries).
 * arrival < 0 stamps the current server time.  Rejected with MLP_ERR_NOMEM if
 * its footprint exceeds the whole budget, MLP_ERR_ARG for a malformed tour. */
MLP_API int mlp_server_submit(mlp_server_t s, int32_t n, const int32_t* x, const int32_t* y, int32_t dist_round,
                              const int32_t* tour, int32_t len, int32_t nb_mask, int32_t max_iters,
                              double arrival, int64_t* id);
/* Admits, iterates `iters` times, retires; reports the active and queued counts. */
MLP_API int mlp_server_step(mlp_server_t s, int32_t iters, int32_t* active, int32_t* queued);
/* Ids finished since the last call (at most cap of them). */
MLP_API int mlp_server_finished(mlp_server_t s, int64_t* ids, int32_t cap, int32_t* count);
/* Takes a finished request's result (tour may be NULL); MLP_PENDING while it
 * is queued or running. */
MLP_API int mlp_server_result(mlp_server_t s, int64_t id, int32_t* tour, int32_t len, mlp_dvnd_stats_t* stats,
                              mlp_serve_info_t* info);
/* Cancels a queued request at once, a running one at the end of the next step. */
MLP_API int mlp_server_cancel(mlp_server_t s, int64_t id);
MLP_API int mlp_server_status(mlp_server_t s, int64_t* mem_in_use, int32_t* active, int32_t* queued,
                              int32_t* finished);
/* Failure injection on the host: the next `count` admissions fail as if a
 * host allocation had failed (their requests end with MLP_ERR_NOMEM). */
MLP_API int mlp_server_fail_next_admissions(mlp_server_t s, int32_t count);

#ifdef __cplusplus
}
#endif

#endif
