/*
 * mlp_oracle.h -- CPU restatement of the reference's MLP local-search path.
 *
 * TEST INFRASTRUCTURE.  This library is the checker for the GPU engine: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The
 * product (libmlpgpu.so) never links, loads or calls it.
 *
 * Parity is pinned by the reference's own known answers (tests/mtrand.Test.cpp,
 * tests/mlproblem.Test.cpp, tests/mlsolution.Test.cpp,
 * tests/WamcaExperiment.Test.cpp) and by fixtures generated from the
 * reference's compiled CPU evaluator (oracle/_ref, tests/golden/).
 *
 * Conventions
 *   n      number of instance nodes (TSPLIB DIMENSION); node ids 0..n-1.
 *   size   tour length = n + costTour (the reference's problem.size); with
 *          costTour the tour ends with a copy of the depot (node 0).
 *   D      n x n row-major int32 distance matrix indexed by node id.
 *   wide   0: costs and deltas are int32 / uint32 with the reference's
 *          wrap-around arithmetic; 1: exact int64 (the widened evaluator).
 *   nb     neighbourhood: 0 SWAP, 1 2OPT, 2 OROPT1, 3 OROPT2, 4 OROPT3
 *          (move id = nb; Or-opt-k has id k+1, source/mlads.h:26-28).
 */
#ifndef MLP_ORACLE_H
#define MLP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- RNG (source/mtrand.cpp, source/mtrand.h) ---- */
void orc_mt_rand(uint32_t seed, int count, uint32_t* out);
void orc_mt_rand_max(uint32_t seed, uint32_t max, int count, uint32_t* out);

/* ---- instance (source/tsplib.cpp, source/mlproblem.cpp) ---- */
/* Reads a TSPLIB EUC_2D file; writes inear()-rounded coords; returns DIMENSION,
 * -1 on I/O error, -2 if not EUC_2D, -3 if DIMENSION > maxn. */
int orc_tsplib_read(const char* path, int maxn, int32_t* x, int32_t* y);
/* D[a][b] = int(sqrtf(float(dx^2+dy^2)) + dr), dr = 0.5 iff distRound. */
void orc_dist_from_coords(int n, const int32_t* x, const int32_t* y, int distRound, int32_t* D);

/* ---- solution (source/mlsolution.cpp) ---- */
/* MLSolution::random(rng(seed), alpha); writes `size` = n + costTour entries. */
void orc_random_tour(int n, const int32_t* D, int costTour, uint32_t seed, float alpha, int32_t* tour);
/* The same constructor with equal distances ordered by client id (the
 * reference's std::sort leaves their order to the library); costTour = 1. */
void orc_random_tour_canonical(int n, const int32_t* D, uint32_t seed, float alpha, int32_t* tour);
/* update() + costCalc(): weights w[p] = D[t[p-1]][t[p]], cost = sum (size-p) w[p].
 * wide=0 returns the uint32 cost zero-extended. `w_out` may be NULL. */
int64_t orc_cost(int size, const int32_t* tour, int n, const int32_t* D, int wide, int32_t* w_out);
/* ldsUpdate(): reference ADS buffer (uint32 words, 32 + size*(size+3) words).
 * coords: packed x<<16|y of the tour's clients (x,y given per node). */
void orc_ads_build(int size, const int32_t* tour, int n, const int32_t* D,
                   const int32_t* x, const int32_t* y, int costTour, int distRound,
                   uint32_t* ads);

/* ---- neighbourhood evaluation (ODC kernels) ---- */
int orc_num_blocks(int nb, int size);   /* candidates per neighbourhood */
int orc_num_threads(int nb, int size);  /* ctx range per block */
/* Per-block candidate: argmin over ctx of delta, ties to the smallest ctx.
 * faithful=1 restates the reference loops; faithful=0 uses prefix sums (O(1)).
 * Outputs (length orc_num_blocks): cost, i, j, ctx.  A block with no
 * selectable move gets cost = sentinel (INT32_MAX / INT64_MAX), i=j=ctx=0. */
void orc_eval(int nb, int size, const int32_t* tour, int n, const int32_t* D, int wide,
              int faithful, int64_t* cost, int32_t* mi, int32_t* mj, int32_t* mctx);
/* Delta of a single move by brute force: apply to a copy, recompute cost. */
int64_t orc_move_delta_bruteforce(int id, int i, int j, int size, const int32_t* tour,
                                  int n, const int32_t* D, int wide);
/* Delta of a single move by the faithful reference formula. */
int64_t orc_move_delta(int id, int i, int j, int size, const int32_t* tour, int n,
                       const int32_t* D, int wide);

/* ---- merge ---- */
/* Same-neighbourhood predicates of the GPU merge (source/mlkernel.cu:51-71). */
int orc_can_merge_same(int nb, int id1, int i1, int j1, int id2, int i2, int j2);
/* Cross-neighbourhood canMerge (source/mlkernel.cu:649-729). */
int orc_can_merge(int id1, int i1, int j1, int id2, int i2, int j2);
/* Stage-2 merge of one neighbourhood's candidates: stable sort by (cost, index)
 * of the negative ones, greedy keep with the same-neighbourhood predicate.
 * Writes kept candidate indices in order; returns their count. */
int orc_merge_same(int nb, int m, const int64_t* cost, const int32_t* mi, const int32_t* mj,
                   int32_t* kept);
/* Cross merge of an already ordered move list (ids, i, j, cost): stable sort by
 * cost then greedy keep with canMerge.  Writes kept positions; returns count. */
int orc_merge_cross(int m, const int32_t* id, const int32_t* mi, const int32_t* mj,
                    const int64_t* cost, int32_t* kept);

/* ---- apply (applyMove of each kernel) ---- */
/* Applies one move to `tour` in place (size entries). */
void orc_apply(int id, int i, int j, int size, int32_t* tour);

/* ---- one reference neighbourhood pass (runKernel of WAMCAExperiment) ---- */
/* Evaluate nb, merge (stage 2), apply kept negative moves in order, update.
 * Writes applied moves (up to max_moves) and returns their count; the new
 * tour replaces `tour`; *new_cost gets the recomputed cost. */
int orc_pass(int nb, int size, int32_t* tour, int n, const int32_t* D, int wide,
             int max_moves, int32_t* ids, int32_t* is, int32_t* js, int64_t* costs,
             int64_t* new_cost);

/* ---- DVND to a local optimum ---- */
/* Canonical multi-improvement DVND: per iteration evaluate the nb_count
 * neighbourhoods of `nbs`, merge each (stage 2), merge across (stage 3),
 * apply, update; stop when no improving candidate remains or after
 * max_iters iterations.  Returns iterations run; writes the final tour and
 * cost, the number of move evaluations and of applied moves.
 * threads: OpenMP threads for the evaluation (<=0: library default). */
int orc_dvnd(int size, int32_t* tour, int n, const int32_t* D, int wide,
             int nb_count, const int32_t* nbs, int max_iters, int threads,
             int64_t* final_cost, int64_t* evals, int64_t* moves_applied);
/* ---- TOTAL multi-improvement (every evaluated move is a candidate) ---- */
/* Kept moves of the TOTAL greedy of neighbourhood nb on `tour`, in greedy
 * (delta, i, j) order: writes up to cap of them, returns their count;
 * *candidates = number of improving moves it chose from. */
int orc_total_select(int nb, int size, const int32_t* tour, int n, const int32_t* D, int wide,
                     int cap, int64_t* cost, int32_t* is, int32_t* js, int64_t* candidates);
/* One TOTAL pass of nb: select as above, apply in order, update. */
int orc_total_pass(int nb, int size, int32_t* tour, int n, const int32_t* D, int wide,
                   int max_moves, int32_t* ids, int32_t* is, int32_t* js, int64_t* costs,
                   int64_t* new_cost);
/* DVND whose iterations use TOTAL candidate sets (nbs ascending). */
int orc_dvnd_total(int size, int32_t* tour, int n, const int32_t* D, int wide, int nb_count,
                   const int32_t* nbs, int max_iters, int64_t* final_cost, int64_t* evals,
                   int64_t* moves_applied);
/* One full sweep of the given neighbourhoods (fast evaluator, OpenMP);
 * returns the number of move evaluations (for the CPU baseline). */
int64_t orc_sweep(int size, const int32_t* tour, int n, const int32_t* D, int wide,
                  int nb_count, const int32_t* nbs, int threads, int64_t* cost_out,
                  int32_t* i_out, int32_t* j_out);

/* ---- legacy C-ABI helpers (source/dvnd.cu, source/dvnd.cpp) ---- */
int orc_legacy_no_conflict(int id1, int i1, int j1, int id2, int i2, int j2);
int orc_legacy_better_no_conflict(int m, const int32_t* ids, const int32_t* is,
                                  const int32_t* js, const int32_t* costs,
                                  int32_t* selected, int32_t* imp_value,
                                  int maximize, int melhor_para_pior);
/* applyMoves: applies ids/is/js in order with the legacy semantics (2-opt ids
 * are applied as swaps); returns the recomputed uint32 cost. */
uint32_t orc_legacy_apply_moves(int size, int32_t* tour, int n, const int32_t* D,
                                int m, const int32_t* ids, const int32_t* is,
                                const int32_t* js);

#ifdef __cplusplus
}
#endif

#endif
