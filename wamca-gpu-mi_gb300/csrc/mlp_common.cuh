// mlp_common.cuh -- shared definitions of the GB300 MLP local-search engine.
//
// Position/move conventions follow the reference task API:
//   size  = tour length = n + 1 (costTour: the tour ends with a copy of depot 0),
//           source/mlproblem.cpp:68
//   w[p]  = D[t[p-1]][t[p]] (w[0] = 0), source/mlsolution.cpp:216-228
//   cost  = sum_{p=1}^{size-1} (size - p) * w[p]
//   move ids: SWAP 0, 2OPT 1, OROPT-k k+1 (source/mlads.h:26-28, 150-181)
//
// Candidate keys.  Each reference "block" of a neighbourhood kernel yields one
// candidate (source/mlkswap.cu:944-964, mlk2opt.cu:590-611, mlkoropt.cu:742-764).
// The engine stores it as a 64-bit key ordered by (delta, ctx):
//   key = (uint64(delta + 2^45) << 14) | ctx          (sweep output)
// |delta| < 2^45 holds for size <= 16384 and distances <= 65535 (the reference's
// 14-bit move indices and ushort weights, source/mlads.h:190-195,
// source/mlsolution.h:79-80).
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define MLP_HD __host__ __device__ __forceinline__
#else
#define MLP_HD inline
#endif

namespace mlp {

constexpr int kNumNb = 5;            // SWAP, 2OPT, OROPT1, OROPT2, OROPT3
constexpr int kMaxSize = 16384;      // 14-bit i/j in MLMove64
constexpr int kMaxDist = 65535;      // ushort weights
constexpr int kCtxBits = 14;
constexpr uint64_t kCostBias = 1ull << 45;
constexpr uint64_t kKeyNone = ~0ull;
constexpr int32_t kCostInfty32 = 0x7fffffff;  // COST_INFTY, source/mlads.h:24

// ---------------- per-neighbourhood candidate layout ----------------
// Number of reference blocks (= candidates) per neighbourhood for costTour=1.
MLP_HD int nb_blocks(int nb, int size) {
  if (nb == 0) return ((size + 1) / 2) - 1;  // mlkswap.cu:1001
  if (nb == 1) return (size + 1) / 2;        // mlk2opt.cu:680
  return size - (nb - 1) - 2;                // mlkoropt.cu:842 (tour)
}
// ctx range per block (threads that hold a move).
MLP_HD int nb_threads(int nb, int size) {
  if (nb == 0) return size - 4;              // mlkswap.cu:763
  if (nb == 1) return size - 3;              // mlk2opt.cu:559
  return size - (nb - 1) - 2;                // mlkoropt.cu:699
}
MLP_HD int nb_offset(int nb, int size) {
  int off = 0;
  for (int q = 0; q < nb; q++) off += nb_blocks(q, size);
  return off;
}
MLP_HD int total_blocks(int size) { return nb_offset(kNumNb, size); }

// (nb, block by, ctx) -> (i, j) of the ODC kernels (costTour = 1).
MLP_HD void map_move(int nb, int size, int by, int ctx, int& i, int& j) {
  const bool k = ctx >= by;
  if (nb == 0) {  // mlkswap.cu:766-768
    i = k ? by + 1 : size - by - 3;
    j = k ? ctx + 3 : size - ctx - 2;
  } else if (nb == 1) {  // mlk2opt.cu:561-563
    i = k ? ctx - by + 1 : by - ctx;
    j = k ? ctx + 2 : size - ctx - 2;
  } else {  // mlkoropt.cu:701-722
    const int kk = nb - 1;
    if (k) {
      i = ctx - by + 1;
      j = ctx + 2;
    } else {
      i = size - ctx - kk - 1;
      j = by - ctx;
    }
  }
}

// Or-opt-k for any k in [1, kMaxOroptK] (MLKernelOrOpt(problem, k), the
// kernel's tag = k; move id k + 1, source/mlads.h:26-27): reference blocks
// (= candidates) and the ODC block mapping, costTour = 1
// (source/mlkoropt.cu:699-722, :842).
constexpr int kMaxOroptK = 28;  // launchKernel rejects k > MLP_MAX_NEIGHBOR - 2 (mlkoropt.cu:866-868)
MLP_HD int oropt_blocks(int k, int size) { return size - k - 2; }
MLP_HD void map_oropt(int k, int size, int by, int ctx, int& i, int& j) {
  if (ctx >= by) {
    i = ctx - by + 1;
    j = ctx + 2;
  } else {
    i = size - ctx - k - 1;
    j = by - ctx;
  }
}

MLP_HD uint64_t make_key(int64_t delta, uint32_t low, int low_bits) {
  return ((uint64_t)(delta + (int64_t)kCostBias) << low_bits) | (uint64_t)low;
}
MLP_HD int64_t key_cost(uint64_t key, int low_bits) {
  return (int64_t)(key >> low_bits) - (int64_t)kCostBias;
}

// Footprint of a move: the tour positions whose client changes.
MLP_HD void move_footprint(int id, int i, int j, int& f0, int& f1) {
  if (id == 0) {
    f0 = i;
    f1 = j;
  } else if (id == 1) {
    f0 = i;
    f1 = j;
  } else {
    const int k = id - 1;
    if (i < j) {
      f0 = i;
      f1 = j + k - 1;
    } else {
      f0 = j;
      f1 = i + k - 1;
    }
  }
}

// Source position of new position p inside the footprint of a move
// (the permutation performed by applyMove: mlkswap.cu:1070-1078,
// mlk2opt.cu:737-745, mlkoropt.cu:896-925).
MLP_HD int move_source(int id, int i, int j, int p) {
  if (id == 0) return p == i ? j : (p == j ? i : p);
  if (id == 1) return i + j - p;
  const int k = id - 1;
  if (i < j) return p < j ? p + k : p - j + i;
  return p < j + k ? p - j + i : p - k;
}

// ---------------- TOTAL candidate keys ----------------
// A move of a TOTAL list is one key ordered by (delta, i, j): the delta with
// its sign bit flipped above 14-bit i and j.  int32 mode: 60 bits of a uint64;
// wide mode: 92 bits of a 128-bit integer.
constexpr int kTotalKeyShift = 28;
MLP_HD uint64_t total_key32(int32_t d, int i, int j) {
  return ((uint64_t)((uint32_t)d ^ 0x80000000u) << kTotalKeyShift) | ((uint64_t)i << 14) | (uint64_t)j;
}
MLP_HD int32_t total_key32_delta(uint64_t k) { return (int32_t)((uint32_t)(k >> kTotalKeyShift) ^ 0x80000000u); }
#ifdef __CUDACC__
typedef unsigned __int128 u128;
MLP_HD u128 total_key64(int64_t d, int i, int j) {
  return ((u128)((uint64_t)d ^ 0x8000000000000000ull) << kTotalKeyShift) | ((u128)i << 14) | (u128)j;
}
MLP_HD int64_t total_key64_delta(u128 k) {
  return (int64_t)((uint64_t)(k >> kTotalKeyShift) ^ 0x8000000000000000ull);
}
#endif
// Capacity of neighbourhood nb's TOTAL list: swap and 2-opt have at most one
// move per position pair, Or-opt-k one per ordered pair.
MLP_HD int64_t total_list_cap(int nb, int size) {
  const int64_t pairs = (int64_t)size * (size - 1) / 2;
  return (nb < 2 ? pairs : 2 * pairs) + 64;
}
MLP_HD int64_t total_list_off(int nb, int size) {
  int64_t o = 0;
  for (int q = 0; q < nb; q++) o += total_list_cap(q, size);
  return o;
}

// Stage-2 output region of neighbourhood nb: kept moves are independent
// sets, at most size/4 + 1 swaps, size/3 + 1 2-opt and size/(k+2) + 1
// Or-opt-k moves.
MLP_HD int region_cap(int nb, int size) {
  const int div = nb == 0 ? 4 : nb == 1 ? 2 : nb == 2 ? 3 : nb == 3 ? 4 : 5;
  return size / div + 2;
}
MLP_HD int region_off(int nb, int size) {
  int o = 0;
  for (int q = 0; q < nb; q++) o += region_cap(q, size);
  return o;
}

// ---------------- merge predicates ----------------
MLP_HD int iabs_(int v) { return v < 0 ? -v : v; }
MLP_HD int imin_(int a, int b) { return a < b ? a : b; }
MLP_HD int imax_(int a, int b) { return a > b ? a : b; }

// f_canSwapMerge (mlkernel.cu:51-54)
MLP_HD bool can_swap_same(int i1, int j1, int i2, int j2) {
  return iabs_(i1 - i2) > 1 && iabs_(i1 - j2) > 1 && iabs_(j1 - i2) > 1 && iabs_(j1 - j2) > 1;
}
// f_can2OptMerge (mlkernel.cu:56-59)
MLP_HD bool can_2opt_same(int i1, int j1, int i2, int j2) {
  return (j1 < i2 - 1) || (i1 > j2 + 1) || (j2 < i1 - 1) || (i2 > j1 + 1);
}
// f_canOrOptMerge (mlkernel.cu:61-71)
MLP_HD bool can_oropt_same(int id1, int i1, int j1, int id2, int i2, int j2) {
  return (imax_(i1, j1) + (id1 - 1) < imin_(i2, j2)) || (imin_(i1, j1) > imax_(i2, j2) + (id2 - 1));
}
// canSwapMerge / can2OptMerge / canOrOptMerge / canMerge (mlkernel.cu:649-729)
MLP_HD bool can_merge_swap(int i1, int j1, int id2, int i2, int j2) {
  if (id2 == 0) return can_swap_same(i1, j1, i2, j2);
  if (id2 == 1) return ((i1 < i2 - 1) || (i1 > j2 + 1)) && ((j1 < i2 - 1) || (j1 > j2 + 1));
  const int mn = imin_(i2, j2), mx = imax_(i2, j2), k2 = id2 - 1;
  return (j1 < mn - 1) || (i1 > mx + k2) || ((i1 < mn - 1) && (j1 > mx + k2));
}
MLP_HD bool can_merge_2opt(int i1, int j1, int id2, int i2, int j2) {
  if (id2 == 0) return can_merge_swap(i2, j2, 1, i1, j1);
  if (id2 == 1) return can_2opt_same(i1, j1, i2, j2);
  const int mn = imin_(i2, j2), mx = imax_(i2, j2), k2 = id2 - 1;
  return (i1 > mx + k2) || (j1 < mn - 1);
}
MLP_HD bool can_merge(int id1, int i1, int j1, int id2, int i2, int j2) {
  if (id1 == 0) return can_merge_swap(i1, j1, id2, i2, j2);
  if (id1 == 1) return can_merge_2opt(i1, j1, id2, i2, j2);
  if (id2 == 0) return can_merge_swap(i2, j2, id1, i1, j1);
  if (id2 == 1) return can_merge_2opt(i2, j2, id1, i1, j1);
  return can_oropt_same(id1, i1, j1, id2, i2, j2);
}

// Conflict interval of a same-neighbourhood interval move: two moves of
// neighbourhood nb (2OPT or OROPT-k) conflict iff their closed intervals
// intersect.  2OPT: f_can2OptMerge <=> [i1, j1+1] and [i2, j2+1] disjoint.
// OROPT-k: f_canOrOptMerge <=> [min, max+k] disjoint.
MLP_HD void conflict_interval(int id, int i, int j, int& a, int& b) {
  if (id == 1) {
    a = i;
    b = j + 1;
  } else {
    a = imin_(i, j);
    b = imax_(i, j) + (id - 1);
  }
}

// Branch-free form of !canMerge for the cross-neighbourhood merge.  canMerge
// (mlkernel.cu:649-729) rejects a pair when a core interval of the move of
// lower type (0 swap: {i}, {j}; 1 2-opt: [i, j]; 2 Or-opt-k: [min, max+k])
// meets a core interval of the other move widened by one position on the left
// unless the lower type is Or-opt, and on the right unless the higher type is
// Or-opt.  With e(t) = 0 for Or-opt and 1 otherwise that is
//   la <= hb + e(t_hi)  and  ha - e(t_lo) <= lb,
// i.e. [la, lb + e(t_lo)] and [ha, hb + e(t_hi)] intersect: widening every
// move's own intervals by e of its own type on the right makes the test
// symmetric and free of the types.  A shape packs the two right-widened
// intervals as four 16-bit fields (a1, b1, a2, b2); a pair conflicts iff one
// of its four interval pairs intersects.  Exhaustively equal to !canMerge
// over every move pair of small tours (tests/shape_conflict_check.cpp).
MLP_HD uint64_t move_shape(int id, int i, int j) {
  uint32_t a1, b1, a2, b2;
  if (id == 0) {
    a1 = (uint32_t)i; b1 = (uint32_t)i + 1u; a2 = (uint32_t)j; b2 = (uint32_t)j + 1u;
  } else if (id == 1) {
    a1 = a2 = (uint32_t)i; b1 = b2 = (uint32_t)j + 1u;
  } else {
    a1 = a2 = (uint32_t)imin_(i, j); b1 = b2 = (uint32_t)(imax_(i, j) + id - 1);
  }
  return (uint64_t)(a1 | (b1 << 16)) | ((uint64_t)(a2 | (b2 << 16)) << 32);
}
MLP_HD bool shapes_conflict(uint64_t s1, uint64_t s2) {
  const uint32_t p1 = (uint32_t)s1, p2 = (uint32_t)(s1 >> 32), q1 = (uint32_t)s2, q2 = (uint32_t)(s2 >> 32);
  const uint32_t pa1 = p1 & 0xffffu, pb1 = p1 >> 16, pa2 = p2 & 0xffffu, pb2 = p2 >> 16;
  const uint32_t qa1 = q1 & 0xffffu, qb1 = q1 >> 16, qa2 = q2 & 0xffffu, qb2 = q2 >> 16;
  return (pa1 <= qb1 && qa1 <= pb1) | (pa1 <= qb2 && qa2 <= pb1) | (pa2 <= qb1 && qa1 <= pb2) |
         (pa2 <= qb2 && qa2 <= pb2);
}

// ---------------- device job descriptor ----------------
// All pointers are device pointers.  Arrays of per-position data are padded
// to size + 8 entries (zero beyond size - 1).
struct JobDev {
  const int32_t* D;   // n x n distances (node ids)
  int32_t* tour;      // size
  int32_t* tour_alt;  // size (apply double buffer)
  int32_t* w;         // size + 8
  void* W;            // prefix of w: uint32 (int32 mode) or int64 (wide)
  void* Q;            // prefix of p * w[p]
  int32_t* A;         // 3 x (size + 8): A[k-1][p] = D[t[p-1]][t[p+k]]
  uint64_t* keys;     // total_blocks(size) candidate keys
  uint64_t* kept;     // total_blocks(size) stage-2 kept entries (packed)
  int32_t* kept_count;  // kNumNb counters
  uint8_t* ws;        // global workspace for large sizes (may be null)
  int64_t* stats;     // kStat* words
  uint32_t* moves_out;  // optional: applied moves (id | i << 4 | j << 18)
  int64_t* moves_cost;  // optional: applied move deltas
  int32_t moves_cap;
  int32_t n;
  int32_t size;
  int32_t nb_mask;    // neighbourhoods evaluated and merged
  int32_t flags;
  // TOTAL candidate mode (all null otherwise): the sweep appends every
  // improving move to its neighbourhood's list, the TOTAL greedy writes the
  // kept moves of neighbourhood nb at region_off(nb, size) + rank.
  void* tlist;        // list nb: total_list_cap(nb) keys at total_list_off(nb)
  int32_t* tcount;    // kNumNb list lengths
  int64_t* tkcost;    // kept moves: delta
  uint32_t* tkij;     // kept moves: i | j << 16
  int32_t* tkcount;   // kNumNb kept counts
  // Row and column terms of the DVND sweep (32-bit jobs; null otherwise):
  // kTermWords words per position p < size, rebuilt with the prefix arrays.
  int32_t* RT;
  int32_t* CT;
};

// The five deltas of a position pair (r, c), r < c, split into a term of r,
// a term of c and a few products of the pair's distances (all modulo 2^32).
// With sz = size, s_p = sz - p, w, W, Q, A the prefix arrays and
// V_k(p) = W[p+k-1] - W[p] (V_1 = 0, V_2 = w[p+1], V_3 = w[p+1] + w[p+2]):
//   S(p)    = -s_p w[p] - (s_p - 1) w[p+1]
//   row r:  RS = S(r);  R2 = -s_r w[r] - 2 Q[r] + (r + 1 + sz) W[r];
//           RF_k = s_r (A_k[r] - w[r]) - (s_r - k) w[r+k] + (r - sz) V_k(r) - k W[r+k];
//           RB_k = -s_r w[r] + k W[r];   then -W[r], V_2(r), V_3(r)
//   col c:  CS = S(c);  C2 = -(s_c - 1) w[c+1] + 2 Q[c] - (c + 1 + sz) W[c];
//           CF_k = -(s_c - k) w[c+k] + k W[c+k-1];
//           CB_k = (s_c - k)(A_k[c] - w[c+k]) - s_c w[c] + (c - sz) V_k(c) - k W[c-1];
//           then W[c], V_2(c), V_3(c)
// Words: 0 S, 1 R2 / C2, 2..4 RF_k / CF_k, 5..7 RB_k / CB_k, 8 -W[r] / W[c],
// 9 V_2, 10 V_3, 11 zero.  The sweep's deltas from them are given where it
// evaluates them (k_sweep_dvnd).
constexpr int kTermWords = 12;

#ifdef __CUDACC__
// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization (launch_pdl) may start while its stream predecessor still
// runs: pdl_wait() returns once the predecessor has completed and its memory
// operations are visible; pdl_launch_dependents() lets the stream successor,
// if launched the same way, start early.  Both do nothing in an ordinary
// launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Inputs of position p's terms: w[p..p+3] (zero at and beyond size), W[p],
// Q[p] and A_k[p], all modulo 2^32.
struct TermIn {
  uint32_t w0, w1, w2, w3, W, Q, A1, A2, A3;
};
__device__ __forceinline__ void row_terms(const TermIn& x, int p, int sz, int4& o0, int4& o1, int4& o2) {
  const uint32_t up = (uint32_t)p, usz = (uint32_t)sz, sp = usz - up, upsz = up - usz;
  const uint32_t W1 = x.W + x.w1, W2 = W1 + x.w2, W3 = W2 + x.w3, V2 = x.w1, V3 = x.w1 + x.w2;
  const uint32_t S = 0u - sp * x.w0 - (sp - 1u) * x.w1, RB0 = 0u - sp * x.w0;
  o0 = make_int4((int)S, (int)(RB0 - 2u * x.Q + (up + 1u + usz) * x.W), (int)(sp * (x.A1 - x.w0) - (sp - 1u) * x.w1 - W1),
                 (int)(sp * (x.A2 - x.w0) - (sp - 2u) * x.w2 + upsz * V2 - 2u * W2));
  o1 = make_int4((int)(sp * (x.A3 - x.w0) - (sp - 3u) * x.w3 + upsz * V3 - 3u * W3), (int)(RB0 + x.W),
                 (int)(RB0 + 2u * x.W), (int)(RB0 + 3u * x.W));
  o2 = make_int4((int)(0u - x.W), (int)V2, (int)V3, 0);
}
__device__ __forceinline__ void col_terms(const TermIn& x, int p, int sz, int4& o0, int4& o1, int4& o2) {
  const uint32_t up = (uint32_t)p, usz = (uint32_t)sz, sp = usz - up, upsz = up - usz;
  const uint32_t Wm1 = x.W - x.w0, W1 = x.W + x.w1, W2 = W1 + x.w2, V2 = x.w1, V3 = x.w1 + x.w2;
  const uint32_t S = 0u - sp * x.w0 - (sp - 1u) * x.w1, RB0 = 0u - sp * x.w0;
  o0 = make_int4((int)S, (int)(0u - (sp - 1u) * x.w1 + 2u * x.Q - (up + 1u + usz) * x.W),
                 (int)(0u - (sp - 1u) * x.w1 + x.W), (int)(0u - (sp - 2u) * x.w2 + 2u * W1));
  o1 = make_int4((int)(0u - (sp - 3u) * x.w3 + 3u * W2), (int)((sp - 1u) * (x.A1 - x.w1) + RB0 - Wm1),
                 (int)((sp - 2u) * (x.A2 - x.w2) + RB0 + upsz * V2 - 2u * Wm1),
                 (int)((sp - 3u) * (x.A3 - x.w3) + RB0 + upsz * V3 - 3u * Wm1));
  o2 = make_int4((int)x.W, (int)V2, (int)V3, 0);
}
#endif

enum : int {
  kStatCost = 0,       // current cost (int64, or uint32 zero-extended)
  kStatIters = 1,      // iterations that applied moves
  kStatMoves = 2,      // moves applied (total)
  kStatConverged = 3,  // 1 once an iteration found no improving candidate
  kStatLastMoves = 4,  // moves applied by the last iteration
  kStatDone = 5,       // stage-2 CTA arrival counter
  kStatSweeps = 6,     // sweeps run
  kStatError = 7,      // nonzero: device-detected error
  kStatLimit = 8,      // sweeps allowed (kernels become no-ops past it)
  kStatWords = 16
};

enum : int { kFlagWide = 1, kFlagRecordMoves = 2 };

// Sweep work item: one parallelogram tile of the (row r, diagonal L) plane.
struct SweepTile {
  int32_t job;
  int32_t r0;
  int32_t L0;
  int32_t pad;
};

// Tiles of one job's sweep with tl diagonals x tr rows: row blocks start at
// r0 = 1, 1 + tr, ... <= size - 3, and row block r0 holds the tiles
// L0 = 1, 1 + tl, ... with r0 + L0 <= size - 2.  Every tile list (the
// engine's job sets, the allocation-free evaluation) is built from these.
MLP_HD int sweep_row_blocks(int size, int tr) { return size >= 4 ? (size - 3 + tr - 1) / tr : 0; }
MLP_HD int sweep_row_tiles(int size, int r0, int tl) { return r0 <= size - 3 ? (size - 2 - r0 + tl - 1) / tl : 0; }
MLP_HD int sweep_tiles(int size, int tl, int tr) {
  int c = 0;
  for (int rb = 0; rb < sweep_row_blocks(size, tr); rb++) c += sweep_row_tiles(size, 1 + rb * tr, tl);
  return c;
}

}  // namespace mlp
