// mlp_kernels.cu -- CUDA kernels of the GB300 MLP local-search engine (sm_103a).
//
// Data path of one DVND iteration (see mlp_engine.cpp for the host side):
//   k_sweep   all five neighbourhoods (swap, 2-opt, Or-opt-1/2/3) over the
//             tour, tiled over (row r, diagonal L = c - r) parallelograms; one
//             64-bit (delta, ctx) key per reference block via atomicMin.
//   k_merge   a cluster of six CTAs per job: five run the stage-2 greedy
//             independent set of one neighbourhood each (the reference's
//             per-kernel GPU merge) and pass the kept moves to the sixth over
//             distributed shared memory; it runs the cross-neighbourhood
//             greedy, applies the selected moves, rebuilds w / prefix arrays /
//             cost and resets the candidate keys.
//   k_prepare the ADS prefix rebuild alone (after a new tour is set).
//
// All arithmetic is integer.  In int32 mode every delta and cost is computed in
// uint32 modular arithmetic, which reproduces the reference's 32-bit wrap-around
// results exactly; in wide mode everything is int64.
#include <cooperative_groups.h>

#include <cstdint>

#include "mlp_common.cuh"
#include "mlp_kernels.cuh"

namespace mlp {

namespace cg = cooperative_groups;

namespace {

constexpr unsigned kFull = 0xffffffffu;

template <bool WIDE>
struct Arith;
template <>
struct Arith<false> {
  using C = uint32_t;  // modular arithmetic type
  using V = int32_t;   // value type of a delta
  static constexpr int32_t kInf = 0x7fffffff;
};
template <>
struct Arith<true> {
  using C = int64_t;
  using V = int64_t;
  static constexpr int64_t kInf = 0x7fffffffffffffffLL;
};

__host__ __device__ __forceinline__ size_t align_up(size_t v, size_t a) {
  return (v + a - 1) / a * a;
}

// Block-wide exclusive scan of one value per thread; `total` receives the sum.
// blockDim.x must be a multiple of 32.  `sm` holds 32 entries.
template <typename T>
__device__ T block_exclusive_scan(T v, T* sm, T& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[wid] = x;
  __syncthreads();
  if (wid == 0) {
    T s = lane < nw ? sm[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(kFull, s, o);
      if (lane >= o) s += y;
    }
    sm[lane] = s;
  }
  __syncthreads();
  const T before = wid > 0 ? sm[wid - 1] : T(0);
  total = sm[nw - 1];
  __syncthreads();
  return before + x - v;
}

// Three block-wide scans at once (one set of barriers): exclusive prefixes of
// a and b, totals of a, b and c.
template <typename T>
__device__ void block_exclusive_scan3(T a, T b, T c, T* sa, T* sb, T* sc, T& ea, T& eb, T& ta, T& tb,
                                      T& tc) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  T xa = a, xb = b, xc = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T ya = __shfl_up_sync(kFull, xa, o), yb = __shfl_up_sync(kFull, xb, o),
            yc = __shfl_up_sync(kFull, xc, o);
    if (lane >= o) {
      xa += ya;
      xb += yb;
      xc += yc;
    }
  }
  if (lane == 31) {
    sa[wid] = xa;
    sb[wid] = xb;
    sc[wid] = xc;
  }
  __syncthreads();
  if (wid == 0) {
    T pa = lane < nw ? sa[lane] : T(0), pb = lane < nw ? sb[lane] : T(0), pc = lane < nw ? sc[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T ya = __shfl_up_sync(kFull, pa, o), yb = __shfl_up_sync(kFull, pb, o),
              yc = __shfl_up_sync(kFull, pc, o);
      if (lane >= o) {
        pa += ya;
        pb += yb;
        pc += yc;
      }
    }
    sa[lane] = pa;
    sb[lane] = pb;
    sc[lane] = pc;
  }
  __syncthreads();
  ea = (wid > 0 ? sa[wid - 1] : T(0)) + xa - a;
  eb = (wid > 0 ? sb[wid - 1] : T(0)) + xb - b;
  ta = sa[nw - 1];
  tb = sb[nw - 1];
  tc = sc[nw - 1];
  __syncthreads();
}

// Row and column terms of position p (mlp_common.cuh, kTermWords), from
// w (w_s: the job's sz weights), W[p], Q[p] and A; 32-bit modular arithmetic.
__device__ __forceinline__ void write_terms(const JobDev* J, int p, int sz, const int32_t* w_s, uint32_t Wp,
                                            uint32_t Qp, const int32_t* A, int pad) {
  TermIn x;
  x.w0 = (uint32_t)w_s[p];
  x.w1 = p + 1 < sz ? (uint32_t)w_s[p + 1] : 0u;
  x.w2 = p + 2 < sz ? (uint32_t)w_s[p + 2] : 0u;
  x.w3 = p + 3 < sz ? (uint32_t)w_s[p + 3] : 0u;
  x.W = Wp;
  x.Q = Qp;
  x.A1 = (uint32_t)A[p];
  x.A2 = (uint32_t)A[pad + p];
  x.A3 = (uint32_t)A[2 * pad + p];
  int4* rt = reinterpret_cast<int4*>(J->RT + (size_t)p * kTermWords);
  int4* ct = reinterpret_cast<int4*>(J->CT + (size_t)p * kTermWords);
  row_terms(x, p, sz, rt[0], rt[1], rt[2]);
  col_terms(x, p, sz, ct[0], ct[1], ct[2]);
}

// --------------------------------------------------------------------------
// ADS prefix rebuild: w[p] = D[t[p-1]][t[p]], W = prefix(w), Q = prefix(p w),
// A[k-1][p] = D[t[p-1]][t[p+k]], cost = sum (size - p) w[p]
// (source/mlsolution.cpp:216-228 and :454-458 for T = W).  With t_prev, the
// tour that J->w and J->A currently describe, a position whose window
// t[p-1 .. p+3] is unchanged keeps its w and A (no distance gathers); w_prev,
// when given, is a copy of J->w to read those from.  With src as well
// (t[p] = t_prev[src[p]], the applied moves' position map) every weight and
// skip distance whose two clients were already kt + 1 positions apart in the
// old tour, in either order (D is symmetric), is taken from the old arrays:
// inside a reversed or shifted segment nothing is gathered, only around its
// ends.  Every value is read before any is written (two phases).
// --------------------------------------------------------------------------
constexpr int kPrepMaxPer = 4;  // positions per thread of the two-phase rebuild

template <bool WIDE>
__device__ __forceinline__ void cta_prepare(const JobDev* J, const int32_t* t_override, int32_t* w_s,
                                            const int32_t* t_prev = nullptr, const int32_t* w_prev = nullptr,
                                            const int32_t* src = nullptr) {
  using C = typename Arith<WIDE>::C;
  __shared__ C smW[32], smQ[32], smC[32];
  const int sz = J->size, n = J->n, pad = sz + 8;
  const int32_t* __restrict__ t = t_override ? t_override : J->tour;
  const int32_t* __restrict__ D = J->D;
  int32_t* w = J->w;
  int32_t* A = J->A;
  C* W = (C*)J->W;
  C* Q = (C*)J->Q;
  const int nt = blockDim.x;
  const int chunk = (sz + nt - 1) / nt;
  const int p0 = threadIdx.x * chunk;
  const int p1 = min(sz, p0 + chunk);
  auto gather = [&](int p) {
    if (t_prev != nullptr) {
      bool same = true;
#pragma unroll
      for (int d = -1; d <= 3; d++) {
        const int q = p + d;
        if (q >= 0 && q < sz) same &= t[q] == t_prev[q];
      }
      if (same) {
        const int32_t wp = w_prev != nullptr ? w_prev[p] : w[p];
        w_s[p] = wp;
        return wp;
      }
    }
    const int32_t prev = p > 0 ? t[p - 1] : 0;
    const int32_t wp = p > 0 ? D[(size_t)prev * n + t[p]] : 0;
    w[p] = wp;
    w_s[p] = wp;
#pragma unroll
    for (int k = 1; k <= 3; k++)
      A[(k - 1) * pad + p] = (p >= 1 && p + k <= sz - 1) ? D[(size_t)prev * n + t[p + k]] : 0;
    return wp;
  };
  C sW = 0, sQ = 0, sC = 0;
  if (src != nullptr && t_prev != nullptr && chunk <= kPrepMaxPer) {
    // Phase 1: the new w and A of this thread's positions (p = tid + u nt).
    int32_t nw[kPrepMaxPer], na[kPrepMaxPer][3];
    bool keep[kPrepMaxPer];
#pragma unroll
    for (int u = 0; u < kPrepMaxPer; u++) {
      const int p = threadIdx.x + u * nt;
      keep[u] = true;
      nw[u] = 0;
      na[u][0] = na[u][1] = na[u][2] = 0;
      if (u >= chunk || p >= sz || p == 0) continue;
      const int qa = src[p - 1], qb = src[p];
      if (qb == qa + 1) {
        nw[u] = w_prev != nullptr ? w_prev[qb] : w[qb];
      } else if (qa == qb + 1) {
        nw[u] = w_prev != nullptr ? w_prev[qa] : w[qa];
      } else {
        nw[u] = D[(size_t)t[p - 1] * n + t[p]];
      }
      bool same = qa == p - 1 && qb == p;
#pragma unroll
      for (int k = 1; k <= 3; k++) {
        if (p + k > sz - 1) continue;
        const int qc = src[p + k];
        same &= qc == p + k;
        if (qc == qa + k + 1) na[u][k - 1] = A[(k - 1) * pad + qa + 1];
        else if (qa == qc + k + 1) na[u][k - 1] = A[(k - 1) * pad + qc + 1];
        else na[u][k - 1] = D[(size_t)t[p - 1] * n + t[p + k]];
      }
      keep[u] = same;  // window unchanged: the stored values stand
    }
    __syncthreads();
    // Phase 2: stores (only where something changed) and the staged w.
#pragma unroll
    for (int u = 0; u < kPrepMaxPer; u++) {
      const int p = threadIdx.x + u * nt;
      if (u >= chunk || p >= sz) continue;
      w_s[p] = nw[u];
      if (keep[u]) continue;
      w[p] = nw[u];
#pragma unroll
      for (int k = 0; k < 3; k++) A[k * pad + p] = na[u][k];
    }
    __syncthreads();
    for (int p = p0; p < p1; p++) {
      const C wp = (C)w_s[p];
      sW += wp;
      sQ += (C)p * wp;
      sC += (C)(sz - p) * wp;
    }
  } else if (chunk == 1) {  // one position per thread at most
    if (p0 < p1) {
      const C wp = (C)gather(p0);
      sW = wp;
      sQ = (C)p0 * wp;
      sC = (C)(sz - p0) * wp;
    }
  } else {
    // Gathers first, strided so that each thread's positions are independent
    // (several in flight); then the per-thread contiguous chunks of the scan.
#pragma unroll 4
    for (int p = threadIdx.x; p < sz; p += nt) gather(p);
    __syncthreads();
    for (int p = p0; p < p1; p++) {
      const C wp = (C)w_s[p];
      sW += wp;
      sQ += (C)p * wp;
      sC += (C)(sz - p) * wp;
    }
  }
  C totW, totQ, totC, eW, eQ;
  block_exclusive_scan3<C>(sW, sQ, sC, smW, smQ, smC, eW, eQ, totW, totQ, totC);
  for (int p = p0; p < p1; p++) {
    const C wp = (C)w_s[p];
    eW += wp;
    eQ += (C)p * wp;
    W[p] = eW;
    Q[p] = eQ;
    if constexpr (!WIDE) {
      if (J->RT != nullptr) write_terms(J, p, sz, w_s, eW, eQ, A, pad);
    }
  }
  for (int p = sz + threadIdx.x; p < pad; p += nt) {
    w[p] = 0;
    W[p] = totW;
    Q[p] = totQ;
#pragma unroll
    for (int k = 0; k < 3; k++) A[k * pad + p] = 0;
  }
  if (threadIdx.x == 0) J->stats[kStatCost] = WIDE ? (int64_t)totC : (int64_t)(uint32_t)totC;
}

__device__ void cta_reset_keys(const JobDev* J) {
  const int tb = total_blocks(J->size);
  for (int q = threadIdx.x; q < tb; q += blockDim.x) J->keys[q] = kKeyNone;
  if (J->tcount != nullptr && threadIdx.x < kNumNb) J->tcount[threadIdx.x] = 0;
}

template <bool WIDE>
__global__ void __launch_bounds__(1024) k_prepare(const JobDev* __restrict__ jobs, int reset_stats) {
  extern __shared__ int32_t prep_w[];
  const JobDev* J = jobs + blockIdx.x;
  if (reset_stats && threadIdx.x < kStatWords) {
    const int q = threadIdx.x;
    if (q != kStatLimit) J->stats[q] = 0;
  }
  cta_prepare<WIDE>(J, nullptr, prep_w);
  cta_reset_keys(J);
}

// --------------------------------------------------------------------------
// Sweep.  A tile covers rows r in [r0, r0+TR) and diagonals L in [L0, L0+TL)
// of the position-pair plane (r < c = r + L).  Thread `tid` owns diagonal
// L = L0 + tid and walks the rows.  For each pair it evaluates, with the ODC
// kernels' formulas rewritten over prefix sums:
//   swap(i=r, j=c)        mlkswap.cu:770-785
//   2opt(i=r, j=c)        mlk2opt.cu:565-571
//   oropt-k(i=r, j=c)     mlkoropt.cu:704-716   (forward)
//   oropt-k(i=c, j=r)     mlkoropt.cu:724-736   (backward)
// Distances E(x, y) = D[t[x]][t[y]] of the tile are staged in shared memory
// in skewed layout S[a][b] = E(r0-1+a, r0-1+a + L0-1+b).
// Reference block attribution (which block of the reference grid evaluates
// the pair, and with which thread index ctx):
//   swap   A: by = r-1, ctx = c-3          B: by = size-3-r, ctx = size-2-c
//   2opt   A: by = L-1, ctx = c-2          B: by = size-2-L, ctx = size-2-c
//   fwd-k     by = L-1, ctx = c-2
//   bwd-k     by = size-k-1-L, ctx = size-k-1-c
// --------------------------------------------------------------------------
template <bool WIDE, int TL, int TR, bool COLLECT = false>
__global__ void __launch_bounds__(TL) k_sweep(const SweepTile* __restrict__ tiles,
                                              const JobDev* __restrict__ jobs, int improve_only) {
  using Ar = Arith<WIDE>;
  using C = typename Ar::C;
  using V = typename Ar::V;
  constexpr V kInf = Ar::kInf;
  constexpr int SR = TR + 3, SC = TL + 3, NR = TR + 4, NC = TR + TL + 4, NT = TR + TL + 5;
  __shared__ int32_t sS[SR][SC];
  __shared__ int32_t sRowT[SR];
  __shared__ int32_t sColT[NT];
  __shared__ int32_t sRw[NR];
  __shared__ int32_t sRA[3][NR];
  __shared__ C sRW[NR];
  __shared__ C sRQ[NR];
  __shared__ int32_t sCw[NC];
  __shared__ int32_t sCA[3][NC];
  __shared__ C sCW[NC];
  __shared__ C sCQ[NC];

  const SweepTile tile = tiles[blockIdx.x];
  const JobDev* J = jobs + tile.job;
  const int64_t* stats = J->stats;
  const int sz = J->size, n = J->n, mask = J->nb_mask;
  const int r0 = tile.r0, L0 = tile.L0, tid = threadIdx.x;
  const int pad = sz + 8;
  const int32_t* __restrict__ t = J->tour;
  const int32_t* __restrict__ D = J->D;
  const int32_t* __restrict__ w = J->w;
  const int32_t* __restrict__ Ag = J->A;
  const C* __restrict__ W = (const C*)J->W;
  const C* __restrict__ Q = (const C*)J->Q;
  // In a programmatic launch (the TOTAL iteration's collecting sweep) the
  // previous iteration has completed past this point; the TOTAL greedy may
  // then be launched.  A job that converged or used its sweep limit is
  // skipped before its distance gathers.
  pdl_wait();
  pdl_launch_dependents();
  const bool done = stats[kStatConverged] || stats[kStatSweeps] >= stats[kStatLimit];

  {
    // Tour positions and per-position arrays of the tile's rows and columns:
    // every load is issued before any is stored, so the tile pays one L2
    // round trip here instead of one per array.
    constexpr int kSR = (SR + TL - 1) / TL, kNT = (NT + TL - 1) / TL;
    constexpr int kNR = (NR + TL - 1) / TL, kNC = (NC + TL - 1) / TL;
    int32_t vRT[kSR], vCT[kNT], vRw[kNR], vRA[3][kNR], vCw[kNC], vCA[3][kNC];
    C vRW[kNR], vRQ[kNR], vCW[kNC], vCQ[kNC];
#pragma unroll
    for (int u = 0; u < kSR; u++) {
      const int q = tid + u * TL, p = r0 - 1 + q;
      vRT[u] = (q < SR && p <= sz - 1) ? t[p] : 0;
    }
#pragma unroll
    for (int u = 0; u < kNT; u++) {
      const int q = tid + u * TL, p = r0 + L0 - 2 + q;
      vCT[u] = (q < NT && p <= sz - 1) ? t[p] : 0;
    }
#pragma unroll
    for (int u = 0; u < kNR; u++) {
      const int q = tid + u * TL, p = r0 + q;
      const bool ok = q < NR && p < pad;
      vRw[u] = ok ? w[p] : 0;
      vRW[u] = ok ? W[p] : C(0);
      vRQ[u] = ok ? Q[p] : C(0);
#pragma unroll
      for (int k = 0; k < 3; k++) vRA[k][u] = ok ? Ag[k * pad + p] : 0;
    }
#pragma unroll
    for (int u = 0; u < kNC; u++) {
      const int q = tid + u * TL, p = r0 + L0 - 1 + q;
      const bool ok = q < NC && p < pad;
      vCw[u] = ok ? w[p] : 0;
      vCW[u] = ok ? W[p] : C(0);
      vCQ[u] = ok ? Q[p] : C(0);
#pragma unroll
      for (int k = 0; k < 3; k++) vCA[k][u] = ok ? Ag[k * pad + p] : 0;
    }
#pragma unroll
    for (int u = 0; u < kSR; u++) {
      const int q = tid + u * TL;
      if (q < SR) sRowT[q] = vRT[u];
    }
#pragma unroll
    for (int u = 0; u < kNT; u++) {
      const int q = tid + u * TL;
      if (q < NT) sColT[q] = vCT[u];
    }
#pragma unroll
    for (int u = 0; u < kNR; u++) {
      const int q = tid + u * TL;
      if (q < NR) {
        sRw[q] = vRw[u];
        sRW[q] = vRW[u];
        sRQ[q] = vRQ[u];
#pragma unroll
        for (int k = 0; k < 3; k++) sRA[k][q] = vRA[k][u];
      }
    }
#pragma unroll
    for (int u = 0; u < kNC; u++) {
      const int q = tid + u * TL;
      if (q < NC) {
        sCw[q] = vCw[u];
        sCW[q] = vCW[u];
        sCQ[q] = vCQ[u];
#pragma unroll
        for (int k = 0; k < 3; k++) sCA[k][q] = vCA[k][u];
      }
    }
  }
  __syncthreads();
  if (done) return;
  {
    // All gathers of the tile are issued before any is stored, so their
    // latencies overlap (one L2/HBM round trip per tile instead of one per load).
    // At most GB loads per thread in flight at once (bounds the registers of
    // the tallest tiles; every other shape needs a single batch).
    constexpr int NG = (SR * SC + TL - 1) / TL, GB = 21;
#pragma unroll
    for (int u0 = 0; u0 < NG; u0 += GB) {
      int32_t gv[GB];
#pragma unroll
      for (int u = 0; u < GB; u++) {
        const int idx = tid + (u0 + u) * TL;
        int32_t v = 0;
        if (u0 + u < NG && idx < SR * SC) {
          const int a = idx / SC, b = idx - a * SC;
          const int rp = r0 - 1 + a, cp = rp + L0 - 1 + b;
          if (rp <= sz - 1 && cp <= sz - 1) v = __ldg(D + (size_t)sRowT[a] * n + sColT[a + b]);
        }
        gv[u] = v;
      }
#pragma unroll
      for (int u = 0; u < GB; u++) {
        const int idx = tid + (u0 + u) * TL;
        if (u0 + u < NG && idx < SR * SC) {
          const int a = idx / SC, b = idx - a * SC;
          sS[a][b] = gv[u];
        }
      }
    }
  }
  __syncthreads();

  uint64_t* keys = J->keys;
  const int L = L0 + tid, b = tid + 1, lane = tid & 31;
  const int nbS = nb_blocks(0, sz), nb2 = nb_blocks(1, sz);
  const int off0 = 0, off1 = nb_offset(1, sz);
  const bool mSw = mask & 1, m2o = mask & 2;
  const bool has2A = (L - 1) < nb2;
  const int blk2B = sz - 2 - L;
  const bool has2B = blk2B >= 0 && blk2B < nb2;
  V b2A = kInf, b2B = kInf, bF[3] = {kInf, kInf, kInf}, bB[3] = {kInf, kInf, kInf};
  int c2A = -1, c2B = -1, cF[3] = {-1, -1, -1}, cB[3] = {-1, -1, -1};
  // E(x, y) around the pair (r, c) of row a; the four that row a + 1 shares
  // with row a are carried in registers.
  int32_t sM1P1 = sS[0][b + 1];  // E(r-1, c)
  int32_t s0M1 = sS[1][b - 1];   // E(r, c-1)
  int32_t s0P1 = sS[1][b + 1];   // E(r, c+1)
  int32_t sP1P1 = sS[2][b + 1];  // E(r+1, c+2)
  // 64-bit costs: every factor of every product fits 32 bits (distances and
  // weights <= 65535, positions < 16384, W <= 16392 * 65535 < 2^31), so each
  // product is one exact widening multiply(-add) instead of a 64 x 64 one.
  auto mw = [](int32_t x, int32_t y) -> int64_t { return (int64_t)x * (int64_t)y; };
  // TOTAL candidate mode: every improving move (i, j) of neighbourhood nb is
  // appended to nb's list, one atomic per warp and neighbourhood (every lane
  // of the warp calls this at the same point).
  auto emit = [&](int nb, bool p, V d, int i, int j) {
    const unsigned bal = __ballot_sync(kFull, p);
    if (bal == 0) return;
    const int leader = __ffs(bal) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&J->tcount[nb], __popc(bal));
    base = __shfl_sync(kFull, base, leader);
    if (!p) return;
    const int64_t pos = (int64_t)base + __popc(bal & ((1u << lane) - 1u));
    if (pos >= total_list_cap(nb, sz)) return;  // the TOTAL greedy reports the overflow
    const int64_t at = total_list_off(nb, sz) + pos;
    if constexpr (WIDE) ((u128*)J->tlist)[at] = total_key64((int64_t)d, i, j);
    else ((uint64_t*)J->tlist)[at] = total_key32((int32_t)d, i, j);
  };
#pragma unroll 1
  for (int a = 1; a <= TR; a++) {
    const int r = r0 + a - 1;
    if (r > sz - 3) break;  // uniform across the CTA
    const int c = r + L;
    const bool vpair = c <= sz - 2;
    const int qr = a - 1, qc = a + tid;
    const int32_t sP1M1 = sS[a + 1][b - 1];  // E(r+1, c)
    const int32_t s00 = sS[a][b];            // E(r, c)
    const int32_t s0P2 = sS[a][b + 2];       // E(r, c+2)
    const int32_t sP2P1 = sS[a + 2][b + 1];  // E(r+2, c+3)
    const int32_t wr0 = sRw[qr], wr1 = sRw[qr + 1];
    const int32_t wc0 = sCw[qc], wc1 = sCw[qc + 1];
    const int iszr = sz - r, iszc = sz - c;
    const C szr = (C)iszr, szc = (C)iszc;

    // ---- swap (row-owned blocks): warp argmin per row ----
    if (mSw) {
      const bool v = vpair && L >= 2;
      V d;
      if constexpr (WIDE)
        d = mw(iszr, sM1P1 - wr0) + mw(iszr - 1, sP1M1 - wr1) + mw(iszc, s0M1 - wc0) + mw(iszc - 1, s0P1 - wc1);
      else
        d = (V)(szr * ((C)sM1P1 - (C)wr0) + (szr - C(1)) * ((C)sP1M1 - (C)wr1) + szc * ((C)s0M1 - (C)wc0) +
                (szc - C(1)) * ((C)s0P1 - (C)wc1));
      if constexpr (COLLECT) {
        emit(0, v && d < 0, d, r, c);
      } else {
      const int blkA = r - 1, blkB = sz - 3 - r;
      const bool hasA = blkA < nbS, hasB = blkB >= 0 && blkB < nbS;
      unsigned ties;
      bool any;
      if (!WIDE) {
        const uint32_t u = (v && d != kInf) ? ((uint32_t)d ^ 0x80000000u) : 0xffffffffu;
        const uint32_t mn = __reduce_min_sync(kFull, u);
        any = improve_only ? mn < 0x80000000u : mn != 0xffffffffu;
        ties = __ballot_sync(kFull, u == mn);
      } else {
        const uint64_t u = v ? (uint64_t)((int64_t)d + (int64_t)kCostBias) : ~0ull;
        const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
        const uint32_t mh = __reduce_min_sync(kFull, hi);
        const uint32_t ml = __reduce_min_sync(kFull, hi == mh ? lo : 0xffffffffu);
        const uint64_t mn = ((uint64_t)mh << 32) | ml;
        any = improve_only ? mn < kCostBias : mn != ~0ull;
        ties = __ballot_sync(kFull, hi == mh && lo == ml);
      }
      if (any) {
        if (hasA && lane == __ffs(ties) - 1)
          atomicMin((unsigned long long*)&keys[off0 + blkA],
                    (unsigned long long)make_key((int64_t)d, (uint32_t)(c - 3), kCtxBits));
        if (hasB && lane == 31 - __clz(ties))
          atomicMin((unsigned long long*)&keys[off0 + blkB],
                    (unsigned long long)make_key((int64_t)d, (uint32_t)(sz - 2 - c), kCtxBits));
      }
      }
    }

    // ---- 2-opt (diagonal-owned blocks) ----
    if (m2o && (COLLECT || vpair)) {
      V d;
      if constexpr (WIDE)
        d = mw(iszr, sM1P1 - wr0) + mw(iszc - 1, s0P1 - wc1) + 2 * ((int64_t)sCQ[qc] - (int64_t)sRQ[qr]) -
            mw(r + c + 1, (int32_t)sCW[qc] - (int32_t)sRW[qr]);
      else
        d = (V)(szr * ((C)sM1P1 - (C)wr0) + (szc - C(1)) * ((C)s0P1 - (C)wc1) + C(2) * (sCQ[qc] - sRQ[qr]) -
                (C)(r + c + 1) * (sCW[qc] - sRW[qr]));
      if constexpr (COLLECT) emit(1, vpair && d < 0, d, r, c);
      else if (has2A && d < b2A) {
        b2A = d;
        c2A = c;
      }
      if (has2B && d <= b2B && d != kInf) {
        b2B = d;
        c2B = c;
      }
    }

    // ---- Or-opt-k forward (i=r, j=c) and backward (i=c, j=r) ----
#pragma unroll
    for (int k = 1; k <= 3; k++) {
      if (!((mask >> (k + 1)) & 1)) continue;
      const bool vk = c + k <= sz - 1;
      if (!COLLECT && !vk) continue;
      const int32_t Sf = k == 1 ? s0P1 : (k == 2 ? sP1P1 : sP2P1);  // E(r+k-1, c+k)
      const int32_t Sg = k == 1 ? s00 : (k == 2 ? s0P1 : s0P2);     // E(r, c+k-1)
      const int32_t wrk = sRw[qr + k], wck = sCw[qc + k];
      {
        V d;
        if constexpr (WIDE) {
          const int32_t Wr0 = (int32_t)sRW[qr];
          d = mw(iszr, sRA[k - 1][qr] - wr0) + mw(iszc - k, Sf - wck) + mw(iszc, Sg) - mw(iszr - k, wrk) +
              mw(r - c, (int32_t)sRW[qr + k - 1] - Wr0) + mw(k, (int32_t)sCW[qc + k - 1] - (int32_t)sRW[qr + k]);
        } else {
          const C kk = (C)k;
          d = (V)(szr * ((C)sRA[k - 1][qr] - (C)wr0) + (szc - kk) * ((C)Sf - (C)wck) + szc * (C)Sg -
                  (szr - kk) * (C)wrk + ((C)r - (C)c) * (sRW[qr + k - 1] - sRW[qr]) +
                  kk * (sCW[qc + k - 1] - sRW[qr + k]));
        }
        if constexpr (COLLECT) {
          emit(k + 1, vk && d < 0, d, r, c);
        } else if (d < bF[k - 1]) {
          bF[k - 1] = d;
          cF[k - 1] = c;
        }
      }
      if (COLLECT || L >= 2) {
        V d;
        if constexpr (WIDE) {
          const int32_t Wc0 = (int32_t)sCW[qc];
          d = mw(iszr, sM1P1 - wr0) + mw(iszc - k, sCA[k - 1][qc] - wck) + mw(iszr - k, Sg) - mw(iszc, wc0) +
              mw(c - r, (int32_t)sCW[qc + k - 1] - Wc0) - mw(k, (int32_t)sCW[qc - 1] - (int32_t)sRW[qr]);
        } else {
          const C kk = (C)k;
          d = (V)(szr * ((C)sM1P1 - (C)wr0) + (szc - kk) * ((C)sCA[k - 1][qc] - (C)wck) + (szr - kk) * (C)Sg -
                  szc * (C)wc0 + (C)(c - r) * (sCW[qc + k - 1] - sCW[qc]) - kk * (sCW[qc - 1] - sRW[qr]));
        }
        if constexpr (COLLECT) {
          emit(k + 1, vk && L >= 2 && d < 0, d, c, r);
        } else if (d <= bB[k - 1] && d != kInf) {
          bB[k - 1] = d;
          cB[k - 1] = c;
        }
      }
    }
    sM1P1 = s0P1;
    s0M1 = sP1M1;
    s0P1 = sP1P1;
    sP1P1 = sP2P1;
  }

  // DVND sweeps publish improving candidates only (the merge ignores the
  // rest); evaluation sweeps publish every block's best.
  if constexpr (COLLECT) return;

  if (c2A >= 0 && (!improve_only || b2A < 0))
    atomicMin((unsigned long long*)&keys[off1 + (L - 1)],
              (unsigned long long)make_key((int64_t)b2A, (uint32_t)(c2A - 2), kCtxBits));
  if (c2B >= 0 && (!improve_only || b2B < 0))
    atomicMin((unsigned long long*)&keys[off1 + blk2B],
              (unsigned long long)make_key((int64_t)b2B, (uint32_t)(sz - 2 - c2B), kCtxBits));
#pragma unroll
  for (int k = 1; k <= 3; k++) {
    const int offk = nb_offset(k + 1, sz);
    if (cF[k - 1] >= 0 && (!improve_only || bF[k - 1] < 0))
      atomicMin((unsigned long long*)&keys[offk + (L - 1)],
                (unsigned long long)make_key((int64_t)bF[k - 1], (uint32_t)(cF[k - 1] - 2), kCtxBits));
    if (cB[k - 1] >= 0 && (!improve_only || bB[k - 1] < 0))
      atomicMin((unsigned long long*)&keys[offk + (sz - k - 1 - L)],
                (unsigned long long)make_key((int64_t)bB[k - 1], (uint32_t)(sz - k - 1 - cB[k - 1]),
                                             kCtxBits));
  }
}

// --------------------------------------------------------------------------
// Merge.
// --------------------------------------------------------------------------
enum : uint8_t { kNone = 0, kUndec = 1, kIn = 2, kOut = 3 };

// Stage-2 candidate record: one 128-bit shared-memory access per candidate.
struct __align__(16) Rec {
  uint64_t key;  // (delta, block) order key
  uint32_t ab;   // swap: i | j << 16; 2-opt / Or-opt: conflict interval a | b << 16
  uint32_t st;   // kNone / kUndec / kIn / kOut
};
constexpr int kBitMax = 512;         // stage-3 conflict bit-matrix capacity (moves)
constexpr int kBitMaxWs = 4096;      // the same in a global merge workspace (large tours: 2 MB)
constexpr int kWarpRoundWords = 4;   // stage-3 lists up to 128 moves: one-warp rounds
constexpr int kMergeThreads = 1024;
constexpr int kClusterCtas = 6;  // five stage-2 CTAs and the stage-3 leader
// Dynamic shared memory a merge workspace may use: the 227 KB opt-in limit
// less room for the kernels' static shared memory.
constexpr size_t kMergeSmemLimit = 227 * 1024 - 4096;

// Workspace layout (bytes) of the merge CTA of a job of a given size.
//   A: per-candidate key / move / state of the five neighbourhoods (stage 2);
//      reused for the apply owner map once stage 3 has compacted the kept set
//   B: swap endpoint tables (stage 2), then the stage-3 move list and bit rows
//   T: the old and the new tour

struct MergeLayout {
  int tb, mmax, m3cap;
  // stage-2 CTA: records, moves, swap tables
  size_t o_ij2, o_tab, s2;
  // leader: stage-3 list, conflict bits, owner map, old and new tour
  size_t o_key3, o_shp3, o_ij3, o_st3, o_bits, o_owner, o_told, o_tnew, o_wold, s3;
  bool has_wold;  // the leader's copy of w fits (it is left out where it would cost shared-memory mode)
  size_t total;
  __host__ __device__ explicit MergeLayout(int size) {
    tb = total_blocks(size);
    mmax = nb_blocks(2, size);
    // Kept moves of stage 2 are independent sets: at most size/4 + 1 swaps,
    // size/3 + 1 2-opt and size/(k+2) + 1 Or-opt-k moves; each neighbourhood
    // gets a region of the leader's list of at least that capacity.
    m3cap = 0;
    for (int nb = 0; nb < kNumNb; nb++) m3cap += region_cap(nb, size);
    o_ij2 = align_up((size_t)mmax * sizeof(Rec), 16);
    o_tab = o_ij2 + align_up((size_t)mmax * 4, 16);
    s2 = o_tab + align_up((size_t)3 * (size + 4) * 8, 16);
    o_key3 = 0;
    o_shp3 = o_key3 + align_up((size_t)m3cap * 8, 16);
    o_ij3 = o_shp3 + align_up((size_t)m3cap * 8, 16);
    o_st3 = o_ij3 + align_up((size_t)m3cap * 4, 16);
    o_bits = o_st3 + align_up((size_t)m3cap, 16);
    o_owner = o_bits + (size_t)kBitMax * (kBitMax / 32) * 4;
    o_told = o_owner + align_up((size_t)size * 4, 16);
    o_tnew = o_told + align_up((size_t)size * 4, 16);
    o_wold = o_tnew + align_up((size_t)size * 4, 16);
    const size_t with_w = o_wold + align_up((size_t)size * 4, 16);
    has_wold = align_up(s2 > with_w ? s2 : with_w, 128) <= kMergeSmemLimit;
    s3 = has_wold ? with_w : o_wold;
    total = align_up(s2 > s3 ? s2 : s3, 128);
  }
};

// A global merge workspace holds the cluster's (or the one-CTA) layout and,
// when a job's stage-3 list can exceed kBitMax moves, a kBitMaxWs-move
// conflict bit matrix after it.
__host__ __device__ size_t ws_big_bits_offset(int size);
__host__ __device__ __forceinline__ size_t ws_big_bits_bytes() { return (size_t)kBitMaxWs * (kBitMaxWs / 32) * 4; }

__device__ __forceinline__ void amin(uint64_t* p, uint64_t v) {
  atomicMin((unsigned long long*)p, (unsigned long long)v);
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
  const uint32_t hi = __reduce_min_sync(kFull, (uint32_t)(v >> 32));
  const uint32_t lo = __reduce_min_sync(kFull, (uint32_t)(v >> 32) == hi ? (uint32_t)v : 0xffffffffu);
  return ((uint64_t)hi << 32) | lo;
}

// Split cluster barrier.
__device__ __forceinline__ void cluster_arrive_release() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// Named barriers (ids 1..5) synchronise one warp group without the others.
__device__ __forceinline__ void group_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ int group_sync_or(int pred, int id, int nthreads) {
  int r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.s32 p, %1, 0;\n\tbar.red.or.pred q, %2, %3, p;\n\t"
      "selp.s32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"(pred), "r"(id), "r"(nthreads)
      : "memory");
  return r;
}

// Lexicographically-first maximal independent set of c <= 32 * kWarpRoundWords
// moves by one warp (every lane calls it): word w of row x of `bits` (W words
// a row) marks with bit y the earlier moves 32 w + y that conflict with move x.
// Lane l holds moves l, l + 32, ... with their rows in registers; the kept and
// undecided masks are ballots, so a round needs no CTA barrier.  On return
// st_out[x] is kIn or kOut for every x < c.
__device__ __forceinline__ void warp_lfmis(int c, int W, const uint32_t* bits, volatile uint8_t* st_out) {
  const int lane = threadIdx.x & 31;
  uint32_t row[kWarpRoundWords][kWarpRoundWords];
  uint8_t st[kWarpRoundWords];
  uint32_t in[kWarpRoundWords], und[kWarpRoundWords];
#pragma unroll
  for (int q = 0; q < kWarpRoundWords; q++) {
    const int x = 32 * q + lane;
    st[q] = (q < W && x < c) ? kUndec : kNone;
#pragma unroll
    for (int w = 0; w < kWarpRoundWords; w++) row[q][w] = (st[q] == kUndec && w < W) ? bits[x * W + w] : 0u;
    in[q] = 0u;
    und[q] = __ballot_sync(kFull, st[q] == kUndec);
  }
  for (int round = 0; round <= c; round++) {
#pragma unroll
    for (int q = 0; q < kWarpRoundWords; q++) {
      if (st[q] != kUndec) continue;
      uint32_t hin = 0, hund = 0;
#pragma unroll
      for (int w = 0; w < kWarpRoundWords; w++) {
        hin |= row[q][w] & in[w];
        hund |= row[q][w] & und[w];
      }
      if (hin) st[q] = kOut;
      else if (!hund) st[q] = kIn;
    }
    uint32_t left = 0;
#pragma unroll
    for (int q = 0; q < kWarpRoundWords; q++) {
      in[q] = __ballot_sync(kFull, st[q] == kIn);
      und[q] = __ballot_sync(kFull, st[q] == kUndec);
      left |= und[q];
    }
    if (!left) break;
  }
#pragma unroll
  for (int q = 0; q < kWarpRoundWords; q++) {
    const int x = 32 * q + lane;
    if (q < W && x < c) st_out[x] = st[q];
  }
}

// Stage 2 of one neighbourhood, run by one warp group: greedy independent set
// of its negative candidates in (delta, block) order with the same-
// neighbourhood predicate of the reference's GPU merge (mlkernel.cu:51-170
// after the sort at :256), i.e. the lexicographically-first maximal
// independent set of the conflict graph.
//   swap:      rounds of "roots" (no earlier undecided/kept conflicting move)
//              using per-position tables of the smallest undecided key and
//              the smallest kept key with an endpoint there (f_canSwapMerge
//              conflicts are endpoints within 1); a kept key enters its table
//              once, when it is decided.
//   2-opt, Or-opt: conflicts are closed-interval intersections and kept sets
//              are small: the first alive candidate is kept and its conflicts
//              removed, repeatedly.
// On return st[x] == kIn marks the kept candidates.
__device__ __forceinline__ void stage2_group(int nb, int sz, int m, int gtid, int gnt, int bar, Rec* rec, uint64_t* tables,
                             uint64_t* gmin) {
  if (nb == 0) {
    uint64_t* minK = tables;
    uint64_t* minB = tables + (sz + 4);
    uint64_t* minB2 = tables + 2 * (sz + 4);
    for (int q = gtid; q < sz + 4; q += gnt) {
      minK[q] = kKeyNone;
      minB[q] = kKeyNone;
      minB2[q] = kKeyNone;
    }
    group_sync(bar, gnt);
    for (int round = 0; round <= m; round++) {
      uint64_t* cur = (round & 1) ? minB2 : minB;
      uint64_t* nxt = (round & 1) ? minB : minB2;
      for (int x = gtid; x < m; x += gnt) {
        const Rec r = rec[x];
        if (r.st != kUndec) continue;
        const int i = (int)(r.ab & 0xffff), j = (int)(r.ab >> 16);
        amin(&cur[i], r.key);
        amin(&cur[j], r.key);
      }
      group_sync(bar, gnt);
      int any = 0;
      for (int q = gtid; q < sz + 4; q += gnt) nxt[q] = kKeyNone;
      for (int x = gtid; x < m; x += gnt) {
        const Rec r = rec[x];
        if (r.st != kUndec) continue;
        const int i = (int)(r.ab & 0xffff), j = (int)(r.ab >> 16);
        uint64_t qB = kKeyNone, qK = kKeyNone;
#pragma unroll
        for (int e = -1; e <= 1; e++) {
          qB = min(qB, min(cur[i + e], cur[j + e]));
          qK = min(qK, min(minK[i + e], minK[j + e]));
        }
        if (qK < r.key) {
          rec[x].st = kOut;
        } else if (qB >= r.key) {
          // Kept: its key joins the kept table once.  A later candidate that
          // misses it in this pass still saw this one as undecided in cur.
          rec[x].st = kIn;
          amin(&minK[i], r.key);
          amin(&minK[j], r.key);
        } else {
          any = 1;
        }
      }
      if (!group_sync_or(any, bar, gnt)) break;
    }
  } else {
    const int lane = gtid & 31, gw = gtid >> 5, nw = gnt >> 5;
    int xs = -1, as = 0, bs = -1;
    for (int step = 0; step <= m; step++) {
      uint64_t mk = kKeyNone;
      constexpr int U = 4;
      for (int x0 = gtid; x0 < m; x0 += U * gnt) {
        Rec r[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int x = x0 + u * gnt;
          if (x < m) r[u] = rec[x];
          else r[u].st = kNone;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (r[u].st != kUndec) continue;
          const int x = x0 + u * gnt;
          if (xs >= 0) {
            if (x == xs) {
              rec[x].st = kIn;
              continue;
            }
            const int a = (int)(r[u].ab & 0xffff), b = (int)(r[u].ab >> 16);
            if (a <= bs && as <= b) {
              rec[x].st = kOut;
              continue;
            }
          }
          mk = min(mk, r[u].key);
        }
      }
      mk = warp_min_u64(mk);
      uint64_t* buf = gmin + (step & 1) * 32;
      if (lane == 0) buf[gw] = mk;
      group_sync(bar, gnt);
      mk = warp_min_u64(lane < nw ? buf[lane] : kKeyNone);
      if (mk == kKeyNone) break;
      xs = (int)(mk & ((1u << kCtxBits) - 1));
      const uint32_t abs_ = rec[xs].ab;
      as = (int)(abs_ & 0xffff);
      bs = (int)(abs_ >> 16);
    }
  }
}

// Stage-2 records of neighbourhood nb, by the whole CTA: every block's
// candidate with a negative delta becomes a kUndec record keyed
// (delta, block), with its move in ij (i | j << 16) and its conflict interval
// (2-opt, Or-opt) or endpoints (swap) in ab; the other blocks get kNone.
// Every key read is reset to kKeyNone for the next sweep (nothing else reads
// the keys after this point of a merge).
__device__ __forceinline__ void stage2_records(const JobDev* J, int nb, int sz, Rec* rec, uint32_t* ij) {
  const int m = nb_blocks(nb, sz), off = nb_offset(nb, sz);
  const int tid = threadIdx.x, nt = blockDim.x;
  uint64_t* keys = J->keys + off;
  constexpr int U = 4;
  for (int x0 = 0; x0 < m; x0 += U * nt) {
    uint64_t kv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int x = x0 + u * nt + tid;
      kv[u] = x < m ? keys[x] : kKeyNone;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int x = x0 + u * nt + tid;
      if (x < m && kv[u] != kKeyNone) keys[x] = kKeyNone;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int x = x0 + u * nt + tid;
      if (x >= m) continue;
      Rec r;
      r.key = kKeyNone;
      r.ab = 0;
      r.st = kNone;
      if (kv[u] != kKeyNone) {
        const int64_t cost = key_cost(kv[u], kCtxBits);
        if (cost < 0) {
          int i, j;
          map_move(nb, sz, x, (int)(kv[u] & ((1u << kCtxBits) - 1)), i, j);
          r.key = make_key(cost, (uint32_t)x, kCtxBits);
          ij[x] = (uint32_t)i | ((uint32_t)j << 16);
          if (nb == 0) {
            r.ab = (uint32_t)i | ((uint32_t)j << 16);
          } else {
            int a, b;
            conflict_interval(nb, i, j, a, b);
            r.ab = (uint32_t)a | ((uint32_t)b << 16);
          }
          r.st = kUndec;
        }
      }
      rec[x] = r;
    }
  }
}

__device__ __forceinline__ int id_of(uint64_t key3) { return (int)((key3 >> kCtxBits) & 7); }

// Stage 3 (cross-neighbourhood greedy with canMerge, mlkernel.cu:649-864 with
// a stable order), the parallel apply of the selected moves (footprints are
// disjoint for every pair canMerge accepts), statistics, the ADS prefix
// rebuild and the candidate-key reset, by one whole CTA on the list
// key3 / shp3 / ij3 / st3[0, m3) of kept stage-2 moves (any order; every
// st3 entry kUndec).  t_old holds the current tour; bits, owner and t_new are
// workspace (bits: min(m3, kBitMax)^2 bits); bits_big (may be null) holds
// kBitMaxWs^2 bits for lists longer than kBitMax (global merge workspaces);
// w_old (may be null) is a copy of J->w for the prefix rebuild; without
// reset_keys the candidate keys were reset as stage 2 read them.
template <bool WIDE>
__device__ __forceinline__ void merge_finish(const JobDev* J, int sz, int m3, const uint64_t* key3, const uint64_t* shp3,
                             const uint32_t* ij3, volatile uint8_t* st3, uint32_t* bits, int32_t* owner,
                             int32_t* t_old, int32_t* t_new, uint32_t* bits_big = nullptr,
                             const int32_t* w_old = nullptr, bool reset_keys = true, int bits_words = 0) {
  __shared__ uint32_t s_in[kBitMaxWs / 32], s_und[kBitMaxWs / 32];
  __shared__ int s_ns;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  int32_t* tour = J->tour;
  if (tid == 0) s_ns = 0;
  __syncthreads();
  // The conflict-bit area (bits_words words, dead once stage 3 is decided)
  // then holds the applied moves' position map for the ADS rebuild.
  int32_t* const srcmap = bits_words >= sz ? reinterpret_cast<int32_t*>(bits) : nullptr;
  if (m3 > kBitMax) bits = m3 <= kBitMaxWs ? bits_big : nullptr;
  if (bits != nullptr) {
    // conflict rows: bit y of row x <=> y precedes x and !canMerge(y, x)
    const int W3 = (m3 + 31) >> 5;
    for (int x = wid; x < m3; x += nw) {
      const uint64_t kx = key3[x], sx = shp3[x];
#pragma unroll 4
      for (int w = 0; w < W3; w++) {
        const int y = 32 * w + lane;
        bool c = false;
        if (y < m3) c = key3[y] < kx && shapes_conflict(shp3[y], sx);
        const uint32_t word = __ballot_sync(kFull, c);
        if (lane == 0) bits[x * W3 + w] = word;
      }
    }
    if (W3 <= kWarpRoundWords) {
      // Up to 32 * kWarpRoundWords moves: one warp runs the rounds with the
      // rows in registers (lane l holds moves l, l + 32, ...) and the kept /
      // undecided masks as ballots, with no CTA barrier per round.
      __syncthreads();
      if (wid == 0) warp_lfmis(m3, W3, bits, st3);
      __syncthreads();
    } else {
    for (int w = tid; w < W3; w += nt) {
      s_in[w] = 0;
      const int rem = m3 - 32 * w;
      s_und[w] = rem >= 32 ? 0xffffffffu : ((1u << rem) - 1u);
    }
    __syncthreads();
    for (int round = 0; round <= m3; round++) {
      int any = 0;
      for (int x = tid; x < m3; x += nt) {
        if (st3[x] != kUndec) continue;
        uint32_t hin = 0, hund = 0;
        for (int w = 0; w < W3; w++) {
          const uint32_t r = bits[x * W3 + w];
          hin |= r & s_in[w];
          hund |= r & s_und[w];
        }
        if (hin) st3[x] = kOut;
        else if (!hund) st3[x] = kIn;
        else any = 1;
      }
      __syncthreads();
      for (int w = wid; w < W3; w += nw) {
        const int x = 32 * w + lane;
        const uint8_t sx = x < m3 ? st3[x] : kNone;
        const uint32_t bi = __ballot_sync(kFull, sx == kIn), bu = __ballot_sync(kFull, sx == kUndec);
        if (lane == 0) {
          s_in[w] = bi;
          s_und[w] = bu;
        }
      }
      if (!__syncthreads_or(any)) break;
    }
    }
  } else {
    // long lists: one warp per undecided move scans the earlier ones
    for (int round = 0; round <= m3; round++) {
      int any = 0;
      for (int x = wid; x < m3; x += nw) {
        if (st3[x] != kUndec) continue;
        const uint64_t kx = key3[x], sx = shp3[x];
        bool out = false, blocked = false;
        for (int y0 = 0; y0 < m3; y0 += 32) {
          const int y = y0 + lane;
          bool cin = false, cund = false;
          if (y < m3) {
            const uint64_t ky = key3[y];
            const uint8_t sy = st3[y];
            if (ky < kx && (sy == kUndec || sy == kIn) && shapes_conflict(shp3[y], sx)) {
              cin = sy == kIn;
              cund = sy == kUndec;
            }
          }
          out |= __any_sync(kFull, cin);
          blocked |= __any_sync(kFull, cund);
          if (out) break;
        }
        if (lane == 0) {
          if (out) st3[x] = kOut;
          else if (!blocked) st3[x] = kIn;
        }
        if (!out && blocked) any = 1;
      }
      if (!__syncthreads_or(any)) break;
    }
  }
  // ---- apply: every position learns which selected move (if any) owns it ----
  for (int p = tid; p < sz; p += nt) owner[p] = -1;
  __syncthreads();
  for (int x = wid; x < m3; x += nw) {
    if (st3[x] != kIn) continue;
    const int id = id_of(key3[x]);
    const int i = (int)(ij3[x] & 0xffff), j = (int)(ij3[x] >> 16);
    if (id == 0) {
      if (lane == 0) owner[i] = x;
      if (lane == 1) owner[j] = x;
    } else {
      int f0, f1;
      move_footprint(id, i, j, f0, f1);
      for (int p = f0 + lane; p <= f1; p += 32) owner[p] = x;
    }
    if (lane == 0) atomicAdd(&s_ns, 1);
  }
  __syncthreads();
  for (int p = tid; p < sz; p += nt) {
    const int o = owner[p];
    const int q = o >= 0 ? move_source(id_of(key3[o]), (int)(ij3[o] & 0xffff), (int)(ij3[o] >> 16), p) : p;
    const int32_t v = t_old[q];
    t_new[p] = v;
    tour[p] = v;
    if (srcmap != nullptr) srcmap[p] = q;
  }
  const int ns = s_ns;
  // Applied moves in (delta, neighbourhood, block) order, for callers that
  // ask for them (the legacy bestNeighbor move vectors).
  if (J->moves_out != nullptr && (J->flags & kFlagRecordMoves)) {
    for (int x = tid; x < m3; x += nt) {
      if (st3[x] != kIn) continue;
      int rank3 = 0;
      for (int y = 0; y < m3; y++)
        if (st3[y] == kIn && key3[y] < key3[x]) rank3++;
      if (rank3 < J->moves_cap) {
        const uint32_t id = (uint32_t)id_of(key3[x]);
        const uint32_t i = ij3[x] & 0xffff, j = ij3[x] >> 16;
        J->moves_out[rank3] = id | (i << 4) | (j << 18);
        J->moves_cost[rank3] = key_cost(key3[x], kCtxBits + 3);
      }
    }
  }
  if (tid == 0) {
    unsigned long long* stt = (unsigned long long*)J->stats;
    atomicAdd(&stt[kStatSweeps], 1ull);
    atomicExch(&stt[kStatLastMoves], (unsigned long long)ns);
    atomicAdd(&stt[kStatMoves], (unsigned long long)ns);
    if (ns > 0) atomicAdd(&stt[kStatIters], 1ull);
    else atomicExch(&stt[kStatConverged], 1ull);
  }
  __syncthreads();
  cta_prepare<WIDE>(J, t_new, owner, t_old, w_old, srcmap);  // the owner map is dead: w staging
  if (reset_keys) cta_reset_keys(J);
  else if (J->tcount != nullptr && tid < kNumNb) J->tcount[tid] = 0;
}

// One cluster of six CTAs per job.  CTAs 0..4 run stage 2 of neighbourhood
// 0..4 with the whole CTA and hand their kept moves straight to CTA 5 (the
// leader) through distributed shared memory.  Two phases of the hardware
// cluster barrier order the hand-off: every CTA arrives at phase 1 when it
// starts (a stage-2 CTA waits for it before its first remote write, so the
// leader is running); a stage-2 CTA arrives at phase 2 with release semantics
// once its moves and count are written, and the leader's acquire wait of
// phase 2 sees all five lists.  Every CTA arrives and waits at both phases.
// The leader, which has fetched the current tour meanwhile, runs stage 3 (cross-neighbourhood greedy with
// canMerge, mlkernel.cu:649-864 with a stable order), the parallel apply of
// the selected moves (footprints are disjoint for every pair canMerge
// accepts), the ADS prefix rebuild and the candidate-key reset.
template <bool WIDE, bool SMEM>
__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kMergeThreads)
    k_merge(const JobDev* __restrict__ jobs) {
  constexpr bool use_smem = SMEM;
  extern __shared__ __align__(16) uint8_t dsm[];
  __shared__ uint64_t s_gmin[64];  // two step buffers of one entry per warp
  __shared__ int s_m3, s_cnt;
  __shared__ int s_kept[kNumNb];  // leader: the kept-move count of each stage-2 CTA
  __shared__ JobDev s_job;        // leader: its copy of the job descriptor
  // The next sweep may be launched now: it waits for this merge to end
  // before it reads anything.  Before pdl_wait this kernel reads only what
  // the sweep it follows does not write (statistics, tour, w).
  pdl_launch_dependents();
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const JobDev* J = jobs + blockIdx.x / kClusterCtas;
  {
    const int64_t* stt = J->stats;
    if (stt[kStatConverged] || stt[kStatSweeps] >= stt[kStatLimit]) return;  // the whole cluster
  }
  const int sz = J->size, mask = J->nb_mask, tid = threadIdx.x, nt = blockDim.x;
  const MergeLayout lay(sz);
  // Workspace of this CTA, and the leader's stage-3 lists as seen from here.
  uint8_t* ws = use_smem ? dsm : (J->ws + (size_t)rank * lay.total);
  uint8_t* lead = use_smem ? cluster.map_shared_rank(dsm, kClusterCtas - 1)
                           : (J->ws + (size_t)(kClusterCtas - 1) * lay.total);
  uint64_t* key3 = (uint64_t*)(lead + lay.o_key3);
  uint64_t* shp3 = (uint64_t*)(lead + lay.o_shp3);
  uint32_t* ij3 = (uint32_t*)(lead + lay.o_ij3);
  volatile uint8_t* st3 = (volatile uint8_t*)(lead + lay.o_st3);
  int* lead_kept = cluster.map_shared_rank(s_kept, kClusterCtas - 1);
  int32_t* tour = J->tour;
  const bool leader = rank == kClusterCtas - 1;
  int32_t* t_old = (int32_t*)(ws + lay.o_told);
  int32_t* t_new = (int32_t*)(ws + lay.o_tnew);
  // In shared memory the leader keeps a copy of w (a global workspace gains
  // nothing from one: the prefix rebuild reads J->w).
  int32_t* w_old = (use_smem && lay.has_wold) ? (int32_t*)(ws + lay.o_wold) : nullptr;
  if (leader) {
    cluster_arrive_relaxed();  // phase 1: this CTA runs
    // Copies that complete while stage 2 runs: the tour and, in shared memory,
    // the job descriptor (its later field reads stay on chip) and w.
    static_assert(sizeof(JobDev) % 8 == 0, "JobDev copy in 8-byte words");
    if (use_smem && tid < (int)(sizeof(JobDev) / 8)) ((uint64_t*)&s_job)[tid] = ((const uint64_t*)J)[tid];
    const int32_t* w_cur = J->w;
    for (int p = tid; p < sz; p += nt) {
      t_old[p] = tour[p];
      if (w_old != nullptr) w_old[p] = w_cur[p];
    }
    pdl_wait();
    cluster_wait();            // phase 1
    cluster_arrive_relaxed();  // phase 2: the leader has nothing to publish
    cluster_wait();            // phase 2 (acquire): the five kept lists and counts
  } else {
    cluster_arrive_relaxed();  // phase 1: this CTA runs
    const int nb = rank;
    int count = 0;
    pdl_wait();  // the sweep's keys
    if ((mask >> nb) & 1) {
      const int m = nb_blocks(nb, sz);
      Rec* rec = (Rec*)ws;
      uint32_t* ij = (uint32_t*)(ws + lay.o_ij2);
      stage2_records(J, nb, sz, rec, ij);
      if (tid == 0) s_cnt = 0;
      __syncthreads();
      stage2_group(nb, sz, m, tid, nt, 1, rec, (uint64_t*)(ws + lay.o_tab), s_gmin);
      __syncthreads();
      // Write the kept moves into this neighbourhood's region of the leader.
      int nmine = 0;
      for (int x = tid; x < m; x += nt) nmine += rec[x].st == kIn;
      int slot = nmine ? atomicAdd(&s_cnt, nmine) : 0;
      cluster_wait();  // phase 1: the leader runs (the arrivals overlapped stage 2)
      const int base = region_off(nb, sz), cap = region_cap(nb, sz);
      for (int x = tid; x < m; x += nt) {
        if (rec[x].st != kIn) continue;
        if (slot < cap) {
          const uint32_t ijx = ij[x];
          key3[base + slot] = make_key(key_cost(rec[x].key, kCtxBits), ((uint32_t)nb << kCtxBits) | (uint32_t)x,
                                       kCtxBits + 3);
          shp3[base + slot] = move_shape(nb, (int)(ijx & 0xffff), (int)(ijx >> 16));
          ij3[base + slot] = ijx;
        }
        slot++;
      }
      __syncthreads();
      count = min(s_cnt, cap);
      if (tid == 0 && s_cnt > cap) J->stats[kStatError] = 3;
    } else {
      cluster_wait();  // phase 1
    }
    if (tid == 0) lead_kept[nb] = count;
    __syncwarp();
    cluster_arrive_release();  // phase 2: publishes this thread's remote writes
    cluster_wait();            // phase 2
    return;
  }
  // ---- leader: its own list through its own workspace pointer (the same
  // bytes as through the cluster window; in shared memory the compiler then
  // addresses them as shared memory) ----
  key3 = (uint64_t*)(ws + lay.o_key3);
  shp3 = (uint64_t*)(ws + lay.o_shp3);
  ij3 = (uint32_t*)(ws + lay.o_ij3);
  st3 = (volatile uint8_t*)(ws + lay.o_st3);
  // ---- leader: compact the five regions ----
  {
    int cbase[kNumNb + 1];
    cbase[0] = 0;
#pragma unroll
    for (int nb = 0; nb < kNumNb; nb++) cbase[nb + 1] = cbase[nb] + s_kept[nb];
    // Region offsets (constant divisors once the loop is unrolled).
    int roff[kNumNb];
    roff[0] = 0;
#pragma unroll
    for (int nb = 1; nb < kNumNb; nb++) roff[nb] = roff[nb - 1] + region_cap(nb - 1, sz);
    // Move every region's entries to the front: all loads of a chunk, a
    // barrier, then all stores (a destination may be another region's
    // unread source).
    const int total = cbase[kNumNb];
    constexpr int V = 4;
    for (int g0 = 0; g0 < total; g0 += V * nt) {
      uint64_t kk[V], ss[V];
      uint32_t jj[V];
      int dst[V];
#pragma unroll
      for (int v = 0; v < V; v++) {
        const int g = g0 + tid + v * nt;
        dst[v] = -1;
        if (g >= total) continue;
        // The region holding compact index g: the last one starting at or
        // before g (empty regions share their start with the next one).
        int src = g;
#pragma unroll
        for (int q = 0; q < kNumNb; q++)
          if (g >= cbase[q]) src = roff[q] + (g - cbase[q]);
        dst[v] = g;
        kk[v] = key3[src];
        ss[v] = shp3[src];
        jj[v] = ij3[src];
      }
      __syncthreads();
#pragma unroll
      for (int v = 0; v < V; v++) {
        if (dst[v] < 0) continue;
        key3[dst[v]] = kk[v];
        shp3[dst[v]] = ss[v];
        ij3[dst[v]] = jj[v];
        st3[dst[v]] = kUndec;
      }
      __syncthreads();
    }
    if (tid == 0) s_m3 = cbase[kNumNb];
    __syncthreads();
  }
  uint32_t* big = (!use_smem && lay.m3cap > kBitMax) ? (uint32_t*)(J->ws + ws_big_bits_offset(sz)) : nullptr;
  merge_finish<WIDE>(use_smem ? &s_job : J, sz, s_m3, key3, shp3, ij3, st3, (uint32_t*)(ws + lay.o_bits),
                     (int32_t*)(ws + lay.o_owner), t_old, t_new, big, w_old, false,
                     (int)((lay.o_owner - lay.o_bits) / 4));
}

// --------------------------------------------------------------------------
// Throughput merge: one CTA per job.  The five stage-2 passes run one after
// the other on the whole CTA and append their kept moves to the stage-3 list;
// merge_finish then does the rest.  A job uses one CTA of one SM (several jobs
// share an SM) instead of a six-SM cluster: for sets of many jobs the merge
// throughput matters, not one job's latency.  Same moves, same order of
// application, same results as k_merge.
// --------------------------------------------------------------------------
constexpr int kSoloThreads = 512;

struct SoloLayout {
  int m3cap, mmax;
  size_t o_key3, o_shp3, o_ij3, o_st3, o_rec, o_ij2, o_tab, o_bits, o_owner, o_told, o_tnew, total;
  __host__ __device__ explicit SoloLayout(int size) {
    const MergeLayout ml(size);
    m3cap = ml.m3cap;
    mmax = ml.mmax;
    o_key3 = 0;
    o_shp3 = o_key3 + align_up((size_t)m3cap * 8, 16);
    o_ij3 = o_shp3 + align_up((size_t)m3cap * 8, 16);
    o_st3 = o_ij3 + align_up((size_t)m3cap * 4, 16);
    const size_t u = o_st3 + align_up((size_t)m3cap, 16);
    // stage 2 (dead once the list is complete)
    o_rec = u;
    o_ij2 = o_rec + align_up((size_t)mmax * sizeof(Rec), 16);
    o_tab = o_ij2 + align_up((size_t)mmax * 4, 16);
    const size_t e2 = o_tab + align_up((size_t)3 * (size + 4) * 8, 16);
    // stage 3 and apply, over the same bytes
    const size_t b = m3cap < kBitMax ? (size_t)m3cap : (size_t)kBitMax;
    o_bits = u;
    o_owner = o_bits + align_up(b * ((b + 31) / 32) * 4, 16);
    o_told = o_owner + align_up((size_t)size * 4, 16);
    o_tnew = o_told + align_up((size_t)size * 4, 16);
    const size_t e3 = o_tnew + align_up((size_t)size * 4, 16);
    total = align_up(e2 > e3 ? e2 : e3, 128);
  }
};

__host__ __device__ size_t ws_big_bits_offset(int size) {
  const size_t c = MergeLayout(size).total * kClusterCtas, o = SoloLayout(size).total;
  return align_up(c > o ? c : o, 256);
}

template <bool WIDE, bool SMEM>
__global__ void __launch_bounds__(kSoloThreads) k_merge_solo(const JobDev* __restrict__ jobs) {
  constexpr bool use_smem = SMEM;
  extern __shared__ __align__(16) uint8_t dsm[];
  __shared__ uint64_t s_gmin[64];
  __shared__ int s_m3;
  pdl_launch_dependents();  // as in k_merge
  const JobDev* J = jobs + blockIdx.x;
  {
    const int64_t* stt = J->stats;
    if (stt[kStatConverged] || stt[kStatSweeps] >= stt[kStatLimit]) return;
  }
  pdl_wait();  // the sweep's keys
  const int sz = J->size, mask = J->nb_mask, tid = threadIdx.x, nt = blockDim.x;
  const SoloLayout lay(sz);
  uint8_t* ws = use_smem ? dsm : J->ws;
  uint64_t* key3 = (uint64_t*)(ws + lay.o_key3);
  uint64_t* shp3 = (uint64_t*)(ws + lay.o_shp3);
  uint32_t* ij3 = (uint32_t*)(ws + lay.o_ij3);
  volatile uint8_t* st3 = (volatile uint8_t*)(ws + lay.o_st3);
  Rec* rec = (Rec*)(ws + lay.o_rec);
  uint32_t* ij = (uint32_t*)(ws + lay.o_ij2);
  if (tid == 0) s_m3 = 0;
  __syncthreads();
  for (int nb = 0; nb < kNumNb; nb++) {
    if (!((mask >> nb) & 1)) continue;
    const int m = nb_blocks(nb, sz);
    stage2_records(J, nb, sz, rec, ij);
    __syncthreads();
    stage2_group(nb, sz, m, tid, nt, 1, rec, (uint64_t*)(ws + lay.o_tab), s_gmin);
    __syncthreads();
    int nmine = 0;
    for (int x = tid; x < m; x += nt) nmine += rec[x].st == kIn;
    int slot = nmine ? atomicAdd(&s_m3, nmine) : 0;
    for (int x = tid; x < m; x += nt) {
      if (rec[x].st != kIn) continue;
      if (slot < lay.m3cap) {
        const uint32_t ijx = ij[x];
        key3[slot] = make_key(key_cost(rec[x].key, kCtxBits), ((uint32_t)nb << kCtxBits) | (uint32_t)x,
                              kCtxBits + 3);
        shp3[slot] = move_shape(nb, (int)(ijx & 0xffff), (int)(ijx >> 16));
        ij3[slot] = ijx;
        st3[slot] = kUndec;
      }
      slot++;
    }
    __syncthreads();  // rec and ij are rebuilt for the next neighbourhood
  }
  int m3 = s_m3;
  if (m3 > lay.m3cap) {
    if (tid == 0) J->stats[kStatError] = 3;
    m3 = lay.m3cap;
  }
  int32_t* t_old = (int32_t*)(ws + lay.o_told);
  for (int p = tid; p < sz; p += nt) t_old[p] = J->tour[p];
  __syncthreads();
  uint32_t* big = (!use_smem && lay.m3cap > kBitMax) ? (uint32_t*)(J->ws + ws_big_bits_offset(sz)) : nullptr;
  merge_finish<WIDE>(J, sz, m3, key3, shp3, ij3, st3, (uint32_t*)(ws + lay.o_bits), (int32_t*)(ws + lay.o_owner),
                     t_old, (int32_t*)(ws + lay.o_tnew), big, nullptr, false, (int)((lay.o_owner - lay.o_bits) / 4));
}

// --------------------------------------------------------------------------
// Or-opt-k for any k in [1, 28] (MLKernelOrOpt(problem, k)): the reference's
// ODC kernelOrOpt with tag = k (source/mlkoropt.cu:620-794) and its runKernel
// pass (GPU merge with f_canOrOptMerge, mlkernel.cu:61-71, 73-170; applyMove,
// mlkoropt.cu:896-925).  The five-slot DVND keeps k = 1, 2, 3 in its fused
// sweep; these kernels serve any single Or-opt-k neighbourhood.
// --------------------------------------------------------------------------
// Delta of Or-opt-k move (i, j) from the prefix sums (same formulas as the
// sweep's, with the distances gathered from D; mlkoropt.cu:704-716, :724-736).
template <bool WIDE>
__device__ typename Arith<WIDE>::V oropt_delta(const JobDev* J, int k, int i, int j) {
  using C = typename Arith<WIDE>::C;
  const int32_t* __restrict__ t = J->tour;
  const int32_t* __restrict__ D = J->D;
  const int32_t* __restrict__ w = J->w;
  const C* __restrict__ W = (const C*)J->W;
  const int n = J->n;
  auto d = [&](int a, int b) -> C { return (C)D[(size_t)t[a] * n + t[b]]; };
  auto R = [&](int a, int b) -> C { return a > b ? C(0) : C(W[b] - W[a - 1]); };
  const C sz = (C)J->size, kc = (C)k, ic = (C)i, jc = (C)j;
  C c;
  if (i < j)
    c = (sz - ic) * (d(i - 1, i + k) - (C)w[i]) + (sz - jc - kc) * (d(i + k - 1, j + k) - (C)w[j + k]) +
        (sz - jc) * d(j + k - 1, i) - (sz - ic - kc) * (C)w[i + k] + (ic - jc) * R(i + 1, i + k - 1) +
        kc * R(i + k + 1, j + k - 1);
  else
    c = (sz - jc) * (d(j - 1, i) - (C)w[j]) + (sz - ic - kc) * (d(i - 1, i + k) - (C)w[i + k]) +
        (sz - jc - kc) * d(i + k - 1, j) - (sz - ic) * (C)w[i] + (ic - jc) * R(i + 1, i + k - 1) -
        kc * R(j + 1, i - 1);
  return (typename Arith<WIDE>::V)c;
}

// One CTA per reference block: the block's best move as a (delta, ctx) key
// (strict minimum, first ctx on ties; a delta equal to COST_INFTY never
// wins, as in the reference's chunk loop).
template <bool WIDE>
__global__ void __launch_bounds__(256) k_oropt_eval(const JobDev* __restrict__ J, int k, uint64_t* __restrict__ keys) {
  __shared__ uint64_t s_min[8];
  const int by = blockIdx.x, sz = J->size, nthr = oropt_blocks(k, sz);
  uint64_t best = kKeyNone;
  for (int ctx = threadIdx.x; ctx < nthr; ctx += blockDim.x) {
    int i, j;
    map_oropt(k, sz, by, ctx, i, j);
    const typename Arith<WIDE>::V d = oropt_delta<WIDE>(J, k, i, j);
    if (d == Arith<WIDE>::kInf) continue;
    const uint64_t key = make_key((int64_t)d, (uint32_t)ctx, kCtxBits);
    best = key < best ? key : best;
  }
  best = warp_min_u64(best);
  if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) best = s_min[w] < best ? s_min[w] : best;
    best = s_min[0] < best ? s_min[0] : best;
    keys[by] = best;
  }
}

// The pass: improving block candidates in (delta, block) order, greedily
// independent under f_canOrOptMerge (closed intervals [min, max + k] must not
// meet), applied together (disjoint footprints).  Writes the new tour and the
// kept moves in order (ij: i | j << 14, cost) with their count; the caller
// rebuilds the ADS arrays afterwards.  One CTA; scratch: m records, m ij
// words, and size words each for the owner map and the old tour.
template <bool WIDE>
__global__ void __launch_bounds__(1024) k_oropt_pass(const JobDev* __restrict__ J, int k, const uint64_t* keys,
                                                     uint8_t* scratch, uint32_t* out_ij, int64_t* out_cost,
                                                     int* out_count) {
  __shared__ uint64_t s_gmin[64];
  __shared__ int s_cnt;
  const int sz = J->size, m = oropt_blocks(k, sz), tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  const int id = k + 1;
  Rec* rec = (Rec*)scratch;
  uint32_t* ij = (uint32_t*)(scratch + align_up((size_t)m * sizeof(Rec), 16));
  int32_t* owner = (int32_t*)((uint8_t*)ij + align_up((size_t)m * 4, 16));
  int32_t* t_old = (int32_t*)((uint8_t*)owner + align_up((size_t)sz * 4, 16));
  int32_t* tour = J->tour;
  for (int b = tid; b < m; b += nt) {
    Rec r;
    r.key = kKeyNone;
    r.ab = 0;
    r.st = kNone;
    const uint64_t key = keys[b];
    if (key != kKeyNone) {
      const int64_t cost = key_cost(key, kCtxBits);
      if (cost < 0) {
        int i, j;
        map_oropt(k, sz, b, (int)(key & ((1u << kCtxBits) - 1)), i, j);
        r.key = make_key(cost, (uint32_t)b, kCtxBits);
        r.ab = (uint32_t)imin_(i, j) | ((uint32_t)(imax_(i, j) + k) << 16);
        r.st = kUndec;
        ij[b] = (uint32_t)i | ((uint32_t)j << 16);
      }
    }
    rec[b] = r;
  }
  for (int p = tid; p < sz; p += nt) {
    t_old[p] = tour[p];
    owner[p] = -1;
  }
  if (tid == 0) s_cnt = 0;
  __syncthreads();
  stage2_group(2, sz, m, tid, nt, 1, rec, nullptr, s_gmin);  // the interval branch
  __syncthreads();
  for (int x = wid; x < m; x += nw) {
    if (rec[x].st != kIn) continue;
    const int i = (int)(ij[x] & 0xffff), j = (int)(ij[x] >> 16);
    int f0, f1;
    move_footprint(id, i, j, f0, f1);
    for (int p = f0 + lane; p <= f1; p += 32) owner[p] = x;
    if (lane == 0) atomicAdd(&s_cnt, 1);
  }
  __syncthreads();
  for (int p = tid; p < sz; p += nt) {
    const int o = owner[p];
    if (o >= 0) tour[p] = t_old[move_source(id, (int)(ij[o] & 0xffff), (int)(ij[o] >> 16), p)];
  }
  for (int x = tid; x < m; x += nt) {
    if (rec[x].st != kIn) continue;
    int rank = 0;
    for (int y = 0; y < m; y++)
      if (rec[y].st == kIn && rec[y].key < rec[x].key) rank++;
    out_ij[rank] = (ij[x] & 0xffff) | ((ij[x] >> 16) << 14);
    out_cost[rank] = key_cost(rec[x].key, kCtxBits);
  }
  if (tid == 0) *out_count = s_cnt;
}

// --------------------------------------------------------------------------
// End of a TOTAL iteration: the moves kept by the TOTAL greedy of every
// neighbourhood (k_total_select, mlp_total.cu) form the stage-3 list, keyed
// (delta, neighbourhood, rank in that greedy's order); merge_finish then runs
// the cross-neighbourhood greedy, the apply and the ADS rebuild as after
// k_merge_solo.  One 1024-thread CTA per job (the k_merge_solo workspace).
// --------------------------------------------------------------------------
template <bool WIDE, bool SMEM>
__global__ void __launch_bounds__(kMergeThreads) k_total_finish(const JobDev* __restrict__ jobs) {
  constexpr bool use_smem = SMEM;
  extern __shared__ __align__(16) uint8_t dsm[];
  pdl_launch_dependents();  // the next collecting sweep waits for this kernel's end
  const JobDev* J = jobs + blockIdx.x;
  {
    const int64_t* stt = J->stats;
    if (stt[kStatConverged] || stt[kStatSweeps] >= stt[kStatLimit]) return;
  }
  pdl_wait();  // the greedy's kept moves
  const int sz = J->size, mask = J->nb_mask, tid = threadIdx.x, nt = blockDim.x;
  const SoloLayout lay(sz);
  uint8_t* ws = use_smem ? dsm : J->ws;
  uint64_t* key3 = (uint64_t*)(ws + lay.o_key3);
  uint64_t* shp3 = (uint64_t*)(ws + lay.o_shp3);
  uint32_t* ij3 = (uint32_t*)(ws + lay.o_ij3);
  volatile uint8_t* st3 = (volatile uint8_t*)(ws + lay.o_st3);
  int m3 = 0;
  for (int nb = 0; nb < kNumNb; nb++) {
    if (!((mask >> nb) & 1)) continue;
    const int cnt = J->tkcount[nb], base = region_off(nb, sz);
    for (int r = tid; r < cnt; r += nt) {
      const int slot = m3 + r;
      if (slot >= lay.m3cap) break;
      const uint32_t ijx = J->tkij[base + r];
      key3[slot] = make_key(J->tkcost[base + r], ((uint32_t)nb << kCtxBits) | (uint32_t)r, kCtxBits + 3);
      shp3[slot] = move_shape(nb, (int)(ijx & 0xffff), (int)(ijx >> 16));
      ij3[slot] = ijx;
      st3[slot] = kUndec;
    }
    m3 += cnt;
  }
  if (m3 > lay.m3cap) {
    if (tid == 0) J->stats[kStatError] = 3;
    m3 = lay.m3cap;
  }
  int32_t* t_old = (int32_t*)(ws + lay.o_told);
  for (int p = tid; p < sz; p += nt) t_old[p] = J->tour[p];
  __syncthreads();
  uint32_t* big = (!use_smem && lay.m3cap > kBitMax) ? (uint32_t*)(J->ws + ws_big_bits_offset(sz)) : nullptr;
  merge_finish<WIDE>(J, sz, m3, key3, shp3, ij3, st3, (uint32_t*)(ws + lay.o_bits), (int32_t*)(ws + lay.o_owner),
                     t_old, (int32_t*)(ws + lay.o_tnew), big, nullptr, true, (int)((lay.o_owner - lay.o_bits) / 4));
}

// --------------------------------------------------------------------------
// Reference ADS buffer (mlads.h:38-74, filled like MLSolution::ldsUpdate,
// mlsolution.cpp:420-486).  C is written from the closed form
//   C[i][j] = (P[j] - P[i]) - (j - i) T[i]          (i < j)
//   C[i][j] = (i - j) T[i] - (P[i-1] - P[j-1])       (i > j)
// with P the prefix sum of T (uint32 wrap, like the reference's recurrences).
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_ads_head(const JobDev* __restrict__ J, const int32_t* cx,
                                                   const int32_t* cy, uint32_t* ads, uint32_t* Pbuf,
                                                   int cost_tour, int dist_round) {
  __shared__ uint32_t sm[32];
  const int sz = J->size;
  const uint32_t rowE = (uint32_t)sz;
  uint32_t* coords = ads + 32;
  uint32_t* sol = coords + rowE;
  uint32_t* T = coords + 2 * rowE;
  const int32_t* t = J->tour;
  const int32_t* w = J->w;
  const int nt = blockDim.x, chunk = (sz + nt - 1) / nt;
  const int p0 = threadIdx.x * chunk, p1 = min(sz, p0 + chunk);
  if (threadIdx.x < 32) {
    uint32_t v = 0;
    if (threadIdx.x == 0) v = 128u + rowE * (uint32_t)(sz + 3) * 4u;
    if (threadIdx.x == 1) v = rowE;
    if (threadIdx.x == 2) v = (uint32_t)sz;
    if (threadIdx.x == 3) v = (uint32_t)J->stats[kStatCost];
    if (threadIdx.x == 4) v = (uint32_t)(cost_tour != 0);
    if (threadIdx.x == 5) v = (uint32_t)(dist_round != 0);
    ads[threadIdx.x] = v;
  }
  uint32_t s = 0;
  for (int p = p0; p < p1; p++) s += (uint32_t)(uint16_t)w[p];
  uint32_t tot;
  uint32_t e = block_exclusive_scan<uint32_t>(s, sm, tot);
  uint32_t sP = 0;
  for (int p = p0; p < p1; p++) {
    const int node = t[p];
    coords[p] = ((uint32_t)(uint16_t)cx[node] << 16) | (uint32_t)(uint16_t)cy[node];
    sol[p] = p == 0 ? (uint32_t)(uint16_t)node : (((uint32_t)(uint16_t)node << 16) | (uint32_t)(uint16_t)w[p]);
    e += (uint32_t)(uint16_t)w[p];
    T[p] = e;
    sP += e;
  }
  uint32_t totP;
  uint32_t eP = block_exclusive_scan<uint32_t>(sP, sm, totP);
  for (int p = p0; p < p1; p++) {
    eP += T[p];
    Pbuf[p] = eP;
  }
}

__global__ void k_ads_cost(const int sz, uint32_t* __restrict__ ads, const uint32_t* __restrict__ Pbuf) {
  const uint32_t rowE = (uint32_t)sz;
  const uint32_t* T = ads + 32 + 2 * rowE;
  uint32_t* Cm = ads + 32 + 3 * rowE;
  const int i = blockIdx.y;
  const uint32_t Ti = T[i];
  const uint32_t Pi = Pbuf[i];
  const uint32_t Pim1 = i > 0 ? Pbuf[i - 1] : 0u;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < sz; j += gridDim.x * blockDim.x) {
    uint32_t v;
    if (j > i) v = (Pbuf[j] - Pi) - (uint32_t)(j - i) * Ti;
    else if (j < i) v = (uint32_t)(i - j) * Ti - (Pim1 - (j > 0 ? Pbuf[j - 1] : 0u));
    else v = 0u;
    Cm[(size_t)i * rowE + j] = v;
  }
}

// D from coordinates, exactly like MLProblem::load (float sqrt, +dr, truncate).
__global__ void k_dist(const int32_t* __restrict__ x, const int32_t* __restrict__ y, int n,
                       float dr, int32_t* __restrict__ D, int32_t* dmax) {
  const int i = blockIdx.y;
  const int xi = x[i], yi = y[i];
  int32_t mx = 0;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int dx = xi - x[j], dy = yi - y[j];
    const float s = (float)(dx * dx + dy * dy);
    const int32_t v = (int32_t)(__fsqrt_rn(s) + dr);
    D[(size_t)i * n + j] = v;
    mx = max(mx, v);
  }
  mx = __reduce_max_sync(kFull, (unsigned)mx);
  if ((threadIdx.x & 31) == 0) atomicMax(dmax, mx);
}

// Legacy applyMoves (dvnd.cpp:16-145): moves applied one after the other in
// the given order; move id 1 is applied as a swap (the reference's quirk).
__global__ void __launch_bounds__(1024) k_legacy_apply(const JobDev* __restrict__ J,
                                                       const int32_t* __restrict__ moves, int m) {
  const int sz = J->size;
  int32_t* tour = J->tour;
  int32_t* alt = J->tour_alt;
  for (int q = 0; q < m; q++) {
    int id = moves[3 * q];
    const int i = moves[3 * q + 1], j = moves[3 * q + 2];
    if (id == 1) id = 0;
    int f0, f1;
    move_footprint(id, i, j, f0, f1);
    if (id == 0) {
      f0 = min(i, j);
      f1 = max(i, j);
    }
    for (int p = f0 + (int)threadIdx.x; p <= f1 && p < sz; p += blockDim.x) {
      int src = p;
      if (id == 0) src = p == i ? j : (p == j ? i : p);
      else if (i != j) src = move_source(id, i, j, p);
      alt[p] = tour[src];
    }
    __syncthreads();
    for (int p = f0 + (int)threadIdx.x; p <= f1 && p < sz; p += blockDim.x) tour[p] = alt[p];
    __syncthreads();
  }
}

__global__ void k_stats_begin(const JobDev* __restrict__ jobs, int njobs, int64_t limit) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= njobs) return;
  int64_t* st = jobs[q].stats;
  st[kStatIters] = 0;
  st[kStatMoves] = 0;
  st[kStatConverged] = 0;
  st[kStatLastMoves] = 0;
  st[kStatDone] = 0;
  st[kStatSweeps] = 0;
  st[kStatLimit] = limit;
}

__global__ void k_loop_condition(const JobDev* __restrict__ jobs, int njobs, cudaGraphConditionalHandle h) {
  __shared__ int s_any;
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  int any = 0;
  for (int q = threadIdx.x; q < njobs; q += blockDim.x) {
    const int64_t* st = jobs[q].stats;
    if (!st[kStatConverged] && st[kStatSweeps] < st[kStatLimit]) any = 1;
  }
  if (any) s_any = 1;
  __syncthreads();
  if (threadIdx.x == 0) cudaGraphSetConditional(h, s_any ? 1u : 0u);
}

template <bool WIDE, int TL, int TR>
cudaError_t sweep_collect_launch(const SweepTile* tiles, int ntiles, const JobDev* jobs, cudaStream_t s) {
  return launch_pdl(k_sweep<WIDE, TL, TR, true>, dim3(ntiles), dim3(TL), 0, s, tiles, jobs, 1);
}

template <bool WIDE, int TL, int TR>
cudaError_t sweep_launch(const SweepTile* tiles, int ntiles, const JobDev* jobs, int improve_only,
                         cudaStream_t s) {
  k_sweep<WIDE, TL, TR><<<ntiles, TL, 0, s>>>(tiles, jobs, improve_only);
  return cudaGetLastError();
}

template <bool WIDE>
cudaError_t sweep_dispatch(const SweepTile* tiles, int ntiles, const JobDev* jobs, int shape, int improve_only,
                           cudaStream_t s) {
  switch (shape) {
    case 0: return sweep_launch<WIDE, 32, 4>(tiles, ntiles, jobs, improve_only, s);
    case 1: return sweep_launch<WIDE, 32, 8>(tiles, ntiles, jobs, improve_only, s);
    case 2: return sweep_launch<WIDE, 32, 16>(tiles, ntiles, jobs, improve_only, s);
    case 3: return sweep_launch<WIDE, 64, 4>(tiles, ntiles, jobs, improve_only, s);
    case 4: return sweep_launch<WIDE, 64, 8>(tiles, ntiles, jobs, improve_only, s);
    case 5: return sweep_launch<WIDE, 64, 16>(tiles, ntiles, jobs, improve_only, s);
    case 6: return sweep_launch<WIDE, 128, 8>(tiles, ntiles, jobs, improve_only, s);
    case 7: return sweep_launch<WIDE, 128, 16>(tiles, ntiles, jobs, improve_only, s);
    case 8: return sweep_launch<WIDE, 32, 32>(tiles, ntiles, jobs, improve_only, s);
    case 9: return sweep_launch<WIDE, 64, 32>(tiles, ntiles, jobs, improve_only, s);
    // Two-diagonals-per-thread shapes of the DVND sweep: here one per thread.
    case 10: return sweep_launch<WIDE, 64, 8>(tiles, ntiles, jobs, improve_only, s);
    case 11: return sweep_launch<WIDE, 64, 16>(tiles, ntiles, jobs, improve_only, s);
    case 12: return sweep_launch<WIDE, 64, 32>(tiles, ntiles, jobs, improve_only, s);
    case 13: return sweep_launch<WIDE, 128, 16>(tiles, ntiles, jobs, improve_only, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

size_t merge_smem_bytes(int size) { return MergeLayout(size).total; }
size_t merge_ws_bytes(int size) {
  return ws_big_bits_offset(size) + (MergeLayout(size).m3cap > kBitMax ? ws_big_bits_bytes() : 0);
}
size_t solo_smem_bytes(int size) { return SoloLayout(size).total; }
int solo_smem_max_size() {
  static const int cached = [] {
    int sz = 8;
    while (sz < kMaxSize && SoloLayout(sz + 1).total <= (size_t)(227 * 1024 - 8192)) sz++;
    return sz;
  }();
  return cached;
}
int merge_smem_max_size() {
  // Largest size whose merge workspace fits the 227 KB opt-in shared memory
  // (minus the kernel's static shared memory).
  static const int cached = [] {
    int sz = 8;
    while (sz < kMaxSize && MergeLayout(sz + 1).total <= kMergeSmemLimit) sz++;
    return sz;
  }();
  return cached;
}

cudaError_t launch_prepare(const JobDev* jobs, int njobs, bool wide, bool reset_stats,
                           cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  const size_t smem = sizeof(int32_t) * kMaxSize;
  if (wide) k_prepare<true><<<njobs, 1024, smem, s>>>(jobs, reset_stats ? 1 : 0);
  else k_prepare<false><<<njobs, 1024, smem, s>>>(jobs, reset_stats ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_sweep(const SweepTile* tiles, int ntiles, const JobDev* jobs, bool wide,
                         int shape, bool improve_only, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  const int io = improve_only ? 1 : 0;
  return wide ? sweep_dispatch<true>(tiles, ntiles, jobs, shape, io, s)
              : sweep_dispatch<false>(tiles, ntiles, jobs, shape, io, s);
}

cudaError_t launch_sweep_collect(const SweepTile* tiles, int ntiles, const JobDev* jobs, bool wide, int shape,
                                 cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  static_assert(kTileShapes[kTotalShapeSmall].tl == 64 && kTileShapes[kTotalShapeSmall].tr == 4, "collect shape");
  static_assert(kTileShapes[kTotalShapeLarge].tl == 128 && kTileShapes[kTotalShapeLarge].tr == 16, "collect shape");
  if (shape == kTotalShapeSmall)
    return wide ? sweep_collect_launch<true, 64, 4>(tiles, ntiles, jobs, s)
                : sweep_collect_launch<false, 64, 4>(tiles, ntiles, jobs, s);
  if (shape == kTotalShapeLarge)
    return wide ? sweep_collect_launch<true, 128, 16>(tiles, ntiles, jobs, s)
                : sweep_collect_launch<false, 128, 16>(tiles, ntiles, jobs, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_total_finish(const JobDev* jobs, int njobs, bool wide, bool use_smem, int max_size,
                                cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  const size_t smem = use_smem ? SoloLayout(max_size).total : 0;
  if (wide) {
    if (use_smem) return launch_pdl(k_total_finish<true, true>, dim3(njobs), dim3(kMergeThreads), smem, s, jobs);
    return launch_pdl(k_total_finish<true, false>, dim3(njobs), dim3(kMergeThreads), smem, s, jobs);
  }
  if (use_smem) return launch_pdl(k_total_finish<false, true>, dim3(njobs), dim3(kMergeThreads), smem, s, jobs);
  return launch_pdl(k_total_finish<false, false>, dim3(njobs), dim3(kMergeThreads), smem, s, jobs);
}

size_t oropt_pass_scratch_bytes(int size, int k) {
  const int m = oropt_blocks(k, size);
  return align_up((size_t)m * sizeof(Rec), 16) + align_up((size_t)m * 4, 16) + 2 * align_up((size_t)size * 4, 16);
}

cudaError_t launch_oropt_eval(const JobDev* job, int k, int size, bool wide, uint64_t* keys, cudaStream_t s) {
  const int m = oropt_blocks(k, size);
  if (m <= 0) return cudaErrorInvalidValue;
  if (wide) k_oropt_eval<true><<<m, 256, 0, s>>>(job, k, keys);
  else k_oropt_eval<false><<<m, 256, 0, s>>>(job, k, keys);
  return cudaGetLastError();
}

cudaError_t launch_oropt_pass(const JobDev* job, int k, bool wide, const uint64_t* keys, uint8_t* scratch,
                              uint32_t* out_ij, int64_t* out_cost, int* out_count, cudaStream_t s) {
  if (wide) k_oropt_pass<true><<<1, 1024, 0, s>>>(job, k, keys, scratch, out_ij, out_cost, out_count);
  else k_oropt_pass<false><<<1, 1024, 0, s>>>(job, k, keys, scratch, out_ij, out_cost, out_count);
  return cudaGetLastError();
}

cudaError_t configure_prepare() {
  cudaError_t e = cudaFuncSetAttribute(k_prepare<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(sizeof(int32_t) * kMaxSize));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_prepare<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(sizeof(int32_t) * kMaxSize));
}

cudaError_t configure_merge(size_t bytes) {
  cudaError_t e0 = cudaFuncSetAttribute(k_prepare<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(sizeof(int32_t) * kMaxSize));
  if (e0 != cudaSuccess) return e0;
  e0 = cudaFuncSetAttribute(k_prepare<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)(sizeof(int32_t) * kMaxSize));
  if (e0 != cudaSuccess) return e0;
  // The attribute is a per-device upper bound shared by every job set of the
  // process: never lower it below the largest shared-memory merge layout, or
  // a set configured earlier with larger jobs would fail its next launch.
  bytes = bytes > MergeLayout(merge_smem_max_size()).total ? bytes : MergeLayout(merge_smem_max_size()).total;
  cudaError_t e = cudaFuncSetAttribute(k_merge<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_merge<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  const int solo = (int)SoloLayout(solo_smem_max_size()).total;
  e = cudaFuncSetAttribute(k_merge_solo<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, solo);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_merge_solo<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, solo);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_total_finish<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, solo);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_total_finish<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, solo);
  if (e != cudaSuccess) return e;
  return configure_total();
}

cudaError_t launch_merge(const JobDev* jobs, int njobs, bool wide, bool use_smem, int max_size,
                         cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  const size_t smem = use_smem ? MergeLayout(max_size).total : 0;
  const unsigned g = (unsigned)(njobs * kClusterCtas);
  if (wide) {
    if (use_smem) return launch_pdl(k_merge<true, true>, dim3(g), dim3(kMergeThreads), smem, s, jobs);
    return launch_pdl(k_merge<true, false>, dim3(g), dim3(kMergeThreads), smem, s, jobs);
  }
  if (use_smem) return launch_pdl(k_merge<false, true>, dim3(g), dim3(kMergeThreads), smem, s, jobs);
  return launch_pdl(k_merge<false, false>, dim3(g), dim3(kMergeThreads), smem, s, jobs);
}

cudaError_t launch_merge_solo(const JobDev* jobs, int njobs, bool wide, bool use_smem, int max_size,
                              cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  const size_t smem = use_smem ? SoloLayout(max_size).total : 0;
  if (wide) {
    if (use_smem) return launch_pdl(k_merge_solo<true, true>, dim3(njobs), dim3(kSoloThreads), smem, s, jobs);
    return launch_pdl(k_merge_solo<true, false>, dim3(njobs), dim3(kSoloThreads), smem, s, jobs);
  }
  if (use_smem) return launch_pdl(k_merge_solo<false, true>, dim3(njobs), dim3(kSoloThreads), smem, s, jobs);
  return launch_pdl(k_merge_solo<false, false>, dim3(njobs), dim3(kSoloThreads), smem, s, jobs);
}

cudaError_t launch_loop_condition(const JobDev* jobs, int njobs, cudaGraphConditionalHandle h,
                                  cudaStream_t s) {
  k_loop_condition<<<1, 256, 0, s>>>(jobs, njobs, h);
  return cudaGetLastError();
}

cudaError_t launch_stats_begin(const JobDev* jobs, int njobs, int64_t limit, cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  k_stats_begin<<<(njobs + 127) / 128, 128, 0, s>>>(jobs, njobs, limit);
  return cudaGetLastError();
}

cudaError_t launch_ads(const JobDev* job, const int32_t* cx, const int32_t* cy, uint32_t* ads,
                       int cost_tour, int dist_round, cudaStream_t s, uint32_t* Pbuf, int size) {
  k_ads_head<<<1, 1024, 0, s>>>(job, cx, cy, ads, Pbuf, cost_tour, dist_round);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dim3 grid((size + 255) / 256 < 8 ? (size + 255) / 256 : 8, size);
  k_ads_cost<<<grid, 256, 0, s>>>(size, ads, Pbuf);
  return cudaGetLastError();
}

cudaError_t launch_dist(const int32_t* x, const int32_t* y, int n, int dist_round, int32_t* D,
                        int32_t* dmax, cudaStream_t s) {
  dim3 grid((n + 255) / 256 < 16 ? (n + 255) / 256 : 16, n);
  k_dist<<<grid, 256, 0, s>>>(x, y, n, dist_round ? 0.5f : 0.0f, D, dmax);
  return cudaGetLastError();
}

cudaError_t launch_legacy_apply(const JobDev* job, const int32_t* moves, int m, cudaStream_t s) {
  if (m <= 0) return cudaSuccess;
  k_legacy_apply<<<1, 1024, 0, s>>>(job, moves, m);
  return cudaGetLastError();
}

}  // namespace mlp
