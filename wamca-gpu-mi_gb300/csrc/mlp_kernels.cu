// mlp_kernels.cu -- CUDA kernels of the GB300 MLP local-search engine (sm_103a).
//
// Data path of one DVND iteration (see mlp_engine.cpp for the host side):
//   k_sweep   all five neighbourhoods (swap, 2-opt, Or-opt-1/2/3) over the
//             tour, tiled over (row r, diagonal L = c - r) parallelograms; one
//             64-bit (delta, ctx) key per reference block via atomicMin.
//   k_merge   one CTA per (job, neighbourhood): stage-2 greedy independent set
//             (the reference's per-kernel GPU merge); the last CTA of a job runs
//             the cross-neighbourhood greedy, applies the selected moves,
//             rebuilds w / prefix arrays / cost and resets the candidate keys.
//   k_prepare the ADS prefix rebuild alone (after a new tour is set).
//
// All arithmetic is integer.  In int32 mode every delta and cost is computed in
// uint32 modular arithmetic, which reproduces the reference's 32-bit wrap-around
// results exactly; in wide mode everything is int64.
#include <cstdint>

#include "mlp_common.cuh"
#include "mlp_kernels.cuh"

namespace mlp {

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

// --------------------------------------------------------------------------
// ADS prefix rebuild: w[p] = D[t[p-1]][t[p]], W = prefix(w), Q = prefix(p w),
// A[k-1][p] = D[t[p-1]][t[p+k]], cost = sum (size - p) w[p]
// (source/mlsolution.cpp:216-228 and :454-458 for T = W).
// --------------------------------------------------------------------------
template <bool WIDE>
__device__ void cta_prepare(const JobDev* J) {
  using C = typename Arith<WIDE>::C;
  __shared__ C smW[32], smQ[32], smC[32];
  const int sz = J->size, n = J->n, pad = sz + 8;
  const int32_t* __restrict__ t = J->tour;
  const int32_t* __restrict__ D = J->D;
  int32_t* w = J->w;
  int32_t* A = J->A;
  C* W = (C*)J->W;
  C* Q = (C*)J->Q;
  const int nt = blockDim.x;
  const int chunk = (sz + nt - 1) / nt;
  const int p0 = threadIdx.x * chunk;
  const int p1 = min(sz, p0 + chunk);
  C sW = 0, sQ = 0, sC = 0;
  for (int p = p0; p < p1; p++) {
    const int32_t prev = p > 0 ? t[p - 1] : 0;
    const int32_t wp = p > 0 ? __ldg(D + (size_t)prev * n + t[p]) : 0;
    w[p] = wp;
    sW += (C)wp;
    sQ += (C)p * (C)wp;
    sC += (C)(sz - p) * (C)wp;
#pragma unroll
    for (int k = 1; k <= 3; k++)
      A[(k - 1) * pad + p] = (p >= 1 && p + k <= sz - 1) ? __ldg(D + (size_t)prev * n + t[p + k]) : 0;
  }
  C totW, totQ, totC;
  C eW = block_exclusive_scan<C>(sW, smW, totW);
  C eQ = block_exclusive_scan<C>(sQ, smQ, totQ);
  block_exclusive_scan<C>(sC, smC, totC);
  for (int p = p0; p < p1; p++) {
    const C wp = (C)w[p];
    eW += wp;
    eQ += (C)p * wp;
    W[p] = eW;
    Q[p] = eQ;
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
}

template <bool WIDE>
__global__ void __launch_bounds__(1024) k_prepare(const JobDev* __restrict__ jobs, int reset_stats) {
  const JobDev* J = jobs + blockIdx.x;
  if (reset_stats && threadIdx.x < kStatWords) {
    const int q = threadIdx.x;
    if (q != kStatLimit) J->stats[q] = 0;
  }
  cta_prepare<WIDE>(J);
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
template <bool WIDE, int TL, int TR>
__global__ void __launch_bounds__(TL) k_sweep(const SweepTile* __restrict__ tiles,
                                              const JobDev* __restrict__ jobs) {
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
  if (stats[kStatConverged] || stats[kStatSweeps] >= stats[kStatLimit]) return;
  const int sz = J->size, n = J->n, mask = J->nb_mask;
  const int r0 = tile.r0, L0 = tile.L0, tid = threadIdx.x;
  const int pad = sz + 8;
  const int32_t* __restrict__ t = J->tour;
  const int32_t* __restrict__ D = J->D;
  const int32_t* __restrict__ w = J->w;
  const int32_t* __restrict__ Ag = J->A;
  const C* __restrict__ W = (const C*)J->W;
  const C* __restrict__ Q = (const C*)J->Q;

  for (int q = tid; q < SR; q += TL) {
    const int p = r0 - 1 + q;
    sRowT[q] = p <= sz - 1 ? t[p] : 0;
  }
  for (int q = tid; q < NT; q += TL) {
    const int p = r0 + L0 - 2 + q;
    sColT[q] = p <= sz - 1 ? t[p] : 0;
  }
  for (int q = tid; q < NR; q += TL) {
    const int p = r0 + q;
    const bool ok = p < pad;
    sRw[q] = ok ? w[p] : 0;
    sRW[q] = ok ? W[p] : C(0);
    sRQ[q] = ok ? Q[p] : C(0);
#pragma unroll
    for (int k = 0; k < 3; k++) sRA[k][q] = ok ? Ag[k * pad + p] : 0;
  }
  for (int q = tid; q < NC; q += TL) {
    const int p = r0 + L0 - 1 + q;
    const bool ok = p < pad;
    sCw[q] = ok ? w[p] : 0;
    sCW[q] = ok ? W[p] : C(0);
    sCQ[q] = ok ? Q[p] : C(0);
#pragma unroll
    for (int k = 0; k < 3; k++) sCA[k][q] = ok ? Ag[k * pad + p] : 0;
  }
  __syncthreads();
  for (int idx = tid; idx < SR * SC; idx += TL) {
    const int a = idx / SC, b = idx - a * SC;
    const int rp = r0 - 1 + a, cp = rp + L0 - 1 + b;
    int32_t v = 0;
    if (rp <= sz - 1 && cp <= sz - 1) v = __ldg(D + (size_t)sRowT[a] * n + sColT[a + b]);
    sS[a][b] = v;
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

#pragma unroll 1
  for (int a = 1; a <= TR; a++) {
    const int r = r0 + a - 1;
    if (r > sz - 3) break;  // uniform across the CTA
    const int c = r + L;
    const bool vpair = c <= sz - 2;
    const int qr = a - 1, qc = a + tid;
    const C sM1P1 = (C)sS[a - 1][b + 1];
    const C s0M1 = (C)sS[a][b - 1];
    const C s00 = (C)sS[a][b];
    const C s0P1 = (C)sS[a][b + 1];
    const C s0P2 = (C)sS[a][b + 2];
    const C sP1M1 = (C)sS[a + 1][b - 1];
    const C sP1P1 = (C)sS[a + 1][b + 1];
    const C sP2P1 = (C)sS[a + 2][b + 1];
    const C wr0 = (C)sRw[qr], wr1 = (C)sRw[qr + 1];
    const C wc0 = (C)sCw[qc], wc1 = (C)sCw[qc + 1];
    const C Wr0 = sRW[qr], Wc0 = sCW[qc];
    const C szr = (C)(sz - r), szc = (C)(sz - c);

    // ---- swap (row-owned blocks): warp argmin per row ----
    if (mSw) {
      const bool v = vpair && L >= 2;
      const V d = (V)(szr * (sM1P1 - wr0) + (szr - C(1)) * (sP1M1 - wr1) + szc * (s0M1 - wc0) +
                      (szc - C(1)) * (s0P1 - wc1));
      const int blkA = r - 1, blkB = sz - 3 - r;
      const bool hasA = blkA < nbS, hasB = blkB >= 0 && blkB < nbS;
      unsigned ties;
      bool any;
      if (!WIDE) {
        const uint32_t u = (v && d != kInf) ? ((uint32_t)d ^ 0x80000000u) : 0xffffffffu;
        const uint32_t mn = __reduce_min_sync(kFull, u);
        any = mn != 0xffffffffu;
        ties = __ballot_sync(kFull, u == mn);
      } else {
        const uint64_t u = v ? (uint64_t)((int64_t)d + (int64_t)kCostBias) : ~0ull;
        const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
        const uint32_t mh = __reduce_min_sync(kFull, hi);
        const uint32_t ml = __reduce_min_sync(kFull, hi == mh ? lo : 0xffffffffu);
        any = !(mh == 0xffffffffu && ml == 0xffffffffu);
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

    // ---- 2-opt (diagonal-owned blocks) ----
    if (m2o && vpair) {
      const V d = (V)(szr * (sM1P1 - wr0) + (szc - C(1)) * (s0P1 - wc1) +
                      C(2) * (sCQ[qc] - sRQ[qr]) - (C)(r + c + 1) * (Wc0 - Wr0));
      if (has2A && d < b2A) {
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
      if (!((mask >> (k + 1)) & 1) || c + k > sz - 1) continue;
      const C Sf = k == 1 ? s0P1 : (k == 2 ? sP1P1 : sP2P1);  // E(r+k-1, c+k)
      const C Sg = k == 1 ? s00 : (k == 2 ? s0P1 : s0P2);     // E(r, c+k-1)
      const C wrk = (C)sRw[qr + k], wck = (C)sCw[qc + k];
      const C kk = (C)k;
      {
        const V d = (V)(szr * ((C)sRA[k - 1][qr] - wr0) + (szc - kk) * (Sf - wck) + szc * Sg -
                        (szr - kk) * wrk + ((C)r - (C)c) * (sRW[qr + k - 1] - Wr0) +
                        kk * (sCW[qc + k - 1] - sRW[qr + k]));
        if (d < bF[k - 1]) {
          bF[k - 1] = d;
          cF[k - 1] = c;
        }
      }
      if (L >= 2) {
        const V d = (V)(szr * (sM1P1 - wr0) + (szc - kk) * ((C)sCA[k - 1][qc] - wck) + (szr - kk) * Sg -
                        szc * wc0 + (C)(c - r) * (sCW[qc + k - 1] - Wc0) - kk * (sCW[qc - 1] - Wr0));
        if (d <= bB[k - 1] && d != kInf) {
          bB[k - 1] = d;
          cB[k - 1] = c;
        }
      }
    }
  }

  if (c2A >= 0)
    atomicMin((unsigned long long*)&keys[off1 + (L - 1)],
              (unsigned long long)make_key((int64_t)b2A, (uint32_t)(c2A - 2), kCtxBits));
  if (c2B >= 0)
    atomicMin((unsigned long long*)&keys[off1 + blk2B],
              (unsigned long long)make_key((int64_t)b2B, (uint32_t)(sz - 2 - c2B), kCtxBits));
#pragma unroll
  for (int k = 1; k <= 3; k++) {
    const int offk = nb_offset(k + 1, sz);
    if (cF[k - 1] >= 0)
      atomicMin((unsigned long long*)&keys[offk + (L - 1)],
                (unsigned long long)make_key((int64_t)bF[k - 1], (uint32_t)(cF[k - 1] - 2), kCtxBits));
    if (cB[k - 1] >= 0)
      atomicMin((unsigned long long*)&keys[offk + (sz - k - 1 - L)],
                (unsigned long long)make_key((int64_t)bB[k - 1], (uint32_t)(sz - k - 1 - cB[k - 1]),
                                             kCtxBits));
  }
}

// --------------------------------------------------------------------------
// Merge.
// --------------------------------------------------------------------------
enum : uint8_t { kNone = 0, kUndec = 1, kIn = 2, kOut = 3 };

// Workspace layout (bytes) of one merge CTA for a given size.
struct MergeLayout {
  int mmax, P, tb;
  size_t cand, structs, stage2, stage3, total;
  __host__ __device__ explicit MergeLayout(int size) {
    mmax = nb_blocks(2, size);
    P = 1;
    while (P < size + 4) P <<= 1;
    tb = total_blocks(size);
    cand = align_up((size_t)mmax * 13, 16);
    const size_t swapB = (size_t)2 * (size + 4) * 8, ivB = (size_t)8 * P * 8;
    structs = swapB > ivB ? swapB : ivB;
    stage2 = cand + structs;
    stage3 = align_up((size_t)tb * 13, 16) + align_up((size_t)size * 4, 16);
    total = align_up(stage2 > stage3 ? stage2 : stage3, 128);
  }
};

__device__ __forceinline__ void amin(uint64_t* p, uint64_t v) {
  atomicMin((unsigned long long*)p, (unsigned long long)v);
}

// Stage 2: greedy independent set of one neighbourhood's negative candidates
// in (delta, block) order with the same-neighbourhood predicate of the
// reference's GPU merge (mlkernel.cu:51-170 after the sort at :256).  Computed
// as the lexicographically-first maximal independent set by rounds; conflicts
// are found with point tables (swap) or segment trees (interval moves).
__device__ void stage2(const JobDev* J, int nb, uint8_t* ws, int* s_cnt) {
  const int sz = J->size, tid = threadIdx.x, nt = blockDim.x;
  const MergeLayout lay(sz);
  const int m = nb_blocks(nb, sz), off = nb_offset(nb, sz);
  uint64_t* skey = (uint64_t*)ws;
  uint32_t* ij = (uint32_t*)(skey + lay.mmax);
  uint8_t* st = (uint8_t*)(ij + lay.mmax);
  uint64_t* sb = (uint64_t*)(ws + lay.cand);
  const uint64_t* keys = J->keys;
  if (tid == 0) *s_cnt = 0;
  for (int x = tid; x < m; x += nt) {
    const uint64_t key = keys[off + x];
    uint8_t s = kNone;
    if (key != kKeyNone) {
      const int64_t cost = key_cost(key, kCtxBits);
      if (cost < 0) {
        int i, j;
        map_move(nb, sz, x, (int)(key & ((1u << kCtxBits) - 1)), i, j);
        skey[x] = make_key(cost, (uint32_t)x, kCtxBits);
        ij[x] = (uint32_t)i | ((uint32_t)j << 16);
        s = kUndec;
      }
    }
    st[x] = s;
  }
  const int P = lay.P;
  uint64_t* minB = sb;                 // swap: endpoint tables
  uint64_t* minK = sb + (sz + 4);
  uint64_t* covB = sb;                 // intervals: range-update / point-query trees
  uint64_t* covK = sb + 2 * P;
  uint64_t* stB = sb + 4 * P;          // point-update / range-query trees
  uint64_t* stK = sb + 6 * P;
  const int nclear = nb == 0 ? 2 * (sz + 4) : 8 * P;
  for (int round = 0; round <= m; round++) {
    for (int q = tid; q < nclear; q += nt) sb[q] = kKeyNone;
    __syncthreads();
    for (int x = tid; x < m; x += nt) {
      const uint8_t s = st[x];
      if (s != kUndec && s != kIn) continue;
      const uint64_t v = skey[x];
      const int i = (int)(ij[x] & 0xffff), j = (int)(ij[x] >> 16);
      if (nb == 0) {
        amin(&minB[i], v);
        amin(&minB[j], v);
        if (s == kIn) {
          amin(&minK[i], v);
          amin(&minK[j], v);
        }
      } else {
        int a0, b0;
        conflict_interval(nb, i, j, a0, b0);
        for (int l = a0 + P, r = b0 + P + 1; l < r; l >>= 1, r >>= 1) {
          if (l & 1) {
            amin(&covB[l], v);
            if (s == kIn) amin(&covK[l], v);
            l++;
          }
          if (r & 1) {
            --r;
            amin(&covB[r], v);
            if (s == kIn) amin(&covK[r], v);
          }
        }
        for (int p = a0 + P; p >= 1; p >>= 1) {
          amin(&stB[p], v);
          if (s == kIn) amin(&stK[p], v);
        }
      }
    }
    __syncthreads();
    int any = 0;
    for (int x = tid; x < m; x += nt) {
      if (st[x] != kUndec) continue;
      const uint64_t v = skey[x];
      const int i = (int)(ij[x] & 0xffff), j = (int)(ij[x] >> 16);
      uint64_t qB = kKeyNone, qK = kKeyNone;
      if (nb == 0) {
#pragma unroll
        for (int e = -1; e <= 1; e++) {
          qB = min(qB, min(minB[i + e], minB[j + e]));
          qK = min(qK, min(minK[i + e], minK[j + e]));
        }
      } else {
        int a0, b0;
        conflict_interval(nb, i, j, a0, b0);
        for (int p = a0 + P; p >= 1; p >>= 1) {
          qB = min(qB, covB[p]);
          qK = min(qK, covK[p]);
        }
        for (int l = a0 + 1 + P, r = b0 + 1 + P; l < r; l >>= 1, r >>= 1) {
          if (l & 1) {
            qB = min(qB, stB[l]);
            qK = min(qK, stK[l]);
            l++;
          }
          if (r & 1) {
            --r;
            qB = min(qB, stB[r]);
            qK = min(qK, stK[r]);
          }
        }
      }
      if (qK < v) st[x] = kOut;
      else if (qB >= v) st[x] = kIn;
      else any = 1;
    }
    if (!__syncthreads_or(any)) break;
  }
  uint64_t* kept = J->kept;
  for (int x = tid; x < m; x += nt) {
    if (st[x] != kIn) continue;
    const int q = atomicAdd(s_cnt, 1);
    const int64_t cost = key_cost(skey[x], kCtxBits);
    kept[2 * (off + q)] = make_key(cost, ((uint32_t)nb << kCtxBits) | (uint32_t)x, kCtxBits + 3);
    kept[2 * (off + q) + 1] = ij[x];
  }
  __syncthreads();
  if (tid == 0) J->kept_count[nb] = *s_cnt;
}

// Stage 3 (cross-neighbourhood greedy with canMerge, mlkernel.cu:649-864 with a
// stable order), parallel apply of the selected moves (footprints are disjoint
// for every pair canMerge accepts), prefix rebuild and key reset.
template <bool WIDE>
__device__ void stage3_apply(const JobDev* J, uint8_t* ws) {
  __shared__ int s_m3, s_ns;
  const int sz = J->size, tid = threadIdx.x, nt = blockDim.x;
  const MergeLayout lay(sz);
  uint64_t* key3 = (uint64_t*)ws;
  uint32_t* ij3 = (uint32_t*)(key3 + lay.tb);
  volatile uint8_t* st3 = (volatile uint8_t*)(ij3 + lay.tb);
  int32_t* owner = (int32_t*)(ws + align_up((size_t)lay.tb * 13, 16));
  if (tid == 0) {
    int m3 = 0;
    for (int nb = 0; nb < kNumNb; nb++) m3 += ((volatile int32_t*)J->kept_count)[nb];
    s_m3 = m3;
    s_ns = 0;
  }
  __syncthreads();
  const int m3 = s_m3;
  {
    int base = 0;
    for (int nb = 0; nb < kNumNb; nb++) {
      const int cnt = ((volatile int32_t*)J->kept_count)[nb];
      const int off = nb_offset(nb, sz);
      for (int q = tid; q < cnt; q += nt) {
        key3[base + q] = ((volatile uint64_t*)J->kept)[2 * (off + q)];
        ij3[base + q] = (uint32_t)((volatile uint64_t*)J->kept)[2 * (off + q) + 1];
        st3[base + q] = kUndec;
      }
      base += cnt;
    }
  }
  __syncthreads();
  for (int round = 0; round <= m3; round++) {
    int any = 0;
    for (int x = tid; x < m3; x += nt) {
      if (st3[x] != kUndec) continue;
      const uint64_t kx = key3[x];
      const int idx = (int)((kx >> kCtxBits) & 7);
      const int ix = (int)(ij3[x] & 0xffff), jx = (int)(ij3[x] >> 16);
      bool out = false, blocked = false;
      for (int y = 0; y < m3; y++) {
        const uint64_t ky = key3[y];
        if (ky >= kx) continue;
        const uint8_t sy = st3[y];
        if (sy != kUndec && sy != kIn) continue;
        const int idy = (int)((ky >> kCtxBits) & 7);
        if (can_merge(idy, (int)(ij3[y] & 0xffff), (int)(ij3[y] >> 16), idx, ix, jx)) continue;
        if (sy == kIn) {
          out = true;
          break;
        }
        blocked = true;
      }
      if (out) st3[x] = kOut;
      else if (!blocked) st3[x] = kIn;
      else any = 1;
    }
    if (!__syncthreads_or(any)) break;
  }
  // ---- apply ----
  for (int p = tid; p < sz; p += nt) owner[p] = -1;
  __syncthreads();
  const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  for (int x = wid; x < m3; x += nw) {
    if (st3[x] != kIn) continue;
    const int id = (int)((key3[x] >> kCtxBits) & 7);
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
  int32_t* tour = J->tour;
  int32_t* alt = J->tour_alt;
  for (int p = tid; p < sz; p += nt) {
    const int o = owner[p];
    int src = p;
    if (o >= 0) {
      const int id = (int)((key3[o] >> kCtxBits) & 7);
      src = move_source(id, (int)(ij3[o] & 0xffff), (int)(ij3[o] >> 16), p);
    }
    alt[p] = tour[src];
  }
  __syncthreads();
  for (int p = tid; p < sz; p += nt) tour[p] = alt[p];
  const int ns = s_ns;
  // Applied moves in (delta, neighbourhood, block) order, for callers that
  // ask for them (the legacy bestNeighbor move vectors).
  if (J->moves_out != nullptr) {
    for (int x = tid; x < m3; x += nt) {
      if (st3[x] != kIn) continue;
      int rank = 0;
      for (int y = 0; y < m3; y++)
        if (st3[y] == kIn && key3[y] < key3[x]) rank++;
      if (rank < J->moves_cap) {
        const uint32_t id = (uint32_t)((key3[x] >> kCtxBits) & 7);
        const uint32_t i = ij3[x] & 0xffff, j = ij3[x] >> 16;
        J->moves_out[rank] = id | (i << 4) | (j << 18);
        J->moves_cost[rank] = key_cost(key3[x], kCtxBits + 3);
      }
    }
  }
  __syncthreads();
  if (tid == 0) {
    int64_t* stt = J->stats;
    stt[kStatSweeps] += 1;
    stt[kStatLastMoves] = ns;
    stt[kStatMoves] += ns;
    if (ns > 0) stt[kStatIters] += 1;
    else stt[kStatConverged] = 1;
    stt[kStatDone] = 0;
  }
  cta_prepare<WIDE>(J);
  cta_reset_keys(J);
}

template <bool WIDE>
__global__ void __launch_bounds__(1024) k_merge(const JobDev* __restrict__ jobs, int use_smem) {
  extern __shared__ __align__(16) uint8_t dsm[];
  __shared__ int s_cnt, s_last;
  const int job = blockIdx.x / kNumNb, nb = blockIdx.x % kNumNb;
  const JobDev* J = jobs + job;
  {
    const int64_t* stt = J->stats;
    if (stt[kStatConverged] || stt[kStatSweeps] >= stt[kStatLimit]) return;
  }
  const MergeLayout lay(J->size);
  uint8_t* ws = use_smem ? dsm : (J->ws + (size_t)nb * lay.total);
  if ((J->nb_mask >> nb) & 1) {
    stage2(J, nb, ws, &s_cnt);
  } else if (threadIdx.x == 0) {
    J->kept_count[nb] = 0;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long prev = atomicAdd((unsigned long long*)&J->stats[kStatDone], 1ull);
    s_last = prev == (unsigned long long)(kNumNb - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  stage3_apply<WIDE>(J, ws);
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
cudaError_t sweep_launch(const SweepTile* tiles, int ntiles, const JobDev* jobs, cudaStream_t s) {
  k_sweep<WIDE, TL, TR><<<ntiles, TL, 0, s>>>(tiles, jobs);
  return cudaGetLastError();
}

template <bool WIDE>
cudaError_t sweep_dispatch(const SweepTile* tiles, int ntiles, const JobDev* jobs, int shape,
                           cudaStream_t s) {
  switch (shape) {
    case 0: return sweep_launch<WIDE, 32, 16>(tiles, ntiles, jobs, s);
    case 1: return sweep_launch<WIDE, 64, 8>(tiles, ntiles, jobs, s);
    case 2: return sweep_launch<WIDE, 64, 16>(tiles, ntiles, jobs, s);
    case 3: return sweep_launch<WIDE, 64, 32>(tiles, ntiles, jobs, s);
    case 4: return sweep_launch<WIDE, 128, 16>(tiles, ntiles, jobs, s);
    case 5: return sweep_launch<WIDE, 128, 32>(tiles, ntiles, jobs, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

size_t merge_smem_bytes(int size) { return MergeLayout(size).total; }
size_t merge_ws_bytes(int size) { return MergeLayout(size).total * kNumNb; }
int merge_smem_max_size() { return 2044; }

cudaError_t launch_prepare(const JobDev* jobs, int njobs, bool wide, bool reset_stats,
                           cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  if (wide) k_prepare<true><<<njobs, 1024, 0, s>>>(jobs, reset_stats ? 1 : 0);
  else k_prepare<false><<<njobs, 1024, 0, s>>>(jobs, reset_stats ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_sweep(const SweepTile* tiles, int ntiles, const JobDev* jobs, bool wide,
                         int shape, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  return wide ? sweep_dispatch<true>(tiles, ntiles, jobs, shape, s)
              : sweep_dispatch<false>(tiles, ntiles, jobs, shape, s);
}

cudaError_t configure_merge(size_t bytes) {
  cudaError_t e = cudaFuncSetAttribute(k_merge<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_merge<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t launch_merge(const JobDev* jobs, int njobs, bool wide, bool use_smem, int max_size,
                         cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  const size_t smem = use_smem ? MergeLayout(max_size).total : 0;
  if (wide) k_merge<true><<<njobs * kNumNb, 1024, smem, s>>>(jobs, use_smem ? 1 : 0);
  else k_merge<false><<<njobs * kNumNb, 1024, smem, s>>>(jobs, use_smem ? 1 : 0);
  return cudaGetLastError();
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
