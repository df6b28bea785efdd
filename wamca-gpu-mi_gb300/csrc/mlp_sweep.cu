// mlp_sweep.cu -- the DVND sweep of 32-bit jobs over all five neighbourhoods.
//
// The same evaluation as k_sweep (mlp_kernels.cu) in its DVND mode -- every
// swap, 2-opt and Or-opt-1/2/3 move of the ODC kernels' block -> (i, j)
// mapping (source/mlkswap.cu:766-785, mlk2opt.cu:561-572, mlkoropt.cu:701-737),
// each reference block's best improving candidate published as a 64-bit
// (delta, ctx) key with atomicMin -- with each delta rewritten as
//   delta(r, c) = term(r) + term(c) + a few products of the pair's distances
// (the split is given in mlp_common.cuh at kTermWords).  The row and column
// terms are computed once per iteration by the ADS rebuild and read here as
// three 16-byte shared-memory words per row and per column, so a pair costs
// about 28 integer operations for its eight deltas instead of about 100, and
// the pair's validity (the tour's end, L >= 2) is folded into the predicates
// of the running minima instead of branches.  All arithmetic is modulo 2^32,
// which reproduces the reference's 32-bit results exactly.
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp_common.cuh"
#include "mlp_kernels.cuh"

namespace mlp {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int32_t kInf32 = 0x7fffffff;

// Publishes the improving minima of diagonal L's blocks (2-opt A and B,
// Or-opt-k forward and backward) found over a tile's rows; the pair of row a
// on this diagonal is (r0 + a - 1, r0 + a - 1 + L).  Block and ctx as in k_sweep.
__device__ __forceinline__ void publish_diagonal(uint64_t* keys, int sz, int r0, int L, int32_t b2, int a2A, int a2B,
                                                 int32_t bF1, int32_t bF2, int32_t bF3, int aF1, int aF2, int aF3,
                                                 int32_t bB1, int32_t bB2, int32_t bB3, int aB1, int aB2, int aB3) {
  const int cbase = r0 - 1 + L;
  const int nb2 = nb_blocks(1, sz), off1 = nb_offset(1, sz);
  if (b2 < 0) {
    if (L - 1 < nb2)
      atomicMin((unsigned long long*)&keys[off1 + (L - 1)],
                (unsigned long long)make_key((int64_t)b2, (uint32_t)(cbase + a2A - 2), kCtxBits));
    const int blk2B = sz - 2 - L;
    if (blk2B >= 0 && blk2B < nb2)
      atomicMin((unsigned long long*)&keys[off1 + blk2B],
                (unsigned long long)make_key((int64_t)b2, (uint32_t)(sz - 2 - (cbase + a2B)), kCtxBits));
  }
  const int32_t bF[3] = {bF1, bF2, bF3}, bB[3] = {bB1, bB2, bB3};
  const int aF[3] = {aF1, aF2, aF3}, aB[3] = {aB1, aB2, aB3};
#pragma unroll
  for (int k = 1; k <= 3; k++) {
    const int offk = nb_offset(k + 1, sz);
    if (bF[k - 1] < 0)
      atomicMin((unsigned long long*)&keys[offk + (L - 1)],
                (unsigned long long)make_key((int64_t)bF[k - 1], (uint32_t)(cbase + aF[k - 1] - 2), kCtxBits));
    if (L >= 2 && bB[k - 1] < 0)
      atomicMin((unsigned long long*)&keys[offk + (sz - k - 1 - L)],
                (unsigned long long)make_key((int64_t)bB[k - 1], (uint32_t)(sz - k - 1 - (cbase + aB[k - 1])),
                                             kCtxBits));
  }
}

// Tile: rows r in [r0, r0 + TR), diagonals L in [L0, L0 + TL); thread tid owns
// diagonal L = L0 + tid (c = r + L).  Distances E(x, y) = D[t[x]][t[y]] are
// staged in skewed layout sS[a][b] = E(r0 - 1 + a, r0 - 1 + a + L0 - 1 + b);
// row a (1-based) is r = r0 + a - 1, and thread tid reads column b = tid + 1.
// LOCAL: the tile computes its rows' and columns' terms from the prefix arrays
// itself (a job set of one search: the ADS rebuild, on one SM, then writes no
// term tables; here the work is spread over every tile).
// CAP: registers capped at 64 a thread (more CTAs resident per SM), for
// grids that then fit in one wave when they otherwise would not.
template <int TL, int TR, bool LOCAL, bool CAP = false>
__global__ void __launch_bounds__(TL, CAP ? 1024 / TL : 1) k_sweep_dvnd(const SweepTile* __restrict__ tiles,
                                                   const JobDev* __restrict__ jobs) {
  constexpr int SR = TR + 3, SC = TL + 3, NT = TR + TL + 5, NCS = TL + TR - 1;
  __shared__ int32_t sS[SR][SC];
  __shared__ int32_t sRowT[SR];
  __shared__ int32_t sColT[NT];
  __shared__ int4 sRt[TR][3];
  __shared__ int4 sCt[NCS][3];

  const SweepTile tile = tiles[blockIdx.x];
  const JobDev* J = jobs + tile.job;
  const int64_t* stats = J->stats;
  const int sz = J->size, n = J->n;
  const int r0 = tile.r0, L0 = tile.L0, tid = threadIdx.x;
  const int32_t* __restrict__ t = J->tour;
  const int32_t* __restrict__ D = J->D;
  const int4* __restrict__ RT = reinterpret_cast<const int4*>(J->RT);
  const int4* __restrict__ CT = reinterpret_cast<const int4*>(J->CT);
  // The previous merge's tour, prefix arrays, statistics and key reset are
  // complete past this point; the next merge may then be launched.
  pdl_wait();
  pdl_launch_dependents();
  const bool done = stats[kStatConverged] || stats[kStatSweeps] >= stats[kStatLimit];
  {
    // Tour entries of the tile's rows and columns and the term words of its
    // rows and columns: every load issued before any store.
    constexpr int kSR = (SR + TL - 1) / TL, kNT = (NT + TL - 1) / TL;
    int32_t vRT[kSR], vCT[kNT];
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
    if constexpr (LOCAL) {
      // Term inputs of the tile's TR rows and NCS columns (struct s < TR: row
      // r0 + s; else column r0 + L0 + s - TR), then the terms themselves.
      constexpr int kS = (TR + NCS + TL - 1) / TL;
      const int32_t* __restrict__ w = J->w;
      const uint32_t* __restrict__ Wg = (const uint32_t*)J->W;
      const uint32_t* __restrict__ Qg = (const uint32_t*)J->Q;
      const int32_t* __restrict__ Ag = J->A;
      const int pad = sz + 8;
      TermIn xin[kS];
#pragma unroll
      for (int u = 0; u < kS; u++) {
        const int s = tid + u * TL, p = s < TR ? r0 + s : r0 + L0 + (s - TR);
        TermIn x{};
        if (s < TR + NCS && p <= sz - 1) {
          x.w0 = (uint32_t)w[p];
          x.w1 = (uint32_t)w[p + 1];  // zero at and beyond sz (arrays padded to sz + 8)
          x.w2 = (uint32_t)w[p + 2];
          x.w3 = (uint32_t)w[p + 3];
          x.W = Wg[p];
          x.Q = Qg[p];
          x.A1 = (uint32_t)Ag[p];
          x.A2 = (uint32_t)Ag[pad + p];
          x.A3 = (uint32_t)Ag[2 * pad + p];
        }
        xin[u] = x;
      }
#pragma unroll
      for (int u = 0; u < kS; u++) {
        const int s = tid + u * TL;
        if (s < TR) {
          row_terms(xin[u], r0 + s, sz, sRt[s][0], sRt[s][1], sRt[s][2]);
        } else if (s < TR + NCS) {
          const int q = s - TR;
          col_terms(xin[u], r0 + L0 + q, sz, sCt[q][0], sCt[q][1], sCt[q][2]);
        }
      }
    } else {
      constexpr int kR = (3 * TR + TL - 1) / TL, kC = (3 * NCS + TL - 1) / TL;
      int4 vR[kR], vC[kC];
#pragma unroll
      for (int u = 0; u < kR; u++) {
        const int q = tid + u * TL, p = r0 + q / 3;
        vR[u] = (q < 3 * TR && p <= sz - 1) ? __ldg(RT + (size_t)p * 3 + q % 3) : make_int4(0, 0, 0, 0);
      }
#pragma unroll
      for (int u = 0; u < kC; u++) {
        const int q = tid + u * TL, p = r0 + L0 + q / 3;
        vC[u] = (q < 3 * NCS && p <= sz - 1) ? __ldg(CT + (size_t)p * 3 + q % 3) : make_int4(0, 0, 0, 0);
      }
#pragma unroll
      for (int u = 0; u < kR; u++) {
        const int q = tid + u * TL;
        if (q < 3 * TR) sRt[q / 3][q % 3] = vR[u];
      }
#pragma unroll
      for (int u = 0; u < kC; u++) {
        const int q = tid + u * TL;
        if (q < 3 * NCS) sCt[q / 3][q % 3] = vC[u];
      }
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
  }
  __syncthreads();
  if (done) return;
  {
    // The tile's distances: all gathers issued before any store (at most GB
    // loads a thread in flight at once).
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

  const int L = L0 + tid, b = tid + 1, lane = tid & 31;
  const bool L2 = L >= 2;
  const int rows = min(TR, sz - 2 - r0);  // rows r <= sz - 3
  // Distances around the pair (r, c): e1 = E(r-1, c), e2 = E(r+1, c),
  // e3 = E(r, c-1), e4 = E(r, c+1), e5 = E(r, c), e6 = E(r+1, c+2),
  // e7 = E(r, c+2), e8 = E(r+2, c+3); row a + 1's e1, e3, e4, e6 are row a's
  // e4, e2, e6, e8.
  uint32_t e1 = (uint32_t)sS[0][b + 1], e3 = (uint32_t)sS[1][b - 1], e4 = (uint32_t)sS[1][b + 1],
           e6 = (uint32_t)sS[2][b + 1];
  // s_r = sz - r and s_c = sz - c of row a.
  uint32_t sr = (uint32_t)(sz - r0), sc = (uint32_t)(sz - r0 - L);
  // Running minima of the diagonal-owned blocks and the row (a) where each
  // was found: 2-opt (strict for block A, first row; <= for block B, last
  // row), Or-opt-k forward (strict) and backward (<=).
  int32_t b2 = kInf32, bF1 = kInf32, bF2 = kInf32, bF3 = kInf32, bB1 = kInf32, bB2 = kInf32, bB3 = kInf32;
  int a2A = 0, a2B = 0, aF1 = 0, aF2 = 0, aF3 = 0, aB1 = 0, aB2 = 0, aB3 = 0;
  uint64_t* keys = J->keys;
  const int nbS = nb_blocks(0, sz);
#pragma unroll 2
  for (int a = 1; a <= rows; a++) {
    const uint32_t e2 = (uint32_t)sS[a + 1][b - 1], e5 = (uint32_t)sS[a][b], e7 = (uint32_t)sS[a][b + 2],
                   e8 = (uint32_t)sS[a + 2][b + 1];
    const int4 R0 = sRt[a - 1][0], R1 = sRt[a - 1][1], R2 = sRt[a - 1][2];
    const int4 C0 = sCt[a - 1 + tid][0], C1 = sCt[a - 1 + tid][1], C2 = sCt[a - 1 + tid][2];
    // Validity: c <= sz - 2 (swap, 2-opt, Or-opt-1), c <= sz - 3 (Or-opt-2),
    // c <= sz - 4 (Or-opt-3); swap and backward Or-opt also need L >= 2.
    const int isc = (int)sc;
    const bool v1 = isc >= 2, v2 = isc >= 3, v3 = isc >= 4;
    const uint32_t P1 = sr * e1, P4 = (sc - 1u) * e4;
    // swap: (s_r - 1) e2 + s_c e3 + P1 + P4 + S(r) + S(c)
    const int32_t dS = (int32_t)((sr - 1u) * e2 + sc * e3 + P1 + P4 + (uint32_t)R0.x + (uint32_t)C0.x);
    // 2-opt: -s_c W[r] + s_r W[c] + P1 + P4 + R2 + C2
    const int32_t d2 = (int32_t)(sc * (uint32_t)R2.x + sr * (uint32_t)C2.x + P1 + P4 + (uint32_t)R0.y + (uint32_t)C0.y);
    // Or-opt-k forward: (s_c - k) E(r+k-1, c+k) + s_c (E(r, c+k-1) + V_k(r)) + RF_k + CF_k
    const int32_t f1 = (int32_t)(sc * e5 + P4 + (uint32_t)R0.z + (uint32_t)C0.z);
    const int32_t f2 = (int32_t)((sc - 2u) * e6 + sc * (e4 + (uint32_t)R2.y) + (uint32_t)R0.w + (uint32_t)C0.w);
    const int32_t f3 = (int32_t)((sc - 3u) * e8 + sc * (e7 + (uint32_t)R2.z) + (uint32_t)R1.x + (uint32_t)C1.x);
    // Or-opt-k backward: (s_r - k) E(r, c+k-1) + s_r V_k(c) + P1 + RB_k + CB_k
    const int32_t g1 = (int32_t)((sr - 1u) * e5 + P1 + (uint32_t)R1.y + (uint32_t)C1.y);
    const int32_t g2 = (int32_t)((sr - 2u) * e4 + sr * (uint32_t)C2.y + P1 + (uint32_t)R1.z + (uint32_t)C1.z);
    const int32_t g3 = (int32_t)((sr - 3u) * e7 + sr * (uint32_t)C2.z + P1 + (uint32_t)R1.w + (uint32_t)C1.w);

    // swap: the row's blocks (A: by = r - 1, B: by = sz - 3 - r) take the
    // warp's minimum, ties to the lowest ctx (A: lowest lane, B: highest).
    {
      const uint32_t u = (v1 && L2) ? ((uint32_t)dS ^ 0x80000000u) : 0xffffffffu;
      const uint32_t mn = __reduce_min_sync(kFull, u);
      if (mn < 0x80000000u) {
        const unsigned ties = __ballot_sync(kFull, u == mn);
        const int r = r0 + a - 1, c = r + L;
        const int blkA = r - 1, blkB = sz - 3 - r;
        if (blkA < nbS && lane == __ffs(ties) - 1)
          atomicMin((unsigned long long*)&keys[blkA],
                    (unsigned long long)make_key((int64_t)dS, (uint32_t)(c - 3), kCtxBits));
        if (blkB >= 0 && blkB < nbS && lane == 31 - __clz(ties))
          atomicMin((unsigned long long*)&keys[blkB],
                    (unsigned long long)make_key((int64_t)dS, (uint32_t)(sz - 2 - c), kCtxBits));
      }
    }
    {
      const bool lt = v1 && d2 < b2, le = v1 && d2 <= b2;
      a2A = lt ? a : a2A;
      a2B = le ? a : a2B;
      b2 = lt ? d2 : b2;
    }
#define MLP_TRACK_LT(v, d, best, arg) \
  {                                   \
    const bool up = (v) && (d) < (best); \
    best = up ? (d) : best;           \
    arg = up ? a : arg;               \
  }
#define MLP_TRACK_LE(v, d, best, arg) \
  {                                   \
    const bool up = (v) && (d) <= (best); \
    best = up ? (d) : best;           \
    arg = up ? a : arg;               \
  }
    MLP_TRACK_LT(v1, f1, bF1, aF1)
    MLP_TRACK_LT(v2, f2, bF2, aF2)
    MLP_TRACK_LT(v3, f3, bF3, aF3)
    MLP_TRACK_LE(v1, g1, bB1, aB1)
    MLP_TRACK_LE(v2, g2, bB2, aB2)
    MLP_TRACK_LE(v3, g3, bB3, aB3)
#undef MLP_TRACK_LT
#undef MLP_TRACK_LE
    e1 = e4;
    e3 = e2;
    e4 = e6;
    e6 = e8;
    sr -= 1u;
    sc -= 1u;
  }

  publish_diagonal(keys, sz, r0, L, b2, a2A, a2B, bF1, bF2, bF3, aF1, aF2, aF3, bB1, bB2, bB3, aB1, aB2, aB3);
}

// The same sweep with two adjacent diagonals per thread: thread tid owns
// L = L0 + 2 tid and L + 1 (skewed columns b = 2 tid + 1 and b + 1).  Row by
// row, diagonal L + 1's column term becomes diagonal L's in the next row, so
// a thread reads one column term (three 16-byte words) per row for two pairs,
// and the new distances of a row arrive as one 4-byte and two 8-byte loads.
// Column terms are stored by the parity of their index so that the lanes of
// a warp read consecutive 48-byte words (no bank conflicts).  Results are
// identical to k_sweep_dvnd's.
template <int TLD, int TR>
__global__ void __launch_bounds__(TLD / 2) k_sweep_dvnd2(const SweepTile* __restrict__ tiles,
                                                         const JobDev* __restrict__ jobs) {
  constexpr int NTH = TLD / 2;
  constexpr int SR = TR + 3, SCV = TLD + 3, SC = TLD + 4, NT = TR + TLD + 5, NCS = TLD + TR - 1;
  constexpr int NCE = (NCS + 1) / 2;
  __shared__ __align__(16) int32_t sS[SR][SC];
  __shared__ int32_t sRowT[SR];
  __shared__ int32_t sColT[NT];
  __shared__ int4 sRt[TR][3];
  __shared__ int4 sCt[2][NCE][3];  // column term q at [q & 1][q >> 1]

  const SweepTile tile = tiles[blockIdx.x];
  const JobDev* J = jobs + tile.job;
  const int64_t* stats = J->stats;
  const int sz = J->size, n = J->n;
  const int r0 = tile.r0, L0 = tile.L0, tid = threadIdx.x;
  const int32_t* __restrict__ t = J->tour;
  const int32_t* __restrict__ D = J->D;
  const int4* __restrict__ RT = reinterpret_cast<const int4*>(J->RT);
  const int4* __restrict__ CT = reinterpret_cast<const int4*>(J->CT);
  // The previous merge's tour, prefix arrays, statistics and key reset are
  // complete past this point; the next merge may then be launched.
  pdl_wait();
  pdl_launch_dependents();
  const bool done = stats[kStatConverged] || stats[kStatSweeps] >= stats[kStatLimit];
  {
    constexpr int kSR = (SR + NTH - 1) / NTH, kNT = (NT + NTH - 1) / NTH;
    constexpr int kR = (3 * TR + NTH - 1) / NTH, kC = (3 * NCS + NTH - 1) / NTH;
    int32_t vRT[kSR], vCT[kNT];
    int4 vR[kR], vC[kC];
#pragma unroll
    for (int u = 0; u < kSR; u++) {
      const int q = tid + u * NTH, p = r0 - 1 + q;
      vRT[u] = (q < SR && p <= sz - 1) ? t[p] : 0;
    }
#pragma unroll
    for (int u = 0; u < kNT; u++) {
      const int q = tid + u * NTH, p = r0 + L0 - 2 + q;
      vCT[u] = (q < NT && p <= sz - 1) ? t[p] : 0;
    }
#pragma unroll
    for (int u = 0; u < kR; u++) {
      const int q = tid + u * NTH, p = r0 + q / 3;
      vR[u] = (q < 3 * TR && p <= sz - 1) ? __ldg(RT + (size_t)p * 3 + q % 3) : make_int4(0, 0, 0, 0);
    }
#pragma unroll
    for (int u = 0; u < kC; u++) {
      const int q = tid + u * NTH, p = r0 + L0 + q / 3;
      vC[u] = (q < 3 * NCS && p <= sz - 1) ? __ldg(CT + (size_t)p * 3 + q % 3) : make_int4(0, 0, 0, 0);
    }
#pragma unroll
    for (int u = 0; u < kSR; u++) {
      const int q = tid + u * NTH;
      if (q < SR) sRowT[q] = vRT[u];
    }
#pragma unroll
    for (int u = 0; u < kNT; u++) {
      const int q = tid + u * NTH;
      if (q < NT) sColT[q] = vCT[u];
    }
#pragma unroll
    for (int u = 0; u < kR; u++) {
      const int q = tid + u * NTH;
      if (q < 3 * TR) sRt[q / 3][q % 3] = vR[u];
    }
#pragma unroll
    for (int u = 0; u < kC; u++) {
      const int q = tid + u * NTH;
      if (q < 3 * NCS) {
        const int col = q / 3;
        sCt[col & 1][col >> 1][q % 3] = vC[u];
      }
    }
  }
  __syncthreads();
  if (done) return;
  {
    constexpr int NG = (SR * SCV + NTH - 1) / NTH, GB = 21;
#pragma unroll
    for (int u0 = 0; u0 < NG; u0 += GB) {
      int32_t gv[GB];
#pragma unroll
      for (int u = 0; u < GB; u++) {
        const int idx = tid + (u0 + u) * NTH;
        int32_t v = 0;
        if (u0 + u < NG && idx < SR * SCV) {
          const int a = idx / SCV, bb = idx - a * SCV;
          const int rp = r0 - 1 + a, cp = rp + L0 - 1 + bb;
          if (rp <= sz - 1 && cp <= sz - 1) v = __ldg(D + (size_t)sRowT[a] * n + sColT[a + bb]);
        }
        gv[u] = v;
      }
#pragma unroll
      for (int u = 0; u < GB; u++) {
        const int idx = tid + (u0 + u) * NTH;
        if (u0 + u < NG && idx < SR * SCV) {
          const int a = idx / SCV, bb = idx - a * SCV;
          sS[a][bb] = gv[u];
        }
      }
    }
  }
  __syncthreads();

  const int L = L0 + 2 * tid, b = 2 * tid + 1, lane = tid & 31;
  const bool L2 = L >= 2;  // diagonal L + 1 >= 2 always
  const int rows = min(TR, sz - 2 - r0);
  // Distances carried into row a: row a-1 at b+1, b+2 (x1, x2); row a at
  // b-1 .. b+2 (y0..y3); row a+1 at b+1, b+2 (z2, z3).
  uint32_t x1 = (uint32_t)sS[0][b + 1], x2 = (uint32_t)sS[0][b + 2];
  uint32_t y0 = (uint32_t)sS[1][b - 1], y1 = (uint32_t)sS[1][b], y2 = (uint32_t)sS[1][b + 1], y3 = (uint32_t)sS[1][b + 2];
  uint32_t z2 = (uint32_t)sS[2][b + 1], z3 = (uint32_t)sS[2][b + 2];
  uint32_t sr = (uint32_t)(sz - r0), sc = (uint32_t)(sz - r0 - L);
  // Column term of diagonal L at row 1 (index 2 tid, even).
  int4 K0 = sCt[0][tid][0], K1 = sCt[0][tid][1], K2 = sCt[0][tid][2];
  int32_t b2 = kInf32, bF1 = kInf32, bF2 = kInf32, bF3 = kInf32, bB1 = kInf32, bB2 = kInf32, bB3 = kInf32;
  int32_t c2 = kInf32, cF1 = kInf32, cF2 = kInf32, cF3 = kInf32, cB1 = kInf32, cB2 = kInf32, cB3 = kInf32;
  int a2A = 0, a2B = 0, aF1 = 0, aF2 = 0, aF3 = 0, aB1 = 0, aB2 = 0, aB3 = 0;
  int d2A = 0, d2B = 0, dF1 = 0, dF2 = 0, dF3 = 0, dB1 = 0, dB2 = 0, dB3 = 0;
  uint64_t* keys = J->keys;
  const int nbS = nb_blocks(0, sz);
#pragma unroll 2
  for (int a = 1; a <= rows; a++) {
    // New distances: row a at b+3, row a+1 at b-1 and b, row a+2 at b+1 and b+2.
    const uint32_t y4 = (uint32_t)sS[a][b + 3];
    const int2 zz = *reinterpret_cast<const int2*>(&sS[a + 1][b - 1]);
    const int2 uu = *reinterpret_cast<const int2*>(&sS[a + 2][b + 1]);
    const uint32_t z0 = (uint32_t)zz.x, z1 = (uint32_t)zz.y, u1 = (uint32_t)uu.x, u2 = (uint32_t)uu.y;
    const int4 R0 = sRt[a - 1][0], R1 = sRt[a - 1][1], R2 = sRt[a - 1][2];
    // Column term of diagonal L + 1 (index a + 2 tid).
    const int4 N0 = sCt[a & 1][(a >> 1) + tid][0], N1 = sCt[a & 1][(a >> 1) + tid][1],
               N2 = sCt[a & 1][(a >> 1) + tid][2];
    const int isc = (int)sc;
    const bool v1 = isc >= 2, v2 = isc >= 3, v3 = isc >= 4, v4 = isc >= 5;
    const uint32_t P1 = sr * x1, P4 = (sc - 1u) * y2, Q1 = sr * x2, Q4 = (sc - 2u) * y3;
    const uint32_t sd = sc - 1u;  // s_c of diagonal L + 1
    // Diagonal L: e1 = x1, e2 = z0, e3 = y0, e4 = y2, e5 = y1, e6 = z2, e7 = y3, e8 = u1.
    const int32_t dS = (int32_t)((sr - 1u) * z0 + sc * y0 + P1 + P4 + (uint32_t)R0.x + (uint32_t)K0.x);
    const int32_t d2 = (int32_t)(sc * (uint32_t)R2.x + sr * (uint32_t)K2.x + P1 + P4 + (uint32_t)R0.y + (uint32_t)K0.y);
    const int32_t f1 = (int32_t)(sc * y1 + P4 + (uint32_t)R0.z + (uint32_t)K0.z);
    const int32_t f2 = (int32_t)((sc - 2u) * z2 + sc * (y2 + (uint32_t)R2.y) + (uint32_t)R0.w + (uint32_t)K0.w);
    const int32_t f3 = (int32_t)((sc - 3u) * u1 + sc * (y3 + (uint32_t)R2.z) + (uint32_t)R1.x + (uint32_t)K1.x);
    const int32_t g1 = (int32_t)((sr - 1u) * y1 + P1 + (uint32_t)R1.y + (uint32_t)K1.y);
    const int32_t g2 = (int32_t)((sr - 2u) * y2 + sr * (uint32_t)K2.y + P1 + (uint32_t)R1.z + (uint32_t)K1.z);
    const int32_t g3 = (int32_t)((sr - 3u) * y3 + sr * (uint32_t)K2.z + P1 + (uint32_t)R1.w + (uint32_t)K1.w);
    // Diagonal L + 1: e1 = x2, e2 = z1, e3 = y1, e4 = y3, e5 = y2, e6 = z3, e7 = y4, e8 = u2.
    const int32_t eS = (int32_t)((sr - 1u) * z1 + sd * y1 + Q1 + Q4 + (uint32_t)R0.x + (uint32_t)N0.x);
    const int32_t e2 = (int32_t)(sd * (uint32_t)R2.x + sr * (uint32_t)N2.x + Q1 + Q4 + (uint32_t)R0.y + (uint32_t)N0.y);
    const int32_t h1 = (int32_t)(sd * y2 + Q4 + (uint32_t)R0.z + (uint32_t)N0.z);
    const int32_t h2 = (int32_t)((sd - 2u) * z3 + sd * (y3 + (uint32_t)R2.y) + (uint32_t)R0.w + (uint32_t)N0.w);
    const int32_t h3 = (int32_t)((sd - 3u) * u2 + sd * (y4 + (uint32_t)R2.z) + (uint32_t)R1.x + (uint32_t)N1.x);
    const int32_t k1 = (int32_t)((sr - 1u) * y2 + Q1 + (uint32_t)R1.y + (uint32_t)N1.y);
    const int32_t k2 = (int32_t)((sr - 2u) * y3 + sr * (uint32_t)N2.y + Q1 + (uint32_t)R1.z + (uint32_t)N1.z);
    const int32_t k3 = (int32_t)((sr - 3u) * y4 + sr * (uint32_t)N2.z + Q1 + (uint32_t)R1.w + (uint32_t)N1.w);

    // swap: the row's blocks take the minimum over the warp's 64 pairs; ties
    // to the lowest ctx (block A: lowest c; block B: highest c).
    {
      const uint32_t u0 = (v1 && L2) ? ((uint32_t)dS ^ 0x80000000u) : 0xffffffffu;
      const uint32_t u1s = v2 ? ((uint32_t)eS ^ 0x80000000u) : 0xffffffffu;
      const uint32_t um = min(u0, u1s);
      const uint32_t mn = __reduce_min_sync(kFull, um);
      if (mn < 0x80000000u) {
        const unsigned ties = __ballot_sync(kFull, um == mn);
        const int r = r0 + a - 1, c = r + L;
        const int blkA = r - 1, blkB = sz - 3 - r;
        if (blkA < nbS && lane == __ffs(ties) - 1) {
          const bool first = u0 == mn;
          atomicMin((unsigned long long*)&keys[blkA],
                    (unsigned long long)make_key((int64_t)(first ? dS : eS), (uint32_t)(c + (first ? 0 : 1) - 3),
                                                 kCtxBits));
        }
        if (blkB >= 0 && blkB < nbS && lane == 31 - __clz(ties)) {
          const bool second = u1s == mn;
          atomicMin((unsigned long long*)&keys[blkB],
                    (unsigned long long)make_key((int64_t)(second ? eS : dS),
                                                 (uint32_t)(sz - 2 - (c + (second ? 1 : 0))), kCtxBits));
        }
      }
    }
    {
      const bool lt = v1 && d2 < b2, le = v1 && d2 <= b2;
      a2A = lt ? a : a2A;
      a2B = le ? a : a2B;
      b2 = lt ? d2 : b2;
      const bool mt = v2 && e2 < c2, me = v2 && e2 <= c2;
      d2A = mt ? a : d2A;
      d2B = me ? a : d2B;
      c2 = mt ? e2 : c2;
    }
#define MLP_TRACK_LT(v, d, best, arg) \
  {                                   \
    const bool up = (v) && (d) < (best); \
    best = up ? (d) : best;           \
    arg = up ? a : arg;               \
  }
#define MLP_TRACK_LE(v, d, best, arg) \
  {                                   \
    const bool up = (v) && (d) <= (best); \
    best = up ? (d) : best;           \
    arg = up ? a : arg;               \
  }
    MLP_TRACK_LT(v1, f1, bF1, aF1)
    MLP_TRACK_LT(v2, f2, bF2, aF2)
    MLP_TRACK_LT(v3, f3, bF3, aF3)
    MLP_TRACK_LE(v1, g1, bB1, aB1)
    MLP_TRACK_LE(v2, g2, bB2, aB2)
    MLP_TRACK_LE(v3, g3, bB3, aB3)
    MLP_TRACK_LT(v2, h1, cF1, dF1)
    MLP_TRACK_LT(v3, h2, cF2, dF2)
    MLP_TRACK_LT(v4, h3, cF3, dF3)
    MLP_TRACK_LE(v2, k1, cB1, dB1)
    MLP_TRACK_LE(v3, k2, cB2, dB2)
    MLP_TRACK_LE(v4, k3, cB3, dB3)
#undef MLP_TRACK_LT
#undef MLP_TRACK_LE
    x1 = y2;
    x2 = y3;
    y0 = z0;
    y1 = z1;
    y2 = z2;
    y3 = z3;
    z2 = u1;
    z3 = u2;
    K0 = N0;
    K1 = N1;
    K2 = N2;
    sr -= 1u;
    sc -= 1u;
  }
  publish_diagonal(keys, sz, r0, L, b2, a2A, a2B, bF1, bF2, bF3, aF1, aF2, aF3, bB1, bB2, bB3, aB1, aB2, aB3);
  publish_diagonal(keys, sz, r0, L + 1, c2, d2A, d2B, cF1, cF2, cF3, dF1, dF2, dF3, cB1, cB2, cB3, dB1, dB2, dB3);
}

template <int TL, int TR>
cudaError_t sweep_dvnd_launch(const SweepTile* tiles, int ntiles, const JobDev* jobs, bool local, cudaStream_t s) {
  if (local) {
    // Tile-local terms (one search): shapes whose capped kernel does not
    // spill take it when the grid then fits in one wave and otherwise needs
    // a second.
    if constexpr (TL >= 64 && TR <= 8) {
      // Resident CTAs per SM of both copies, and the SM count (queried once;
      // without them, the plain kernel).
      struct Fit {
        int64_t one_wave = 0, one_wave_cap = 0;
      };
      static const Fit fit = [] {
        Fit f;
        int dev = 0, a = 0, b = 0, c = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_sweep_dvnd<TL, TR, true, false>, TL, 0) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_sweep_dvnd<TL, TR, true, true>, TL, 0) == cudaSuccess) {
          f.one_wave = (int64_t)a * c;
          f.one_wave_cap = (int64_t)b * c;
        }
        return f;
      }();
      if ((int64_t)ntiles > fit.one_wave && (int64_t)ntiles <= fit.one_wave_cap)
        return launch_pdl(k_sweep_dvnd<TL, TR, true, true>, dim3(ntiles), dim3(TL), 0, s, tiles, jobs);
    }
    return launch_pdl(k_sweep_dvnd<TL, TR, true>, dim3(ntiles), dim3(TL), 0, s, tiles, jobs);
  }
  return launch_pdl(k_sweep_dvnd<TL, TR, false>, dim3(ntiles), dim3(TL), 0, s, tiles, jobs);
}

}  // namespace

template <int TLD, int TR>
cudaError_t sweep_dvnd2_launch(const SweepTile* tiles, int ntiles, const JobDev* jobs, cudaStream_t s) {
  return launch_pdl(k_sweep_dvnd2<TLD, TR>, dim3(ntiles), dim3(TLD / 2), 0, s, tiles, jobs);
}

cudaError_t launch_sweep_dvnd(const SweepTile* tiles, int ntiles, const JobDev* jobs, int shape, bool local,
                              cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  switch (shape) {
    case 0: return sweep_dvnd_launch<32, 4>(tiles, ntiles, jobs, local, s);
    case 1: return sweep_dvnd_launch<32, 8>(tiles, ntiles, jobs, local, s);
    case 2: return sweep_dvnd_launch<32, 16>(tiles, ntiles, jobs, local, s);
    case 3: return sweep_dvnd_launch<64, 4>(tiles, ntiles, jobs, local, s);
    case 4: return sweep_dvnd_launch<64, 8>(tiles, ntiles, jobs, local, s);
    case 5: return sweep_dvnd_launch<64, 16>(tiles, ntiles, jobs, local, s);
    case 6: return sweep_dvnd_launch<128, 8>(tiles, ntiles, jobs, local, s);
    case 7: return sweep_dvnd_launch<128, 16>(tiles, ntiles, jobs, local, s);
    case 8: return sweep_dvnd_launch<32, 32>(tiles, ntiles, jobs, local, s);
    case 9: return sweep_dvnd_launch<64, 32>(tiles, ntiles, jobs, local, s);
    // Two diagonals per thread from the term tables; with tile-local terms
    // the same tiles run one diagonal per thread.
    case 10: return local ? sweep_dvnd_launch<64, 8>(tiles, ntiles, jobs, true, s)
                          : sweep_dvnd2_launch<64, 8>(tiles, ntiles, jobs, s);
    case 11: return local ? sweep_dvnd_launch<64, 16>(tiles, ntiles, jobs, true, s)
                          : sweep_dvnd2_launch<64, 16>(tiles, ntiles, jobs, s);
    case 12: return local ? sweep_dvnd_launch<64, 32>(tiles, ntiles, jobs, true, s)
                          : sweep_dvnd2_launch<64, 32>(tiles, ntiles, jobs, s);
    case 13: return local ? sweep_dvnd_launch<128, 16>(tiles, ntiles, jobs, true, s)
                          : sweep_dvnd2_launch<128, 16>(tiles, ntiles, jobs, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace mlp
