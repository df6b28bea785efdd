// mlp_total.cu -- the TOTAL multi-improvement's greedy selection (sm_103a).
//
// In TOTAL mode every move a neighbourhood kernel evaluates is a merge
// candidate, not only each block's best (kernelSwapTotal mlkswap.cu:334-526,
// kernel2OptTotal mlk2opt.cu:270-447, kernelOrOptTotal mlkoropt.cu:368-612;
// moveElems = grid.y * block.x, mlkswap.cu:1022).  The reference sorts them
// (mlkernel.cu:256) and zeroes every later move that conflicts with an earlier
// negative one (testSwapTotal / test2OptTotal / testOrOptTotal,
// mlkernel.cu:183-250): the greedy independent set in sorted order, here in
// (delta, i, j) order.
//
// k_total_select: one cluster of up to kTotCl CTAs per (neighbourhood, job).
// Its input is the list of improving moves the collecting sweep appended
// (unordered, up to ~n^2/2 keys), split into one slice per CTA.  It never
// sorts the whole list: it repeatedly
//   1. finds a threshold T with at most kTotBatch keys <= T (histogram of
//      the keys' offsets from the smallest, refined into the lowest bin when
//      that bin alone is too full): every CTA histograms its slice and adds
//      the cluster's histograms through distributed shared memory;
//   2. gathers those keys (the smallest of the list) into every CTA of the
//      cluster and orders them by rank (each CTA ranks a share);
//   3. resolves them in order with a conflict bit matrix (every CTA computes
//      a share of the rows and stores them into all CTAs; one warp runs the
//      greedy over it) and adds the kept ones to a position bitmap of the
//      kept moves,
//   4. filters the rest of its slice against the bitmap, compacting in
//      place, and histograms the survivors for the next threshold.
// Every CTA resolves each batch itself, so each holds the same bitmap; only
// the first writes the kept moves.  No batch member conflicts with a move
// kept by an earlier batch: step 4 removed those.  Every move decided in
// step 3 only depends on moves with smaller keys, all of them decided before,
// so the result is the sequential greedy's; the slicing changes only which
// SM streams which keys (the list is a set).  The kept moves go to the job's
// TOTAL output region of the neighbourhood, in order.  Cluster barriers order
// every exchange through distributed shared memory.
#include <cooperative_groups.h>

#include <cstdint>

#include "mlp_common.cuh"
#include "mlp_kernels.cuh"

namespace mlp {

namespace {

namespace cg = cooperative_groups;
constexpr int kTotCl = 8;  // most CTAs per neighbourhood list (portable cluster size)

constexpr unsigned kFull = 0xffffffffu;
constexpr int kTotThreads = 1024;
constexpr int kTotBatch = 256;     // keys resolved per batch
constexpr int kTotBins = 2048;     // histogram bins of the threshold search
constexpr int kCovWords = kMaxSize / 32 + 4;
enum : uint8_t { kNone = 0, kUndec = 1, kIn = 2, kOut = 3 };

// Keys loaded per thread per step of a pass over a list: independent loads
// in flight hide the L2 latency (a single CTA streams the whole list).
template <bool WIDE>
struct TK;
template <>
struct TK<false> {
  using K = uint64_t;
  static constexpr int U = 8;
  static __device__ __forceinline__ int64_t delta(K k) { return total_key32_delta(k); }
};
template <>
struct TK<true> {
  using K = u128;
  static constexpr int U = 4;
  static __device__ __forceinline__ int64_t delta(K k) { return total_key64_delta(k); }
};

__device__ __forceinline__ uint64_t shfl_xor_k(uint64_t v, int o) { return __shfl_xor_sync(kFull, v, o); }
__device__ __forceinline__ u128 shfl_xor_k(u128 v, int o) {
  const uint64_t lo = __shfl_xor_sync(kFull, (uint64_t)v, o);
  const uint64_t hi = __shfl_xor_sync(kFull, (uint64_t)(v >> 64), o);
  return ((u128)hi << 64) | lo;
}
__device__ __forceinline__ int bitlen(uint64_t v) { return v ? 64 - __clzll((long long)v) : 0; }
__device__ __forceinline__ int bitlen(u128 v) {
  const uint64_t hi = (uint64_t)(v >> 64);
  return hi ? 128 - __clzll((long long)hi) : bitlen((uint64_t)v);
}
template <typename K>
__device__ __forceinline__ K kmax_value() {
  return ~(K)0;
}

struct TotalSmem {
  static constexpr size_t bat = 0;                                         // K[kTotBatch]: gathered batch
  static constexpr size_t srt = bat + (size_t)kTotBatch * 16;              // K[kTotBatch]: the batch by rank
  static constexpr size_t hist = srt + (size_t)kTotBatch * 16;             // uint32[2][kTotBins]
  static constexpr size_t cov = hist + (size_t)2 * kTotBins * 4;           // uint32[kCovWords]
  static constexpr size_t pw = cov + (size_t)kCovWords * 4;                // int32[kCovWords]
  static constexpr size_t bits = pw + (size_t)kCovWords * 4;               // conflict rows
  static constexpr size_t ab = bits + (size_t)kTotBatch * kTotBatch / 8;   // uint32[kTotBatch]
  static constexpr size_t st = ab + (size_t)kTotBatch * 4;                 // uint8[kTotBatch]
  static constexpr size_t total = st + kTotBatch;
};

// Block-wide min and max of one key per thread (every thread gets both).
template <typename K>
__device__ void block_minmax(K& mn, K& mx, K* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const K a = shfl_xor_k(mn, o), b = shfl_xor_k(mx, o);
    mn = a < mn ? a : mn;
    mx = b > mx ? b : mx;
  }
  __syncthreads();  // red may still be read by a previous call
  if (lane == 0) {
    red[wid] = mn;
    red[32 + wid] = mx;
  }
  __syncthreads();
  mn = red[0];
  mx = red[32];
  for (int w = 1; w < nw; w++) {
    mn = red[w] < mn ? red[w] : mn;
    mx = red[32 + w] > mx ? red[32 + w] : mx;
  }
}

// Block-wide exclusive scan of one int per thread; `total` gets the sum.
__device__ int block_scan_int(int v, int* sm, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();  // sm may still be read by a previous call
  if (lane == 31) sm[wid] = x;
  __syncthreads();
  int s = lane < nw ? sm[lane] : 0;  // every warp scans the warp totals
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, s, o);
    if (lane >= o) s += y;
  }
  total = __shfl_sync(kFull, s, 31);
  const int before = wid > 0 ? __shfl_sync(kFull, s, wid - 1) : 0;
  return before + x - v;
}

// Exclusive scan of one value per warp (v equal on the warp's lanes).
__device__ int block_scan_warps(int v, int* sm, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();  // sm may still be read by a previous call
  if (lane == 0) sm[wid] = v;
  __syncthreads();
  int s = lane < nw ? sm[lane] : 0;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, s, o);
    if (lane >= o) s += y;
  }
  total = __shfl_sync(kFull, s, 31);
  return wid > 0 ? __shfl_sync(kFull, s, wid - 1) : 0;
}

__device__ __forceinline__ void hist_add(uint32_t* hist, int bin) {
  if (bin >= 0) atomicAdd(&hist[bin], 1u);
}

// Bin of key k in the histogram of [lo, lo + range] with bins of 2^sft
// (-1 outside).
template <typename K>
__device__ __forceinline__ int bin_of(K k, K lo, K range, int sft) {
  if (k < lo) return -1;
  const K off = k - lo;
  return off <= range ? (int)(uint32_t)(off >> sft) : -1;
}
__device__ __forceinline__ int bin_shift(int bl) { return bl > 11 ? bl - 11 : 0; }

// The move (i, j) of a key, and its conflict footprint ab: swap endpoints
// i | j << 16, else the closed conflict interval a | b << 16.
__device__ __forceinline__ uint32_t footprint_of(int nb, uint32_t low) {
  const int i = (int)((low >> 14) & 0x3fff), j = (int)(low & 0x3fff);
  if (nb == 0) return (uint32_t)i | ((uint32_t)j << 16);
  int a, b;
  conflict_interval(nb, i, j, a, b);
  return (uint32_t)a | ((uint32_t)b << 16);
}

// Conflicts with a move kept earlier: swap, an endpoint within one position
// of a kept endpoint (f_canSwapMerge); intervals, a kept interval meets it.
__device__ __forceinline__ bool killed(int nb, uint32_t ab, const uint32_t* cov, const int* pw) {
  const int a = (int)(ab & 0xffff), b = (int)(ab >> 16);
  if (nb == 0) {
    const int p = a - 1, q = b - 1;
    const uint64_t vp = (uint64_t)cov[p >> 5] | ((uint64_t)cov[(p >> 5) + 1] << 32);
    const uint64_t vq = (uint64_t)cov[q >> 5] | ((uint64_t)cov[(q >> 5) + 1] << 32);
    return ((vp >> (p & 31)) & 7u) | ((vq >> (q & 31)) & 7u);
  }
  const int wa = a >> 5, wb = b >> 5;
  const uint32_t ma = 0xffffffffu << (a & 31), mb = 0xffffffffu >> (31 - (b & 31));
  if (wa == wb) return (cov[wa] & ma & mb) != 0;
  if ((cov[wa] & ma) | (cov[wb] & mb)) return true;
  return pw[wb] - pw[wa + 1] > 0;
}

__device__ __forceinline__ bool conflict(int nb, uint32_t x, uint32_t y) {
  const int xa = (int)(x & 0xffff), xb = (int)(x >> 16), ya = (int)(y & 0xffff), yb = (int)(y >> 16);
  if (nb == 0) return !can_swap_same(xa, xb, ya, yb);
  return xa <= yb && ya <= xb;
}

// The batch in key order: srt[r] = the key with r smaller keys (keys are
// distinct: each encodes its move) and mab[r] its footprint.  This CTA ranks
// keys rank, rank + ncl, ... (a warp per key) and stores them into every CTA
// of the cluster.
template <bool WIDE>
__device__ void rank_share(cg::cluster_group& cluster, int nb, const typename TK<WIDE>::K* bat,
                           typename TK<WIDE>::K* srt, uint32_t* mab, int nbat, int rank, int ncl) {
  using K = typename TK<WIDE>::K;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int x = rank + ncl * wid; x < nbat; x += ncl * nw) {
    const K kx = bat[x];
    int c = 0;
    for (int y = lane; y < nbat; y += 32) c += bat[y] < kx ? 1 : 0;
    const int r = (int)__reduce_add_sync(kFull, (unsigned)c);
    if (lane < ncl) {
      *cluster.map_shared_rank(srt + r, lane) = kx;
      *cluster.map_shared_rank(mab + r, lane) = footprint_of(nb, (uint32_t)kx);
    }
  }
}

// Rows rank, rank + ncl, ... of the batch's conflict matrix (bit y of row x:
// y precedes x and the two conflict; only words 0 .. x/32 of row x exist),
// stored into every CTA of the cluster.  W = words per row.
__device__ void conflict_rows(cg::cluster_group& cluster, int nb, const uint32_t* mab, uint32_t* bits, int na, int W,
                              int rank, int ncl) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int x = rank + ncl * wid; x < na; x += ncl * nw) {
    const uint32_t fx = mab[x];
    const int nwx = (x >> 5) + 1;
    uint32_t word[kTotBatch / 32];
#pragma unroll
    for (int w = 0; w < kTotBatch / 32; w++) {
      word[w] = 0u;
      if (w < nwx) {
        const int y = 32 * w + lane;  // mab is read for y < x < na only
        word[w] = __ballot_sync(kFull, y < x && conflict(nb, mab[y], fx));
      }
    }
    if (lane < ncl) {
      uint32_t* dst = cluster.map_shared_rank(bits, lane) + x * W;
#pragma unroll
      for (int w = 0; w < kTotBatch / 32; w++)
        if (w < nwx) dst[w] = word[w];
    }
  }
}

// Greedy over the batch in key order, by one warp (every lane calls it):
// member x joins unless an earlier member that joined conflicts with it.
// The members are taken 32 at a time (lane l: member 32 b + l); the earlier
// blocks are decided, so a member conflicting with one of their kept members
// leaves at once, and the rest of the block is settled by rounds of ballots
// (a member joins once every earlier conflicting member of its block has
// left).  The kept masks of the blocks stay in registers.  On return mst[x]
// is kIn or kOut for every x < na.
__device__ void warp_greedy_sorted(const uint32_t* bits, int W, int na, volatile uint8_t* mst) {
  const int lane = threadIdx.x & 31;
  uint32_t in[kTotBatch / 32];
#pragma unroll
  for (int b = 0; b < kTotBatch / 32; b++) {
    in[b] = 0u;
    if (b < W) {
      const int x = 32 * b + lane;
      const bool valid = x < na;
      uint32_t ext = 0u, diag = 0u;
      if (valid) {
#pragma unroll
        for (int w = 0; w < b; w++) ext |= bits[x * W + w] & in[w];
        diag = bits[x * W + b];
      }
      uint8_t st = !valid ? kNone : (ext ? kOut : kUndec);
      uint32_t und = __ballot_sync(kFull, st == kUndec), inb = 0u;
      while (und) {  // every round settles at least the first undecided member
        if (st == kUndec) {
          if (diag & inb) st = kOut;
          else if (!(diag & und)) st = kIn;
        }
        inb = __ballot_sync(kFull, st == kIn);
        und = __ballot_sync(kFull, st == kUndec);
      }
      in[b] = inb;
      if (valid) mst[x] = st;
    }
  }
}

// Histogram of the keys of list[0, m) in [lo, lo + range], bins of 2^sft.
template <bool WIDE>
__device__ void slice_hist(const typename TK<WIDE>::K* list, int m, uint32_t* hist, typename TK<WIDE>::K lo,
                           typename TK<WIDE>::K range, int sft) {
  using K = typename TK<WIDE>::K;
  constexpr int U = TK<WIDE>::U;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int q = tid; q < kTotBins; q += nt) hist[q] = 0;
  __syncthreads();
  for (int x0 = 0; x0 < m; x0 += U * nt) {
    K kv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int x = x0 + u * nt + tid;
      kv[u] = x < m ? list[x] : kmax_value<K>();
    }
#pragma unroll
    for (int u = 0; u < U; u++) hist_add(hist, x0 + u * nt + tid < m ? bin_of(kv[u], lo, range, sft) : -1);
  }
}

// Launched with clusters of 1 .. kTotCl CTAs along x (a cluster per
// neighbourhood and job); blockIdx.y is the job.
template <bool WIDE>
__global__ void __launch_bounds__(kTotThreads) k_total_select(const JobDev* __restrict__ jobs) {
  using K = typename TK<WIDE>::K;
  extern __shared__ __align__(16) uint8_t tsm[];
  __shared__ K s_red[64];
  __shared__ K s_qlo[kTotCl], s_qhi[kTotCl];  // each CTA's bounds, stored by that CTA
  __shared__ int s_qm[kTotCl];                // keys left in each CTA's slice, stored by that CTA
  __shared__ int s_scan[32];
  __shared__ int s_g, s_nbat, s_nb;
  pdl_launch_dependents();  // the TOTAL finish waits for this kernel's end
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank(), ncl = (int)cluster.num_blocks();
  const bool first = rank == 0;
  const int nb = blockIdx.x / ncl;
  const JobDev* J = jobs + blockIdx.y;
  // Exits before the first barrier are taken by the whole cluster (same job
  // and neighbourhood).
  {
    const int64_t* stt = J->stats;
    if (stt[kStatConverged] || stt[kStatSweeps] >= stt[kStatLimit]) return;
  }
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
  const int sz = J->size;
  if (!((J->nb_mask >> nb) & 1)) {
    if (first && tid == 0) J->tkcount[nb] = 0;
    return;
  }
  pdl_wait();  // the collecting sweep's lists
  const int mall = J->tcount[nb];
  if (mall > total_list_cap(nb, sz)) {
    if (first && tid == 0) {
      J->stats[kStatError] = 4;
      J->tkcount[nb] = 0;
    }
    return;
  }
  // This CTA's slice of the list.
  const int slice = (mall + ncl - 1) / ncl;
  const int s0 = min(mall, rank * slice);
  int m = min(mall, s0 + slice) - s0;
  K* list = (K*)J->tlist + total_list_off(nb, sz) + s0;
  K* bat = (K*)(tsm + TotalSmem::bat);
  K* srt = (K*)(tsm + TotalSmem::srt);
  uint32_t* hist = (uint32_t*)(tsm + TotalSmem::hist);
  uint32_t* cov = (uint32_t*)(tsm + TotalSmem::cov);
  int* pw = (int*)(tsm + TotalSmem::pw);
  uint32_t* bits = (uint32_t*)(tsm + TotalSmem::bits);
  uint32_t* mab = (uint32_t*)(tsm + TotalSmem::ab);
  volatile uint8_t* mst = (volatile uint8_t*)(tsm + TotalSmem::st);
  int* l_nbat = cluster.map_shared_rank(&s_nbat, 0);
  const int nwords = (sz >> 5) + 2;  // bitmap words read for positions 0 .. sz
  for (int w = tid; w < kCovWords; w += nt) {
    cov[w] = 0;
    pw[w] = 0;
  }
  if (tid == 0) s_nbat = 0;
  const int kbase = region_off(nb, sz), kcap = region_cap(nb, sz);
  int nk = 0;
  constexpr int U = TK<WIDE>::U;
  {
    K lo = kmax_value<K>(), hi = 0;
    for (int x0 = 0; x0 < m; x0 += U * nt) {
      K kv[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int x = x0 + u * nt + tid;
        kv[u] = x < m ? list[x] : kmax_value<K>();
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int x = x0 + u * nt + tid;
        if (x < m) {
          lo = kv[u] < lo ? kv[u] : lo;
          hi = kv[u] > hi ? kv[u] : hi;
        }
      }
    }
    block_minmax(lo, hi, s_red);
    if (tid < ncl) {
      *cluster.map_shared_rank(&s_qlo[rank], tid) = lo;
      *cluster.map_shared_rank(&s_qhi[rank], tid) = hi;
      *cluster.map_shared_rank(&s_qm[rank], tid) = m;
    }
  }
  cluster.sync();
  // Bounds of the whole list (a CTA with an empty slice reports none).
  K lo = kmax_value<K>(), hi = 0;
  int mtot = 0;
  for (int q = 0; q < ncl; q++) {
    if (s_qm[q] == 0) continue;
    mtot += s_qm[q];
    lo = s_qlo[q] < lo ? s_qlo[q] : lo;
    hi = s_qhi[q] > hi ? s_qhi[q] : hi;
  }
  K range = hi - lo;
  int sft = bin_shift(bitlen(range));
  // Histograms alternate between two buffers: a CTA fills one while the
  // others may still read the previous one.
  int hb = 0;
  if (mtot > kTotBatch) slice_hist<WIDE>(list, m, hist, lo, range, sft);

  for (int round = 0;; round++) {
    // Every slice count and first-level histogram is complete.
    cluster.sync();
    mtot = 0;
    for (int q = 0; q < ncl; q++) mtot += s_qm[q];
    if (mtot == 0) break;
    if (round > (1 << 24)) {  // unreachable: every round removes at least the smallest key
      if (first && tid == 0) J->stats[kStatError] = 5;
      break;
    }
    // ---- 1. threshold: at most kTotBatch keys <= T ----
    K T = hi;
    if (mtot > kTotBatch) {
      // Take the lowest bins that fit the budget; while less than half of
      // the batch is filled, refine into the first bin that did not fit.
      int budget = kTotBatch;
      bool have_t = false;
      for (int lvl = 0; lvl < 16; lvl++) {
        if (lvl > 0) {
          hb ^= 1;
          slice_hist<WIDE>(list, m, hist + hb * kTotBins, lo, range, sft);
          cluster.sync();  // every CTA's histogram of this level is complete
        }
        // The list's histogram: every CTA adds the same histograms.
        int h0 = 0, h1 = 0;
#pragma unroll
        for (int q = 0; q < kTotCl; q++) {
          if (q < ncl) {
            const uint2 v = *reinterpret_cast<const uint2*>(cluster.map_shared_rank(hist + hb * kTotBins, q) + 2 * tid);
            h0 += (int)v.x;
            h1 += (int)v.y;
          }
        }
        if (tid == 0) s_g = -1;
        __syncthreads();
        int tot;
        const int e = block_scan_int(h0 + h1, s_scan, tot);
        // (last bin that fits) << 20 | (keys up to it): both grow together
        int packed = -1;
        if (e + h0 <= budget) packed = ((2 * tid) << 20) | (e + h0);
        if (e + h0 + h1 <= budget) packed = ((2 * tid + 1) << 20) | (e + h0 + h1);
        if (packed >= 0) atomicMax(&s_g, packed);
        __syncthreads();
        const int pk = s_g;
        const int gg = pk >= 0 ? pk >> 20 : -1;
        if (gg >= 0) {
          T = lo + ((K)(gg + 1) << sft) - 1;
          have_t = true;
          budget -= pk & 0xfffff;
        }
        if (gg == kTotBins - 1 || sft == 0 || budget < kTotBatch / 2) break;
        lo = lo + ((K)(gg + 1) << sft);  // the first bin that did not fit
        range = ((K)1 << sft) - 1;
        sft = bin_shift(bitlen(range));
      }
      if (!have_t) T = hi;  // unreachable: single-key bins always fit
    }
    // ---- 2. the keys <= T go to every CTA (slots counted by the first) ----
    for (int x0 = 0; x0 < m; x0 += U * nt) {
      K kv[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int x = x0 + u * nt + tid;
        kv[u] = x < m ? list[x] : kmax_value<K>();
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const bool g = x0 + u * nt + tid < m && kv[u] <= T;
        const unsigned bal = __ballot_sync(kFull, g);
        if (bal) {
          const int src = __ffs(bal) - 1;
          int base = 0;
          if (lane == src) base = atomicAdd(l_nbat, __popc(bal));
          base = __shfl_sync(kFull, base, src);
          const int q = base + __popc(bal & ((1u << lane) - 1u));
          if (g && q < kTotBatch)
            for (int c = 0; c < ncl; c++) *cluster.map_shared_rank(bat + q, c) = kv[u];
        }
      }
    }
    cluster.sync();  // the batch is complete
    if (tid == 0) {
      const int nbat = *l_nbat;
      if (nbat > kTotBatch && first) J->stats[kStatError] = 5;  // unreachable by the threshold's construction
      s_nb = nbat < kTotBatch ? nbat : kTotBatch;
    }
    __syncthreads();
    const int na = s_nb;
    const int W = (na + 31) >> 5;
    // ---- 3. resolve the batch in key order ----
    rank_share<WIDE>(cluster, nb, bat, srt, mab, na, rank, ncl);
    cluster.sync();  // every CTA holds the batch in key order
    if (first && tid == 0) s_nbat = 0;  // every read of it precedes the barrier
    conflict_rows(cluster, nb, mab, bits, na, W, rank, ncl);
    cluster.sync();  // every CTA holds the whole conflict matrix
    if (tid < 32) warp_greedy_sorted(bits, W, na, mst);
    __syncthreads();
    // Kept members, in key order, to the output region.
    const bool kin = tid < na && mst[tid] == kIn;
    int nin;
    const int krank = block_scan_int(kin ? 1 : 0, s_scan, nin);
    if (first && kin) {
      const int o = nk + krank;
      if (o < kcap) {
        const K k = srt[tid];
        const uint32_t low = (uint32_t)k;
        J->tkcost[kbase + o] = TK<WIDE>::delta(k);
        J->tkij[kbase + o] = ((low >> 14) & 0x3fff) | ((low & 0x3fff) << 16);
      }
    }
    nk += nin;
    // Add the kept footprints to the bitmap.
    if (nb == 0) {
      if (kin) {
        const int i = (int)(mab[tid] & 0xffff), j = (int)(mab[tid] >> 16);
        atomicOr(&cov[i >> 5], 1u << (i & 31));
        atomicOr(&cov[j >> 5], 1u << (j & 31));
      }
    } else {
      const int wid = tid >> 5, nw = nt >> 5;
      for (int x = wid; x < na; x += nw) {
        if (mst[x] != kIn) continue;
        const int a = (int)(mab[x] & 0xffff), b = (int)(mab[x] >> 16);
        for (int w = (a >> 5) + lane; w <= (b >> 5); w += 32) {
          uint32_t msk = 0xffffffffu;
          if (w == (a >> 5)) msk &= 0xffffffffu << (a & 31);
          if (w == (b >> 5)) msk &= 0xffffffffu >> (31 - (b & 31));
          atomicOr(&cov[w], msk);
        }
      }
      __syncthreads();
      int tw;
      const int cw = tid < nwords ? __popc(cov[tid]) : 0;
      const int ew = block_scan_int(cw, s_scan, tw);
      if (tid < nwords + 1) pw[tid] = ew;
    }
    // ---- 4. filter the rest of the slice, compacting in place, and
    // histogram the survivors over the next round's first level ----
    lo = T + 1;
    range = hi - lo;
    sft = bin_shift(bitlen(range));
    hb ^= 1;
    uint32_t* nh = hist + hb * kTotBins;
    for (int q = tid; q < kTotBins; q += nt) nh[q] = 0;
    __syncthreads();
    // Each step u of a warp stores its survivors contiguously (ballot
    // ranks) after the warp's offset (one scan over the warps' totals).
    int base = 0;
    for (int x0 = 0; x0 < m; x0 += U * nt) {
      K kv[U];
      unsigned bal[U];
      int cnt = 0;
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int x = x0 + u * nt + tid;
        kv[u] = x < m ? list[x] : kmax_value<K>();
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int x = x0 + u * nt + tid;
        const bool keep = x < m && kv[u] > T && !killed(nb, footprint_of(nb, (uint32_t)kv[u]), cov, pw);
        bal[u] = __ballot_sync(kFull, keep);
        cnt += __popc(bal[u]);
        if (keep) hist_add(nh, bin_of(kv[u], lo, range, sft));
      }
      int tot;
      int o = base + block_scan_warps(cnt, s_scan, tot);  // all loads of the chunk precede its stores
      const unsigned below = (1u << lane) - 1u;
#pragma unroll
      for (int u = 0; u < U; u++) {
        if ((bal[u] >> lane) & 1u) list[o + __popc(bal[u] & below)] = kv[u];
        o += __popc(bal[u]);
      }
      base += tot;
    }
    m = base;
    if (tid < ncl) *cluster.map_shared_rank(&s_qm[rank], tid) = m;
  }
  if (first && tid == 0) {
    J->tkcount[nb] = nk < kcap ? nk : kcap;
    if (nk > kcap) J->stats[kStatError] = 3;
  }
  // After the last barrier no CTA reads or writes another's shared memory.
}

}  // namespace

cudaError_t configure_total() {
  cudaError_t e = cudaFuncSetAttribute(k_total_select<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)TotalSmem::total);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_total_select<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)TotalSmem::total);
}

cudaError_t launch_total_select(const JobDev* jobs, int njobs, bool wide, cudaStream_t s) {
  if (njobs <= 0) return cudaSuccess;
  // Clusters as wide as about two waves of CTAs allow: a single search
  // streams its lists with kTotCl SMs each, a large batch one SM per list.
  // (SM count queried once; without it, clusters of one CTA.)
  static const int sms = [] {
    int dev = 0, c = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return 0;
    return c;
  }();
  int ncl = kTotCl;
  while (ncl > 1 && (int64_t)njobs * kNumNb * ncl > 2 * (int64_t)sms) ncl >>= 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kNumNb * ncl, njobs);
  cfg.blockDim = dim3(kTotThreads);
  cfg.dynamicSmemBytes = TotalSmem::total;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ncl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  // Programmatic stream serialization (see launch_pdl) on a created stream.
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = s != 0 ? 2 : 1;
  if (wide) return cudaLaunchKernelEx(&cfg, k_total_select<true>, jobs);
  return cudaLaunchKernelEx(&cfg, k_total_select<false>, jobs);
}

}  // namespace mlp
