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
// k_total_select: one CTA per (neighbourhood, job).  Its input is the list of
// improving moves the collecting sweep appended (unordered, up to ~n^2/2
// keys).  It never sorts the whole list: it repeatedly
//   1. finds a threshold T with at most kTotBatch keys <= T (histogram of
//      the keys' offsets from the smallest, refined into the lowest bin when
//      that bin alone is too full),
//   2. gathers those keys (the smallest of the list) and sorts them in shared
//      memory,
//   3. drops the ones that conflict with a move kept by earlier batches (a
//      position bitmap of the kept moves), resolves the rest in order with a
//      conflict bit matrix (lexicographically-first maximal independent set,
//      as in the stage-3 merge) and adds the kept ones to the bitmap,
//   4. filters the rest of the list against the bitmap, compacting in place.
// Every move decided in step 3 only depends on moves with smaller keys, all
// of them decided before, so the result is the sequential greedy's.  The kept
// moves go to the job's TOTAL output region of the neighbourhood, in order.
#include <cstdint>

#include "mlp_common.cuh"
#include "mlp_kernels.cuh"

namespace mlp {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kTotThreads = 1024;
constexpr int kTotBatch = 512;     // keys resolved per batch
constexpr int kTotBins = 2048;     // histogram bins of the threshold search
constexpr int kCovWords = kMaxSize / 32 + 4;
enum : uint8_t { kNone = 0, kUndec = 1, kIn = 2, kOut = 3 };

template <bool WIDE>
struct TK;
template <>
struct TK<false> {
  using K = uint64_t;
  static __device__ __forceinline__ int64_t delta(K k) { return total_key32_delta(k); }
};
template <>
struct TK<true> {
  using K = u128;
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
  static constexpr size_t bat = 0;                                         // K[kTotBatch]
  static constexpr size_t hist = bat + (size_t)kTotBatch * 16;             // uint32[kTotBins]
  static constexpr size_t cov = hist + (size_t)kTotBins * 4;               // uint32[kCovWords]
  static constexpr size_t pw = cov + (size_t)kCovWords * 4;                // int32[kCovWords]
  static constexpr size_t bits = pw + (size_t)kCovWords * 4;               // conflict rows
  static constexpr size_t ab = bits + (size_t)kTotBatch * kTotBatch / 8;   // uint32[kTotBatch]
  static constexpr size_t idx = ab + (size_t)kTotBatch * 4;                // int32[kTotBatch]
  static constexpr size_t st = idx + (size_t)kTotBatch * 4;                // uint8[kTotBatch]
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
  int before = 0;
  total = 0;
  for (int w = 0; w < nw; w++) {
    const int s = sm[w];
    if (w < wid) before += s;
    total += s;
  }
  return before + x - v;
}

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

template <bool WIDE>
__global__ void __launch_bounds__(kTotThreads) k_total_select(const JobDev* __restrict__ jobs) {
  using K = typename TK<WIDE>::K;
  extern __shared__ __align__(16) uint8_t tsm[];
  __shared__ K s_red[64];
  __shared__ int s_scan[32];
  __shared__ int s_g, s_nbat;
  __shared__ uint32_t s_in[kTotBatch / 32], s_und[kTotBatch / 32];
  const int nb = blockIdx.x;
  const JobDev* J = jobs + blockIdx.y;
  {
    const int64_t* stt = J->stats;
    if (stt[kStatConverged] || stt[kStatSweeps] >= stt[kStatLimit]) return;
  }
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  const int sz = J->size;
  if (!((J->nb_mask >> nb) & 1)) {
    if (tid == 0) J->tkcount[nb] = 0;
    return;
  }
  int m = J->tcount[nb];
  if (m > total_list_cap(nb, sz)) {
    if (tid == 0) {
      J->stats[kStatError] = 4;
      J->tkcount[nb] = 0;
    }
    return;
  }
  K* list = (K*)J->tlist + total_list_off(nb, sz);
  K* bat = (K*)(tsm + TotalSmem::bat);
  uint32_t* hist = (uint32_t*)(tsm + TotalSmem::hist);
  uint32_t* cov = (uint32_t*)(tsm + TotalSmem::cov);
  int* pw = (int*)(tsm + TotalSmem::pw);
  uint32_t* bits = (uint32_t*)(tsm + TotalSmem::bits);
  uint32_t* mab = (uint32_t*)(tsm + TotalSmem::ab);
  int* midx = (int*)(tsm + TotalSmem::idx);
  volatile uint8_t* mst = (volatile uint8_t*)(tsm + TotalSmem::st);
  const int nwords = (sz >> 5) + 2;  // bitmap words read for positions 0 .. sz
  for (int w = tid; w < kCovWords; w += nt) {
    cov[w] = 0;
    pw[w] = 0;
  }
  const int kbase = region_off(nb, sz), kcap = region_cap(nb, sz);
  int nk = 0;
  K kmin = kmax_value<K>(), kmax = 0;
  for (int x = tid; x < m; x += nt) {
    const K k = list[x];
    kmin = k < kmin ? k : kmin;
    kmax = k > kmax ? k : kmax;
  }
  block_minmax(kmin, kmax, s_red);

  for (int round = 0; m > 0; round++) {
    if (round > (1 << 24)) {  // unreachable: every round removes at least the smallest key
      if (tid == 0) J->stats[kStatError] = 5;
      break;
    }
    // ---- 1. threshold: at most kTotBatch keys <= T ----
    K T = kmax;
    if (m > kTotBatch) {
      K range = kmax - kmin;
      for (int lvl = 0; lvl < 16; lvl++) {
        const int bl = bitlen(range);
        const int sft = bl > 11 ? bl - 11 : 0;
        for (int q = tid; q < kTotBins; q += nt) hist[q] = 0;
        __syncthreads();
        for (int x = tid; x < m; x += nt) {
          const K off = list[x] - kmin;
          if (off <= range) atomicAdd(&hist[(uint32_t)(off >> sft)], 1u);
        }
        if (tid == 0) s_g = -1;
        __syncthreads();
        const int h0 = (int)hist[2 * tid], h1 = (int)hist[2 * tid + 1];
        int tot;
        const int e = block_scan_int(h0 + h1, s_scan, tot);
        int g = -1;
        if (e + h0 <= kTotBatch) g = 2 * tid;
        if (e + h0 + h1 <= kTotBatch) g = 2 * tid + 1;
        if (g >= 0) atomicMax(&s_g, g);
        __syncthreads();
        const int gg = s_g;
        if (gg >= 0) {
          T = kmin + ((K)(gg + 1) << sft) - 1;
          break;
        }
        range = ((K)1 << sft) - 1;  // sft > 0: keys are distinct, a one-key bin never overflows
      }
    }
    // ---- 2. gather the keys <= T and sort them ----
    if (tid == 0) s_nbat = 0;
    __syncthreads();
    for (int x = tid; x < m; x += nt) {
      const K k = list[x];
      if (k <= T) {
        const int q = atomicAdd(&s_nbat, 1);
        if (q < kTotBatch) bat[q] = k;
      }
    }
    __syncthreads();
    int nbat = s_nbat;
    if (nbat > kTotBatch) {  // unreachable by the threshold's construction
      if (tid == 0) J->stats[kStatError] = 5;
      nbat = kTotBatch;
    }
    int P = 1;
    while (P < nbat) P <<= 1;
    for (int q = nbat + tid; q < P; q += nt) bat[q] = kmax_value<K>();
    __syncthreads();
    for (int k2 = 2; k2 <= P; k2 <<= 1) {
      for (int j2 = k2 >> 1; j2 > 0; j2 >>= 1) {
        if (tid < P) {
          const int o = tid ^ j2;
          if (o > tid) {
            const K a = bat[tid], b = bat[o];
            const bool up = (tid & k2) == 0;
            if ((a > b) == up) {
              bat[tid] = b;
              bat[o] = a;
            }
          }
        }
        __syncthreads();
      }
    }
    // ---- 3. resolve the batch in order ----
    // Members not killed by earlier batches, compacted in key order.
    bool alive = false;
    uint32_t fab = 0;
    if (tid < nbat) {
      fab = footprint_of(nb, (uint32_t)bat[tid]);
      alive = !killed(nb, fab, cov, pw);
    }
    int na;
    const int pos = block_scan_int(alive ? 1 : 0, s_scan, na);
    if (alive) {
      mab[pos] = fab;
      midx[pos] = tid;
      mst[pos] = kUndec;
    }
    __syncthreads();
    if (na > 0) {
      const int W = (na + 31) >> 5;
      // bit y of row x <=> y precedes x and the two conflict
      for (int x = wid; x < na; x += nw) {
        const uint32_t fx = mab[x];
        for (int w = 0; w < W; w++) {
          const int y = 32 * w + lane;
          const bool c = y < x && conflict(nb, mab[y], fx);
          const uint32_t word = __ballot_sync(kFull, c);
          if (lane == 0) bits[x * W + w] = word;
        }
      }
      for (int w = tid; w < W; w += nt) {
        s_in[w] = 0;
        const int rem = na - 32 * w;
        s_und[w] = rem >= 32 ? 0xffffffffu : ((1u << rem) - 1u);
      }
      __syncthreads();
      for (int r = 0; r <= na; r++) {
        int any = 0;
        for (int x = tid; x < na; x += nt) {
          if (mst[x] != kUndec) continue;
          uint32_t hin = 0, hund = 0;
          for (int w = 0; w < W; w++) {
            const uint32_t row = bits[x * W + w];
            hin |= row & s_in[w];
            hund |= row & s_und[w];
          }
          if (hin) mst[x] = kOut;
          else if (!hund) mst[x] = kIn;
          else any = 1;
        }
        __syncthreads();
        for (int w = wid; w < W; w += nw) {
          const int x = 32 * w + lane;
          const uint8_t sx = x < na ? mst[x] : kNone;
          const uint32_t bi = __ballot_sync(kFull, sx == kIn), bu = __ballot_sync(kFull, sx == kUndec);
          if (lane == 0) {
            s_in[w] = bi;
            s_und[w] = bu;
          }
        }
        if (!__syncthreads_or(any)) break;
      }
      // Kept members, in key order, to the output region.
      const bool kin = tid < na && mst[tid] == kIn;
      int nin;
      const int rank = block_scan_int(kin ? 1 : 0, s_scan, nin);
      if (kin) {
        const int o = nk + rank;
        if (o < kcap) {
          const K k = bat[midx[tid]];
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
      __syncthreads();
    }
    // ---- 4. filter the rest, compacting in place ----
    K nmin = kmax_value<K>(), nmax = 0;
    int base = 0;
    constexpr int U = 4;
    for (int x0 = 0; x0 < m; x0 += U * nt) {
      K kv[U];
      bool keep[U];
      int cnt = 0;
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int x = x0 + u * nt + tid;
        keep[u] = false;
        if (x < m) {
          kv[u] = list[x];
          keep[u] = kv[u] > T && !killed(nb, footprint_of(nb, (uint32_t)kv[u]), cov, pw);
        }
        cnt += keep[u];
      }
      int tot;
      int o = base + block_scan_int(cnt, s_scan, tot);  // all loads of the chunk precede its stores
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (!keep[u]) continue;
        list[o++] = kv[u];
        nmin = kv[u] < nmin ? kv[u] : nmin;
        nmax = kv[u] > nmax ? kv[u] : nmax;
      }
      base += tot;
    }
    m = base;
    kmin = nmin;
    kmax = nmax;
    block_minmax(kmin, kmax, s_red);
  }
  if (tid == 0) {
    J->tkcount[nb] = nk < kcap ? nk : kcap;
    if (nk > kcap) J->stats[kStatError] = 3;
  }
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
  const dim3 grid(kNumNb, njobs);
  if (wide) k_total_select<true><<<grid, kTotThreads, TotalSmem::total, s>>>(jobs);
  else k_total_select<false><<<grid, kTotThreads, TotalSmem::total, s>>>(jobs);
  return cudaGetLastError();
}

}  // namespace mlp
