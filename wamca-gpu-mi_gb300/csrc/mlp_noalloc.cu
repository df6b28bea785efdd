// mlp_noalloc.cu -- neighbourhood evaluation that allocates no memory.
//
// Some callers cannot allocate device memory: code that runs inside another
// framework's memory pool or budget, a service whose device memory is carved
// up ahead of time, or a host that must not call cudaMalloc/cudaFree at all
// (they synchronise the device and so stall everything else running on it).
// mlp_eval_noalloc() serves them: the caller passes the distance matrix, the
// tour and the three output arrays, all in device memory, and every
// intermediate array (adjacent weights, prefix sums, candidate keys, the job
// descriptor and the sweep tile list) lives in one file-scope __device__ array
// of fixed size that the library holds on every GPU it is loaded on until the
// process exits.
//
// Limits and sharing: tours of at most kNoAllocMaxSize positions
// (n <= 2047); the scratch array is shared by every call in the process and
// keeps the last call's contents, so calls that overlap on the GPU (on
// different streams, or from different threads) race and must be serialised
// by the caller.
//
// Inputs: the tour is checked on the device before any distance is read
// through it (depot 0 at both ends, every client 1..n-1 exactly once).  A tour
// that fails is replaced by a harmless one for the kernels and every output
// entry becomes (cost INT64_MIN, i = j = -1).  Distances are only ever used as
// values, never as addresses; they must be symmetric and in [0, 65535] for the
// candidates to mean anything.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/mlp_gpu.h"
#include "mlp_common.cuh"
#include "mlp_engine.h"
#include "mlp_kernels.cuh"

namespace mlp {
namespace {

constexpr int kNoAllocMaxSize = 2048;
constexpr int kNoAllocShape = 5;  // 64 diagonals x 16 rows
constexpr int kNaTL = 64, kNaTR = 16;
static_assert(kTileShapes[kNoAllocShape].tl == kNaTL && kTileShapes[kNoAllocShape].tr == kNaTR,
              "tile shape of the no-allocation sweep");
constexpr size_t kNoAllocBytes = 256 * 1024;
constexpr int kMaxDevices = 64;

// Scratch of every call, on every device that loads the library.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

struct Layout {
  size_t job, stats, bad, safe, tiles, w, W, Q, A, keys, end;
  int ntiles;
  __host__ __device__ static size_t al(size_t v) { return (v + 255) / 256 * 256; }
  __host__ __device__ explicit Layout(int size) {
    const size_t pad = (size_t)size + 8;
    ntiles = sweep_tiles(size, kNaTL, kNaTR);
    job = 0;
    stats = al(job + sizeof(JobDev));
    bad = al(stats + sizeof(int64_t) * kStatWords);
    safe = al(bad + sizeof(int32_t));
    tiles = al(safe + sizeof(int32_t) * (size_t)size);
    w = al(tiles + sizeof(SweepTile) * (size_t)ntiles);
    W = al(w + 4 * pad);
    Q = al(W + 8 * pad);
    A = al(Q + 8 * pad);
    keys = al(A + 4 * 3 * pad);
    end = al(keys + 8 * (size_t)total_blocks(size));
  }
};

// Checks the tour and writes the job descriptor and the sweep tile list into
// the scratch array.  One CTA of kSetupThreads threads: thread rb places the
// tiles of row block rb (prefix over the row blocks before it).  The tour
// check marks each client in a shared bitmap; a tour that fails points the
// descriptor at an identity tour in the scratch array instead, so that no
// later kernel indexes the distances with an entry of the caller's tour.
constexpr int kSetupThreads = 256;
static_assert((kNoAllocMaxSize - 3 + kNaTR - 1) / kNaTR <= kSetupThreads, "one setup thread per row block");
__global__ void __launch_bounds__(kSetupThreads) k_noalloc_setup(unsigned char* base, const int32_t* D,
                                                                 const int32_t* tour, int n, int size, int nb,
                                                                 int wide) {
  __shared__ int s_cnt[kSetupThreads];
  __shared__ uint32_t s_seen[kNoAllocMaxSize / 32];
  __shared__ int s_bad;
  const Layout lay(size);
  const int tid = threadIdx.x;
  for (int q = tid; q < kNoAllocMaxSize / 32; q += blockDim.x) s_seen[q] = 0;
  if (tid == 0) s_bad = 0;
  __syncthreads();
  int bad = 0;
  for (int p = tid; p < size; p += blockDim.x) {
    const int32_t v = tour[p];
    if (p == 0 || p == size - 1) {
      bad |= v != 0;
    } else if (v < 1 || v >= n) {
      bad = 1;
    } else {
      const uint32_t bit = 1u << (v & 31);
      bad |= (atomicOr(&s_seen[v >> 5], bit) & bit) != 0;  // client seen before
    }
  }
  if (bad) s_bad = 1;
  const int rows = sweep_row_blocks(size, kNaTR);
  const int cnt = tid < rows ? sweep_row_tiles(size, 1 + tid * kNaTR, kNaTL) : 0;
  s_cnt[tid] = cnt;
  __syncthreads();
  const bool ok = s_bad == 0;  // (n - 1 distinct clients in [1, n) and two depots: a permutation)
  int32_t* safe = (int32_t*)(base + lay.safe);
  if (!ok)
    for (int p = tid; p < size; p += blockDim.x) safe[p] = p < size - 1 ? p : 0;
  int off = 0;
  for (int q = 0; q < tid; q++) off += s_cnt[q];
  SweepTile* tiles = (SweepTile*)(base + lay.tiles);
  for (int c = 0; c < cnt; c++) tiles[off + c] = SweepTile{0, 1 + tid * kNaTR, 1 + c * kNaTL, 0};
  if (tid == 0) {
    *(int32_t*)(base + lay.bad) = ok ? 0 : 1;
    JobDev J{};
    J.D = D;
    J.tour = ok ? const_cast<int32_t*>(tour) : safe;
    J.tour_alt = nullptr;
    J.w = (int32_t*)(base + lay.w);
    J.W = base + lay.W;
    J.Q = base + lay.Q;
    J.A = (int32_t*)(base + lay.A);
    J.keys = (uint64_t*)(base + lay.keys);
    J.kept = nullptr;
    J.kept_count = nullptr;
    J.ws = nullptr;
    J.stats = (int64_t*)(base + lay.stats);
    J.moves_out = nullptr;
    J.moves_cost = nullptr;
    J.moves_cap = 0;
    J.n = n;
    J.size = size;
    J.nb_mask = 1 << nb;
    J.flags = wide ? kFlagWide : 0;
    *(JobDev*)(base + lay.job) = J;
  }
}

// Per-block candidates of one neighbourhood from the candidate keys.
__global__ void k_noalloc_decode(const unsigned char* base, int size, int nb, int wide, int64_t* cost,
                                 int32_t* oi, int32_t* oj) {
  const Layout lay(size);
  const uint64_t* keys = (const uint64_t*)(base + lay.keys) + nb_offset(nb, size);
  const bool bad = *(const int32_t*)(base + lay.bad) != 0;
  const int m = nb_blocks(nb, size);
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < m; b += gridDim.x * blockDim.x) {
    if (bad) {  // the caller's tour failed the check
      cost[b] = INT64_MIN;
      oi[b] = oj[b] = -1;
      continue;
    }
    const uint64_t k = keys[b];
    if (k == kKeyNone) {
      cost[b] = wide ? INT64_MAX : (int64_t)kCostInfty32;
      oi[b] = oj[b] = 0;
      continue;
    }
    int i, j;
    map_move(nb, size, b, (int)(k & ((1u << kCtxBits) - 1)), i, j);
    cost[b] = key_cost(k, kCtxBits);
    oi[b] = i;
    oj[b] = j;
  }
}

std::mutex g_mu;
unsigned char* g_base[kMaxDevices] = {};  // device address of the scratch array, per device

}  // namespace
}  // namespace mlp

using namespace mlp;

extern "C" MLP_API int mlp_eval_noalloc(const int32_t* dist_dev, int32_t n, const int32_t* tour_dev, int32_t nb,
                                        int32_t wide, int64_t* cost_dev, int32_t* i_dev, int32_t* j_dev,
                                        void* stream) {
  if (!dist_dev || !tour_dev || !cost_dev || !i_dev || !j_dev) {
    set_error("mlp_eval_noalloc: null pointer argument");
    return kErrArg;
  }
  if (nb < 0 || nb >= kNumNb) {
    set_error("mlp_eval_noalloc: neighbourhood out of range");
    return kErrArg;
  }
  const int size = n + 1;
  if (n < 5 || size > kNoAllocMaxSize) {
    set_error("mlp_eval_noalloc: needs 5 <= n and n + 1 <= 2048 (the fixed scratch array's capacity)");
    return kErrRange;
  }
  if (Layout(size).end > kNoAllocBytes) {
    set_error("mlp_eval_noalloc: instance does not fit the fixed scratch array");
    return kErrRange;
  }
  int dev = 0;
  int st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
  if (st != kOk) return st;
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("mlp_eval_noalloc: device ordinal out of range");
    return kErrRange;
  }
  unsigned char* base = nullptr;
  {
    // One-time set-up per device, with that device current: the host cannot
    // use the array's name as a device address, so look the address up.
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_base[dev]) {
      void* p = nullptr;
      st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
      if (st != kOk) return st;
      st = cuda_status(configure_prepare(), "configure prepare kernel");
      if (st != kOk) return st;
      g_base[dev] = static_cast<unsigned char*>(p);
    }
    base = g_base[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const Layout lay(size);
  // Tour check, job descriptor and tile list, then the ADS prefix arrays
  // (which also reset the candidate keys), then one sweep of neighbourhood
  // nb, then decoding.
  k_noalloc_setup<<<1, kSetupThreads, 0, s>>>(base, dist_dev, tour_dev, n, size, nb, wide ? 1 : 0);
  st = cuda_status(cudaGetLastError(), "noalloc setup kernel");
  if (st != kOk) return st;
  const JobDev* job = reinterpret_cast<const JobDev*>(base + lay.job);
  st = cuda_status(launch_stats_begin(job, 1, 1, s), "stats kernel");
  if (st != kOk) return st;
  st = cuda_status(launch_prepare(job, 1, wide != 0, false, s), "prepare kernel");
  if (st != kOk) return st;
  st = cuda_status(launch_sweep(reinterpret_cast<const SweepTile*>(base + lay.tiles), lay.ntiles, job, wide != 0,
                                kNoAllocShape, false, s),
                   "sweep kernel");
  if (st != kOk) return st;
  const int m = nb_blocks(nb, size);
  k_noalloc_decode<<<(m + 255) / 256, 256, 0, s>>>(base, size, nb, wide ? 1 : 0, cost_dev, i_dev, j_dev);
  return cuda_status(cudaGetLastError(), "noalloc decode kernel");
}
