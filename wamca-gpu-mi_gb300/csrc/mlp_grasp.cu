// mlp_grasp.cu -- multi-start constructor on the device (sm_103a).
//
// MLSolution::random (source/mlsolution.cpp:754-874): a GRASP-style greedy
// randomized construction.  From depot 0, each step draws
//   r = rng.rand(ceil(alpha * count) - 1)          (MTRandom, source/mtrand.h:193-195)
// and appends the candidate of ascending rank r by distance to the client
// added last (both of the reference's branches select that rank: alpha < 0.5
// sorts descending and takes position count - r - 1).  The reference's
// std::sort leaves the order of equal distances to the library; here the
// rank is taken in (distance, client id) order.  costTour: depot 0 closes the
// tour.
//
// One warp builds one start.  MT19937 (source/mtrand.cpp:52-124) runs on
// lane 0 with its state in shared memory.  Each step selects rank r among the
// remaining candidates with a three-level radix select (10-bit digits of the
// 30-bit key distance << 14 | id) over a per-warp 1024-bin histogram.  Up to
// 2048 nodes the candidates and the step's keys stay in shared memory (one
// distance gather per candidate and step); larger instances keep the
// candidates in the tail of the tour being built and gather in every pass.
#include <cmath>
#include <cstdint>

#include "mlp_common.cuh"
#include "mlp_kernels.cuh"
#include "mlp_refsort.cuh"

namespace mlp {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kGraspWarps = 8;     // starts per CTA
constexpr int kGraspSmemN = 2048;  // up to this n a step's keys stay in shared memory
constexpr int kMtN = 624, kMtM = 397;

struct GraspSmem {
  static constexpr size_t mt = 0;                                 // uint32[kMtN] per warp
  static constexpr size_t hist = (size_t)kMtN * 4;                // uint32[1024]
  static constexpr size_t keys = hist + 1024 * 4;                 // uint32[kGraspSmemN]
  static constexpr size_t ids = keys + (size_t)kGraspSmemN * 4;   // int32[kGraspSmemN]
  static constexpr size_t per_warp = ids + (size_t)kGraspSmemN * 4;
  static constexpr size_t total = per_warp * kGraspWarps;
};

// MTRandom::seed (mtrand.cpp:52-61)
__device__ void mt_seed(uint32_t* st, uint32_t s) {
  st[0] = s;
  for (int p = 1; p < kMtN; p++) st[p] = 1812433253u * (st[p - 1] ^ (st[p - 1] >> 30)) + (uint32_t)p;
}

// MTRandom::gen (mtrand.cpp:99-124)
__device__ void mt_gen(uint32_t* st) {
  int i = 0;
  uint32_t y;
  for (; i < kMtN - kMtM; i++) {
    y = (st[i] & 0x80000000u) | (st[i + 1] & 0x7fffffffu);
    st[i] = st[i + kMtM] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
  }
  for (; i < kMtN - 1; i++) {
    y = (st[i] & 0x80000000u) | (st[i + 1] & 0x7fffffffu);
    st[i] = st[i + (kMtM - kMtN)] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
  }
  y = (st[kMtN - 1] & 0x80000000u) | (st[0] & 0x7fffffffu);
  st[kMtN - 1] = st[kMtM - 1] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

// MTRandom::rand() with tempering (mtrand.h:167-179); *pos is the state index.
__device__ uint32_t mt_rand(uint32_t* st, int* pos) {
  if (*pos >= kMtN) {
    mt_gen(st);
    *pos = 0;
  }
  uint32_t x = st[(*pos)++];
  x ^= (x >> 11);
  x ^= (x << 7) & 0x9d2c5680u;
  x ^= (x << 15) & 0xefc60000u;
  return x ^ (x >> 18);
}

// MTRandom::rand(max) (mtrand.h:193-195): IEEE double multiply and divide,
// as on the host.
__device__ uint32_t mt_rand_max(uint32_t* st, int* pos, uint32_t mx) {
  const double v = __dmul_rn((double)mx + 1.0, (double)mt_rand(st, pos));
  return (uint32_t)__ddiv_rn(v, 4294967296.0);
}

__device__ __forceinline__ uint32_t grasp_key(const int32_t* __restrict__ row, int32_t c) {
  return ((uint32_t)row[c] << 14) | (uint32_t)c;
}

// One step's selection: the key of rank r among the cnt keys key_of(q),
// q in [0, cnt) (three 10-bit digits, high first).
template <typename KeyOf>
__device__ uint32_t select_rank(uint32_t* hist, int cnt, uint32_t r, KeyOf key_of) {
  const int lane = threadIdx.x & 31;
  uint32_t prefix = 0;
#pragma unroll 1
  for (int lvl = 0; lvl < 3; lvl++) {
    const int sft = 20 - 10 * lvl;
    for (int q = lane; q < 1024; q += 32) hist[q] = 0;
    __syncwarp();
    for (int q = lane; q < cnt; q += 32) {
      const uint32_t k = key_of(q);
      if (lvl == 0 || (k >> (sft + 10)) == prefix) atomicAdd(&hist[(k >> sft) & 1023u], 1u);
    }
    __syncwarp();
    // lane l owns bins 32l .. 32l+31
    uint32_t own = 0;
#pragma unroll 8
    for (int q = 0; q < 32; q++) own += hist[32 * lane + q];
    uint32_t inc = own;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, inc, o);
      if (lane >= o) inc += y;
    }
    const uint32_t exc = inc - own;
    const unsigned hit = __ballot_sync(kFull, r >= exc && r < inc);
    const int src = hit ? __ffs(hit) - 1 : 0;  // the lane whose bins hold rank r
    uint32_t digit = 0, below = 0;
    if (lane == src) {
      uint32_t acc = exc;
      for (int q = 0; q < 32; q++) {
        const uint32_t h = hist[32 * lane + q];
        if (r < acc + h) {
          digit = 32u * lane + q;
          below = acc;
          break;
        }
        acc += h;
      }
    }
    digit = __shfl_sync(kFull, digit, src);
    below = __shfl_sync(kFull, below, src);
    r -= below;
    prefix = (prefix << 10) | digit;
    __syncwarp();  // hist is cleared by the next level
  }
  return prefix;
}

// The position q in [0, cnt) whose key equals `key` (-1 if none).
template <typename KeyOf>
__device__ int find_key(int cnt, uint32_t key, KeyOf key_of) {
  const int lane = threadIdx.x & 31;
  for (int q0 = 0; q0 < cnt; q0 += 32) {
    const int q = q0 + lane;
    const unsigned b = __ballot_sync(kFull, q < cnt && key_of(q) == key);
    if (b) return q0 + __ffs(b) - 1;
  }
  return -1;
}

__global__ void __launch_bounds__(32 * kGraspWarps)
    k_grasp(const GraspTask* __restrict__ tasks, int count, int* __restrict__ err) {
  extern __shared__ __align__(16) uint8_t gsm[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int start = blockIdx.x * kGraspWarps + wid;
  if (start >= count) return;  // whole warps only
  const GraspTask task = tasks[start];
  const int32_t* __restrict__ D = task.D;
  const int n = task.n;
  const float alpha = task.alpha;
  uint8_t* base = gsm + wid * GraspSmem::per_warp;
  uint32_t* st = (uint32_t*)(base + GraspSmem::mt);
  uint32_t* hist = (uint32_t*)(base + GraspSmem::hist);
  uint32_t* keys = (uint32_t*)(base + GraspSmem::keys);
  int32_t* ids = (int32_t*)(base + GraspSmem::ids);
  int32_t* t = task.tour;
  // Up to kGraspSmemN nodes the remaining candidates are ids[0..cnt) in
  // shared memory and their keys are gathered once per step; above, they
  // are t[len..n) and every pass gathers the keys again.
  const bool smem = n <= kGraspSmemN;
  int pos = kMtN;
  if (lane == 0) mt_seed(st, task.seed);
  if (smem) {
    for (int q = lane; q < n - 1; q += 32) ids[q] = q + 1;
  } else {
    for (int p = lane; p < n; p += 32) t[p] = p;
  }
  if (lane == 0) {
    t[0] = 0;
    t[n] = 0;
  }
  __syncwarp();
  int last = 0;
  for (int len = 1; len < n; len++) {
    const int cnt = n - len;
    uint32_t r = 0;
    if (lane == 0 && cnt > 1) {
      const uint32_t rcl = (uint32_t)ceilf(__fmul_rn(alpha, (float)cnt));
      r = rcl > 0 ? mt_rand_max(st, &pos, rcl - 1) : 0u;
    }
    r = __shfl_sync(kFull, r, 0);
    if (r >= (uint32_t)cnt) r = cnt - 1;  // alpha <= 1 (checked by the host) keeps r < cnt
    const int32_t* __restrict__ row = D + (size_t)last * n;
    uint32_t key;
    int q;
    if (smem) {
      for (int x = lane; x < cnt; x += 32) keys[x] = grasp_key(row, ids[x]);
      __syncwarp();
      auto key_of = [&](int x) { return keys[x]; };
      key = select_rank(hist, cnt, r, key_of);
      q = find_key(cnt, key, key_of);
    } else {
      auto key_of = [&](int x) { return grasp_key(row, t[len + x]); };
      key = select_rank(hist, cnt, r, key_of);
      q = find_key(cnt, key, key_of);
    }
    const int32_t cur = (int32_t)(key & 0x3fffu);
    if (q < 0) {  // unreachable (the rank-r key exists); t stays a permutation
      if (lane == 0) atomicAdd(err, 1);
      return;
    }
    if (lane == 0) {
      if (smem) {
        ids[q] = ids[cnt - 1];
        t[len] = cur;
      } else {
        t[len + q] = t[len];
        t[len] = cur;
      }
    }
    __syncwarp();
    last = cur;
  }
}

// MLSolution::random with the reference's own order of equal distances: the
// candidate array persists across steps exactly as clCands does
// (mlsolution.cpp:766-855) -- the clients 1..n-1 in id order at first; each
// step draws rclIndex (before sorting, as the reference), sorts the array by
// distance to the client added last with the reference's sort (ascending for
// alpha >= 0.5, descending otherwise, then rclIndex = count - rclIndex - 1),
// takes that entry and closes the gap by shifting the tail left.  One warp
// per start: the lanes gather the step's distances, lane 0 draws, sorts and
// shifts.  Up to kGraspRefSmemN nodes the arrays live in shared memory, else
// in the task's 2n words of the scratch buffer.
constexpr size_t kGraspRefSmem = (size_t)kMtN * 4 + (size_t)kGraspRefSmemN * 8;

__global__ void __launch_bounds__(32)
    k_grasp_ref(const GraspTask* __restrict__ tasks, uint32_t* __restrict__ scratch) {
  extern __shared__ __align__(16) uint8_t gsm[];
  const int lane = threadIdx.x;
  const GraspTask task = tasks[blockIdx.x];
  const int32_t* __restrict__ D = task.D;
  const int n = task.n;
  const float alpha = task.alpha;
  const bool desc = alpha < 0.5f;
  int32_t* t = task.tour;
  uint32_t* st = (uint32_t*)gsm;
  uint32_t* keys;
  int32_t* ids;
  if (n <= kGraspRefSmemN) {
    keys = st + kMtN;
    ids = (int32_t*)(keys + kGraspRefSmemN);
  } else {
    keys = scratch + task.scratch;
    ids = (int32_t*)(keys + n);
  }
  int pos = kMtN;
  if (lane == 0) {
    mt_seed(st, task.seed);
    t[0] = 0;
    t[n] = 0;
  }
  for (int q = lane; q < n - 1; q += 32) ids[q] = q + 1;
  __syncwarp();
  int last = 0;
  for (int len = 1; len < n; len++) {
    const int cnt = n - len;
    uint32_t idx = 0;
    if (cnt > 1) {
      if (lane == 0) {
        const uint32_t rcl = (uint32_t)ceilf(__fmul_rn(alpha, (float)cnt));
        idx = rcl > 0 ? mt_rand_max(st, &pos, rcl - 1) : 0u;
      }
      const int32_t* __restrict__ row = D + (size_t)last * n;
      for (int x = lane; x < cnt; x += 32) keys[x] = (uint32_t)row[ids[x]];
      __syncwarp();
      if (lane == 0) {
        RefSort(keys, ids, desc).sort(cnt);
        if (desc) idx = (uint32_t)cnt - idx - 1u;
      }
    }
    int32_t cur = 0;
    if (lane == 0) {
      if (idx >= (uint32_t)cnt) idx = cnt - 1;  // alpha <= 1 (checked by the host) keeps idx < cnt
      cur = ids[idx];
      t[len] = cur;
      for (int q = (int)idx; q + 1 < cnt; q++) ids[q] = ids[q + 1];
    }
    last = __shfl_sync(kFull, cur, 0);
    __syncwarp();
  }
}

}  // namespace

cudaError_t configure_grasp() {
  cudaError_t e = cudaFuncSetAttribute(k_grasp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GraspSmem::total);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_grasp_ref, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGraspRefSmem);
}

cudaError_t launch_grasp(const GraspTask* tasks, int count, int ties, uint32_t* scratch, int* err, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  const cudaError_t e = configure_grasp();
  if (e != cudaSuccess) return e;
  if (ties) {
    k_grasp_ref<<<count, 32, kGraspRefSmem, s>>>(tasks, scratch);
    return cudaGetLastError();
  }
  const int grid = (count + kGraspWarps - 1) / kGraspWarps;
  k_grasp<<<grid, 32 * kGraspWarps, GraspSmem::total, s>>>(tasks, count, err);
  return cudaGetLastError();
}

}  // namespace mlp
