// Host check of RefSort (wamca-gpu-mi_gb300/csrc/mlp_refsort.cuh) against the
// C++ library's std::sort and std::partial_sort: the permutation of (key, id)
// pairs ordered by key alone must be the library's, element for element, in
// both directions, on arrays with many equal keys (random, sorted, reversed,
// organ-pipe and few-distinct-key inputs) of every size up to 300 and some
// larger ones, and along repeated re-sorts of one array as the constructor of
// MLSolution::random performs them.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "mlp_refsort.cuh"

static long g_bad = 0, g_cases = 0;

static void check(const std::vector<uint32_t>& keys, std::vector<int32_t> ids, bool desc, bool heap) {
  std::vector<int32_t> lib = ids;
  auto comp = [&](int32_t a, int32_t b) { return desc ? keys[a] > keys[b] : keys[a] < keys[b]; };
  if (heap) std::partial_sort(lib.begin(), lib.end(), lib.end(), comp);
  else std::sort(lib.begin(), lib.end(), comp);
  std::vector<uint32_t> k(ids.size());
  for (size_t q = 0; q < ids.size(); q++) k[q] = keys[ids[q]];
  mlp::RefSort rs(k.data(), ids.data(), desc);
  if (heap) rs.heap_sort(0, (int)ids.size());
  else rs.sort((int)ids.size());
  g_cases++;
  if (ids != lib) {
    if (g_bad < 5) std::printf("mismatch n=%zu desc=%d heap=%d\n", ids.size(), (int)desc, (int)heap);
    g_bad++;
  }
}

int main() {
  std::mt19937 rng(12345);
  for (int n = 0; n <= 300; n++) {
    for (int rep = 0; rep < 6; rep++) {
      const uint32_t span = rep % 3 == 0 ? 3 : (rep % 3 == 1 ? (uint32_t)n / 4 + 1 : 1000);
      std::vector<uint32_t> keys(n);
      for (auto& v : keys) v = rng() % span;
      if (rep == 3) std::sort(keys.begin(), keys.end());
      if (rep == 4) std::sort(keys.rbegin(), keys.rend());
      if (rep == 5)
        for (int q = 0; q < n; q++) keys[q] = (uint32_t)std::min(q, n - 1 - q) % (span + 7);
      std::vector<int32_t> ids(n);
      for (int q = 0; q < n; q++) ids[q] = q;
      std::shuffle(ids.begin(), ids.end(), rng);
      for (int desc = 0; desc < 2; desc++)
        for (int heap = 0; heap < 2; heap++) check(keys, ids, desc != 0, heap != 0);
    }
  }
  for (int n : {511, 1000, 1023, 2047, 4000, 9999}) {
    for (int rep = 0; rep < 4; rep++) {
      std::vector<uint32_t> keys(n);
      for (auto& v : keys) v = rng() % (rep == 0 ? 2 : (rep == 1 ? 50 : 1500));
      std::vector<int32_t> ids(n);
      for (int q = 0; q < n; q++) ids[q] = q;
      std::shuffle(ids.begin(), ids.end(), rng);
      for (int desc = 0; desc < 2; desc++)
        for (int heap = 0; heap < 2; heap++) check(keys, ids, desc != 0, heap != 0);
    }
  }
  // Repeated re-sorts of one array with fresh keys (the constructor's pattern):
  // each sort starts from the previous permutation.
  for (int n : {52, 300, 1000}) {
    std::vector<int32_t> lib(n - 1), mine(n - 1);
    for (int q = 0; q < n - 1; q++) lib[q] = mine[q] = q + 1;
    for (int step = 0; step < 200 && !lib.empty(); step++) {
      std::vector<uint32_t> keys(n);
      for (auto& v : keys) v = rng() % 40;
      const bool desc = step % 3 == 0;
      auto comp = [&](int32_t a, int32_t b) { return desc ? keys[a] > keys[b] : keys[a] < keys[b]; };
      std::sort(lib.begin(), lib.end(), comp);
      std::vector<uint32_t> k(mine.size());
      for (size_t q = 0; q < mine.size(); q++) k[q] = keys[mine[q]];
      mlp::RefSort(k.data(), mine.data(), desc).sort((int)mine.size());
      g_cases++;
      if (lib != mine) g_bad++;
      const size_t pick = rng() % lib.size();
      lib.erase(lib.begin() + pick);
      mine.erase(mine.begin() + pick);
    }
  }
  std::printf("%ld cases, %ld mismatches\n", g_cases, g_bad);
  return g_bad != 0;
}
