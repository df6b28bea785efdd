// mlp_legacy.cpp -- the reference's extern "C" DVND entry points
// (include/wamca_dvnd.h), implemented on the GB300 engine.
#include <cuda_runtime.h>

#include <algorithm>
#include <csignal>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/wamca_dvnd.h"
#include "mlp_capi_internal.h"
#include "mlp_engine.h"
#include "mlp_kernels.cuh"

using namespace mlp;

namespace {

constexpr unsigned kFail = 0xFFFFFFFFu;

struct DeviceState {
  mlp_problem_t problem = nullptr;  // bestNeighbor's problem on this device
  mlp_solver_t solver = nullptr;
};

struct LegacyState {
  std::mutex mu;
  bool bn_loaded = false;
  std::string bn_file;            // file of the first bestNeighbor call
  unsigned bn_host = 0;
  std::map<int, DeviceState> bn;  // per device
  std::map<unsigned, std::pair<mlp_problem_t, mlp_solver_t>> by_host;  // getProblem cache
  int32_t* dmoves = nullptr;
  size_t dmoves_cap = 0;
};

LegacyState& st() {
  static LegacyState* s = new LegacyState();  // lives until exit, like the reference's statics
  return *s;
}

// getProblem(file, hostCode): one problem per host code, loaded with
// costTour = true, distRound = false, coordShift = false (source/dvnd.cpp:163-175).
int cached_problem(const char* file, unsigned host, mlp_problem_t* p, mlp_solver_t* s) {
  auto& L = st();
  auto it = L.by_host.find(host);
  if (it != L.by_host.end()) {
    *p = it->second.first;
    *s = it->second.second;
    return kOk;
  }
  if (!file) {
    set_error("null instance file");
    return kErrArg;
  }
  mlp_problem_t prob = nullptr;
  int r = mlp_problem_load_tsplib(file, 1, 0, &prob);
  if (r != kOk) return r;
  mlp_solver_t sol = nullptr;
  r = mlp_solver_create(prob, 0, &sol);
  if (r != kOk) {
    mlp_problem_destroy(prob);
    return r;
  }
  L.by_host[host] = {prob, sol};
  *p = prob;
  *s = sol;
  return kOk;
}

}  // namespace

extern "C" {

MLP_API unsigned int bestNeighborSimple(char* file, int* solution, unsigned int solutionSize,
                                        int neighborhood) {
  return bestNeighbor(file, solution, solutionSize, neighborhood, false, 0, nullptr, nullptr, nullptr,
                      nullptr, nullptr, false, 1, nullptr);
}

MLP_API unsigned int bestNeighbor(char* file, int* solution, unsigned int solutionSize, int neighborhood,
                                  bool justCalc, unsigned int hostCode, unsigned int* useMoves,
                                  unsigned short* ids, unsigned int* is, unsigned int* js, int* costs,
                                  bool useMultipleGpu, unsigned int deviceCount, int* solutionResp) {
  auto& L = st();
  std::lock_guard<std::mutex> lock(L.mu);
  int dev = 0;
  if (useMultipleGpu && deviceCount > 0) dev = (int)(hostCode % deviceCount);  // dvnd.cu:14-17
  if (cudaSetDevice(dev) != cudaSuccess) {
    set_error("cudaSetDevice failed");
    return kFail;
  }
  if (!L.bn_loaded) {  // function-static problem of the first call (dvnd.cu:23)
    if (!file) {
      set_error("null instance file");
      return kFail;
    }
    L.bn_file = file;
    L.bn_host = hostCode;
    L.bn_loaded = true;
  }
  DeviceState& D = L.bn[dev];
  if (!D.problem) {
    if (mlp_problem_load_tsplib(L.bn_file.c_str(), 1, 0, &D.problem) != kOk) {
      L.bn.erase(dev);
      return kFail;
    }
    if (mlp_solver_create(D.problem, 0, &D.solver) != kOk) {
      mlp_problem_destroy(D.problem);
      L.bn.erase(dev);
      return kFail;
    }
  }
  if (!solution) {
    set_error("null solution");
    return kFail;
  }
  if (mlp_solver_set_tour(D.solver, solution, (int32_t)solutionSize) != kOk) return kFail;
  if (justCalc) {  // dvnd.cu:34-39
    int64_t c = 0;
    if (mlp_solver_cost(D.solver, &c) != kOk) return kFail;
    return (unsigned)c;
  }
  if (neighborhood < 0 || neighborhood > 4) {
    set_error("invalid neighborhood (the reference builds kernels 0..4 for the DVND)");
    return kFail;
  }
  const unsigned want = useMoves ? *useMoves : 0u;
  const int cap = want > 0 ? (int)std::min<unsigned>(want, 1u << 20) : 0;
  std::vector<int32_t> mi(cap), mj(cap), mid(cap);
  std::vector<int64_t> mc(cap);
  int32_t count = 0;
  int64_t cost = 0;
  if (mlp_solver_pass(D.solver, neighborhood, cap, mid.data(), mi.data(), mj.data(), mc.data(), &count,
                      &cost) != kOk)
    return kFail;
  std::vector<int32_t> tour(solutionSize);
  if (mlp_solver_get_tour(D.solver, tour.data(), (int32_t)solutionSize) != kOk) return kFail;
  if (want > 0) {  // dvnd.cu:55-68
    const int take = std::min<int>(count, cap);
    for (int q = 0; q < take; q++) {
      if (ids) ids[q] = (unsigned short)mid[q];
      if (is) is[q] = (unsigned)mi[q];
      if (js) js[q] = (unsigned)mj[q];
      if (costs) costs[q] = (int)mc[q];
    }
    *useMoves = (unsigned)take;
    if (solutionResp)  // WamcaExperiment.hpp:554-559
      std::copy(tour.begin(), tour.end(), solutionResp);
  } else {
    std::copy(tour.begin(), tour.end(), solution);  // WamcaExperiment.hpp:546-551
  }
  return (unsigned)cost;
}

MLP_API unsigned int applyMoves(char* file, int* solution, unsigned int solutionSize, unsigned int nMoves,
                                unsigned short* ids, unsigned int* is, unsigned int* js, int* costs) {
  (void)costs;  // the reference adds them to a cost it then recomputes (dvnd.cpp:37, 139-140)
  auto& L = st();
  std::lock_guard<std::mutex> lock(L.mu);
  mlp_problem_t p = nullptr;
  mlp_solver_t s = nullptr;
  if (cached_problem(file, 0, &p, &s) != kOk) return kFail;
  if (!solution || (nMoves > 0 && (!ids || !is || !js))) {
    set_error("null argument");
    return kFail;
  }
  if (mlp_solver_set_tour(s, solution, (int32_t)solutionSize) != kOk) return kFail;
  const int size = (int)solutionSize;
  std::vector<int32_t> mv(3 * (size_t)nMoves);
  for (unsigned q = 0; q < nMoves; q++) {
    const int id = ids[q], i = (int)is[q], j = (int)js[q];
    if (id >= 30) continue;  // ignored by the reference (dvnd.cpp:76)
    int f0 = std::min(i, j), f1 = std::max(i, j);
    if (id > 1) f1 = std::max(i, j) + (id - 1) - 1;
    if (f0 < 1 || f1 > size - 2) {
      set_error("move outside the tour's client positions 1..size-2");
      return kFail;
    }
    mv[3 * q] = id;
    mv[3 * q + 1] = i;
    mv[3 * q + 2] = j;
  }
  // Drop ignored ids (>= 30) while keeping the order.
  std::vector<int32_t> keep;
  for (unsigned q = 0; q < nMoves; q++)
    if (ids[q] < 30) keep.insert(keep.end(), mv.begin() + 3 * q, mv.begin() + 3 * q + 3);
  const int m = (int)(keep.size() / 3);
  cudaStream_t stream = s->set->stream();
  if (m > 0) {
    if ((size_t)m * 3 > L.dmoves_cap) {
      if (L.dmoves) cudaFree(L.dmoves);
      L.dmoves_cap = (size_t)m * 3;
      if (cudaMalloc(&L.dmoves, sizeof(int32_t) * L.dmoves_cap) != cudaSuccess) {
        L.dmoves = nullptr;
        L.dmoves_cap = 0;
        set_error("cudaMalloc failed");
        return kFail;
      }
    }
    if (cuda_status(cudaMemcpyAsync(L.dmoves, keep.data(), sizeof(int32_t) * keep.size(),
                                    cudaMemcpyHostToDevice, stream),
                    "copy moves") != kOk)
      return kFail;
    if (cuda_status(launch_legacy_apply(s->set->device_jobs(), L.dmoves, m, stream), "apply kernel") != kOk)
      return kFail;
    if (s->set->prepare(false) != kOk) return kFail;
  }
  if (mlp_solver_get_tour(s, solution, (int32_t)solutionSize) != kOk) return kFail;
  int64_t c = 0;
  if (mlp_solver_cost(s, &c) != kOk) return kFail;
  return (unsigned)c;
}

// noConflict(const MLMove64&, const MLMove64&), dvnd.cu:132-175, with the
// bit-field widths of MLMove64 (id:4, i:14, j:14; mlads.h:190-195).
static bool legacy_no_conflict(int id1, int i1, int j1, int id2, int i2, int j2) {
  auto K = [](int id) -> unsigned { return id == 2 ? 1u : (id == 3 ? 2u : 3u); };
  auto MN = [](int a, int b) { return a < b ? a : b; };
  auto MX = [](int a, int b) { return a > b ? a : b; };
  auto ab = [](int v) { return v >= 0 ? v : -v; };
  if (id1 == 0) {
    if (id2 == 0) return ab(i1 - i2) > 1 && ab(i1 - j2) > 1 && ab(j1 - i2) > 1 && ab(j1 - j2) > 1;
    if (id2 == 1) return ((i1 < i2 - 1) || (i1 > j2 - 1)) && ((j1 < i2 - 1) || (j1 > j2 + 1));
    const unsigned k2 = K(id2);
    return (j1 < MN(i2, j2) - 1) || ((unsigned)i1 > (unsigned)MX(i2, j2) + k2) ||
           ((i1 < MN(i2, j2) - 1) && ((unsigned)j1 > (unsigned)MX(i2, j2) + k2));
  }
  if (id1 == 1) {
    if (id2 == 0) return ((i2 < i1 - 1) || (i2 > j1 + 1)) && ((j2 < i1 - 1) || (j2 > j1 + 1));
    if (id2 == 1) return (j1 < i2 - 1) || (i1 > j2 + 1) || (j2 > i1 - 1) || (i2 > j1 + 1);
    const unsigned k2 = K(id2);
    return ((unsigned)i1 > (unsigned)MX(i2, j2) + k2) || (j1 < MN(i2, j2) - 1);
  }
  const unsigned k1 = K(id1);
  if (id2 == 0)
    return (j2 < MN(i1, i2) - 1) || ((unsigned)i2 > (unsigned)MX(i1, i2) + k1) ||
           ((i2 < MN(i1, i2) - 1) && ((unsigned)j2 > (unsigned)MX(i1, i2) + k1));
  if (id2 == 1) return (j2 < MN(i1, j1) - 1) || ((unsigned)i2 > (unsigned)MX(i1, j1) + k1);
  const unsigned k2 = K(id2);
  return ((unsigned)MX(i1, j1) + k1 < (unsigned)MN(i2, j2)) || ((unsigned)MN(i1, j1) > (unsigned)MX(i2, j2) + k2);
}

MLP_API bool noConflict(unsigned short id1, unsigned int i1, unsigned int j1, unsigned short id2,
                        unsigned int i2, unsigned int j2) {
  return legacy_no_conflict(id1 & 0xf, (int)(i1 & 0x3fff), (int)(j1 & 0x3fff), id2 & 0xf, (int)(i2 & 0x3fff),
                            (int)(j2 & 0x3fff));
}

// betterNoConflict (dvnd.cu:85-130): std::sort (unstable, like the reference),
// then the first-conflict marking loop.
MLP_API int getNoConflictMoves(unsigned int nMoves, unsigned short* ids, unsigned int* is, unsigned int* js,
                               int* costs, int* selectedMoves, int* impValue, bool maximize,
                               bool melhorParaPior) {
  if (nMoves > 0 && (!ids || !is || !js || !costs || !selectedMoves)) {
    set_error("null argument");
    return -1;
  }
  if (!impValue) {
    set_error("null impValue");
    return -1;
  }
  struct MoveIndex {
    int idx;
    unsigned index;
  };
  std::vector<MoveIndex> v(nMoves);
  for (unsigned q = 0; q < nMoves; q++) v[q] = MoveIndex{(int)q, q};
  const bool desc = melhorParaPior ? maximize : !maximize;
  if (desc)
    std::sort(v.begin(), v.end(), [&](const MoveIndex& a, const MoveIndex& b) { return costs[a.idx] > costs[b.idx]; });
  else
    std::sort(v.begin(), v.end(), [&](const MoveIndex& a, const MoveIndex& b) { return costs[a.idx] < costs[b.idx]; });
  for (unsigned a = 0; a < nMoves; a++) {
    for (unsigned b = a + 1; b < nMoves; b++) {
      const int p = v[a].idx, q = v[b].idx;
      if (!noConflict(ids[p], is[p], js[p], ids[q], is[q], js[q])) {
        if (melhorParaPior) v[b].index = (unsigned)-1;
        else v[a].index = (unsigned)-1;
        break;
      }
    }
  }
  int len = 0, imp = 0;
  for (unsigned a = 0; a < nMoves; a++)
    if (v[a].index != (unsigned)-1) {
      selectedMoves[len++] = (int)v[a].index;
      imp += costs[v[a].idx];
    }
  *impValue = imp;
  return len;
}

// dvnd.cpp:230-233: raises SIGSEGV in the calling process, as the reference does.
MLP_API void segFault(void) { std::raise(SIGSEGV); }

MLP_API void mlp_legacy_reset(void) {
  auto& L = st();
  std::lock_guard<std::mutex> lock(L.mu);
  for (auto& kv : L.bn) {
    mlp_solver_destroy(kv.second.solver);
    mlp_problem_destroy(kv.second.problem);
  }
  L.bn.clear();
  for (auto& kv : L.by_host) {
    mlp_solver_destroy(kv.second.second);
    mlp_problem_destroy(kv.second.first);
  }
  L.by_host.clear();
  L.bn_loaded = false;
  L.bn_file.clear();
}

}  // extern "C"
