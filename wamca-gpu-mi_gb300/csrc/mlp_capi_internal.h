// mlp_capi_internal.h -- definitions behind the opaque C-ABI handles.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "mlp_engine.h"

// NVTX range around a public entry point (Nsight Systems / Compute show the
// library's calls by name; a no-op without a tool attached).
struct MlpRange {
  explicit MlpRange(const char* name) { nvtxRangePushA(name); }
  ~MlpRange() { nvtxRangePop(); }
  MlpRange(const MlpRange&) = delete;
  MlpRange& operator=(const MlpRange&) = delete;
};
#define MLP_RANGE(name) MlpRange mlp_range_(name)

struct mlp_solver {
  mlp::Problem* prob = nullptr;
  bool wide = false;
  cudaStream_t own_stream = nullptr;
  std::unique_ptr<mlp::Job> job;
  std::unique_ptr<mlp::JobSet> set;
  uint32_t* dads = nullptr;  // reference ADS buffer (allocated on first use)
  uint32_t* dP = nullptr;    // prefix of T used to write the C matrix
  ~mlp_solver();
};

struct mlp_batch {
  bool wide = false;
  int shape = -1;
  int mask = 0x1f;
  int merge_mode = 0;
  int sweep_kernel = 1;
  int check_interval = 4;
  bool total = false;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<std::unique_ptr<mlp::Job>> jobs;
  std::vector<std::vector<int32_t>> tours;  // empty: the start is built on the device
  struct RandomStart {
    uint32_t seed = 0;
    float alpha = 0;
    int32_t ties = 0;
  };
  std::vector<RandomStart> random_start;  // seed, alpha and tie order of those
  std::unique_ptr<mlp::JobSet> set;
  ~mlp_batch();
};

namespace mlp {
int validate_tour(const int32_t* tour, int len, int n, int size);
int solver_init(mlp_solver* s, Problem* p, int wide);
}  // namespace mlp
