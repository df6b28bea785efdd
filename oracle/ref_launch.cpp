/*
 * ref_launch.cpp -- TEST AND BASELINE INFRASTRUCTURE.
 *
 * Runs the reference's own ODC neighbourhood kernels (kernelSwap
 * source/mlkswap.cu:888-967, kernel2Opt source/mlk2opt.cu:459-635,
 * kernelOrOpt source/mlkoropt.cu:620-794), compiled from its sources into
 * oracle/_ref/ref_*.cubin, through the CUDA driver API with the reference's
 * own launch configuration (defineKernelGrid + launchKernel,
 * source/mlkswap.cu:979-1063, source/mlk2opt.cu:646-723,
 * source/mlkoropt.cu:806-883):
 *   grid   (1, ((size+1)/2)-1)  swap; (1, ceil(size/2)) 2-opt; (1, size-k-2) Or-opt-k
 *   block  cudaOccupancyMaxPotentialBlockSizeVariableSMem with the shared
 *          size 3*4*size + 2*4*blockSize (MLKernelSharedSize,
 *          source/mlkernel.h:331-352), block size limit = size
 *   shared 5 * 4 * size bytes
 * Inputs are the reference's MLADSData buffer (the engine builds it) and a
 * move buffer of one 64-bit MLMovePack per block.  Used by the tests (the
 * reference kernels' block costs against the engine's) and by bench.py (the
 * reference kernels' time on the same GPU).  Never part of the product.
 */
#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <string>

namespace {

CUmodule g_mod[3] = {nullptr, nullptr, nullptr};
CUfunction g_fn[3] = {nullptr, nullptr, nullptr};
int g_size = 0;  // for the occupancy callback
char g_err[256] = "";

// Kernel symbols (Itanium mangling of the reference's signatures).
const char* kFiles[3] = {"ref_mlkswap.cubin", "ref_mlk2opt.cubin", "ref_mlkoropt.cubin"};
const char* kNames[3] = {"_Z10kernelSwapPK9MLADSDataP10MLMovePacki", "_Z10kernel2OptPK9MLADSDataP10MLMovePacki",
                         "_Z11kernelOrOptPK9MLADSDataP10MLMovePackii"};

size_t shared_for_block(int block) {  // MLKernelSharedSize::operator()
  return (size_t)(3 * 4 * g_size + 2 * 4 * block);
}

int fail(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  std::snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "unknown CUDA driver error");
  return (int)r;
}

}  // namespace

extern "C" {

const char* rl_error() { return g_err; }

/* Loads the three cubins from `dir` into the current context (the primary
 * context of device 0 when none is current). */
int rl_init(const char* dir) {
  CUresult r = cuInit(0);
  if (r != CUDA_SUCCESS) return fail("cuInit", r);
  CUcontext ctx = nullptr;
  cuCtxGetCurrent(&ctx);
  if (!ctx) {
    CUdevice dev;
    if ((r = cuDeviceGet(&dev, 0)) != CUDA_SUCCESS) return fail("cuDeviceGet", r);
    if ((r = cuDevicePrimaryCtxRetain(&ctx, dev)) != CUDA_SUCCESS) return fail("cuDevicePrimaryCtxRetain", r);
    if ((r = cuCtxSetCurrent(ctx)) != CUDA_SUCCESS) return fail("cuCtxSetCurrent", r);
  }
  for (int q = 0; q < 3; q++) {
    if (g_fn[q]) continue;
    const std::string path = std::string(dir) + "/" + kFiles[q];
    if ((r = cuModuleLoad(&g_mod[q], path.c_str())) != CUDA_SUCCESS) return fail(path.c_str(), r);
    if ((r = cuModuleGetFunction(&g_fn[q], g_mod[q], kNames[q])) != CUDA_SUCCESS) return fail(kNames[q], r);
  }
  return 0;
}

/* Launches the reference kernel of neighbourhood nb (0 swap, 1 2-opt,
 * 2..4 Or-opt-1..3) `reps` times on the legacy stream over `ads` (device
 * MLADSData of a tour of `size` positions) into `moves` (one uint64 per
 * block); *ms = mean time per launch, *block / *grid = the configuration. */
int rl_eval(int nb, uint64_t ads, int size, uint64_t moves, int reps, float* ms, int* block, int* grid) {
  if (nb < 0 || nb > 4 || size < 8 || reps < 1) {
    std::snprintf(g_err, sizeof(g_err), "bad arguments");
    return -1;
  }
  CUfunction f = g_fn[nb < 2 ? nb : 2];
  if (!f) {
    std::snprintf(g_err, sizeof(g_err), "rl_init first");
    return -1;
  }
  const int k = nb - 1;
  const int gy = nb == 0 ? ((size + 1) / 2) - 1 : (nb == 1 ? (size + 1) / 2 : size - k - 2);
  g_size = size;
  int min_grid = 0, bs = 0;
  CUresult r = cuOccupancyMaxPotentialBlockSize(&min_grid, &bs, f, shared_for_block, 0, size);
  if (r != CUDA_SUCCESS) return fail("cuOccupancyMaxPotentialBlockSize", r);
  const unsigned shared = (unsigned)(5 * 4 * size);
  CUdeviceptr a = (CUdeviceptr)ads, m = (CUdeviceptr)moves;
  int sz = size, kk = k;
  void* p3[] = {&a, &m, &sz};
  void* p4[] = {&a, &m, &kk, &sz};
  CUevent e0, e1;
  if ((r = cuEventCreate(&e0, CU_EVENT_DEFAULT)) != CUDA_SUCCESS) return fail("cuEventCreate", r);
  if ((r = cuEventCreate(&e1, CU_EVENT_DEFAULT)) != CUDA_SUCCESS) return fail("cuEventCreate", r);
  cuEventRecord(e0, nullptr);
  for (int q = 0; q < reps && r == CUDA_SUCCESS; q++)
    r = cuLaunchKernel(f, 1, (unsigned)gy, 1, (unsigned)bs, 1, 1, shared, nullptr, nb < 2 ? p3 : p4, nullptr);
  cuEventRecord(e1, nullptr);
  if (r == CUDA_SUCCESS) r = cuEventSynchronize(e1);
  float t = 0.0f;
  if (r == CUDA_SUCCESS) cuEventElapsedTime(&t, e0, e1);
  cuEventDestroy(e0);
  cuEventDestroy(e1);
  if (r != CUDA_SUCCESS) return fail("reference kernel", r);
  if (ms) *ms = t / (float)reps;
  if (block) *block = bs;
  if (grid) *grid = gy;
  return 0;
}

}  // extern "C"
