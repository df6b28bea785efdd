/*
 * Forced-include prelude used only when the reference's CPU evaluator is
 * compiled from its own sources into oracle/_ref (test infrastructure).
 *
 * The reference's gpu.h pulls in a vendored CUDA-samples helper header that no
 * longer compiles against CUDA 13 (it reads cudaDeviceProp fields that were
 * removed).  The evaluator only needs `checkCudaErrors`, so this prelude marks
 * that header as already included (its include guard is `__gpu_helper_h`) and
 * supplies a minimal `checkCudaErrors` of our own.
 */
#ifndef ORACLE_REF_PRELUDE_H
#define ORACLE_REF_PRELUDE_H

#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>

#define __gpu_helper_h 1

#ifndef checkCudaErrors
#define checkCudaErrors(call)                                              \
  do {                                                                     \
    cudaError_t oracle_ref_err_ = (call);                                  \
    if (oracle_ref_err_ != cudaSuccess) {                                  \
      std::fprintf(stderr, "oracle/_ref: CUDA error %d at %s:%d\n",        \
                   (int)oracle_ref_err_, __FILE__, __LINE__);              \
      std::abort();                                                        \
    }                                                                      \
  } while (0)
#endif

#endif
