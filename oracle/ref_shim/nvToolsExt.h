/* Redirects the reference's legacy NVTX include to the header-only NVTX3 copy shipped with CUDA 13. */
#include <nvtx3/nvToolsExt.h>
