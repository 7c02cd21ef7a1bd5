// Instantiations and launchers of the FP32 subset-split x passes (mwf_xbatch.cuh), one kernel
// per MM.
#include <algorithm>

#include "mwf_kernels.cuh"
#include "mwf_xbatch.cuh"
#include "mwf_launch.h"

namespace mwf {

bool xb_supported(int MM) {
  switch (MM) {
    case 32: case 48: case 64: case 96: case 128: case 192: case 256: return true;
    default: return false;
  }
}

size_t xbf_smem(int MM, int nb) { return xbf_smem_bytes(MM, nb); }
size_t xbi_smem(int MM, int nb) { return xbi_smem_bytes(MM, nb); }

#define MWF_XB_CASES(F) F(32) F(48) F(64) F(96) F(128) F(192) F(256)

cudaError_t launch_x_forward_batched(int MM, const RunDesc* runs, const WorkItem* items, int n, size_t smem,
                                     int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (smem > zb_smem_budget(kXfBlocks)) return cudaErrorInvalidValue;
#define MWF_XF(MM_)                                                                         \
  if (MM == MM_) {                                                                          \
    auto k = xf_batched_kernel<MM_, kXbThreads, kXfBlocks>;                                 \
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                         (int)zb_smem_budget(1));                          \
    if (e != cudaSuccess) return e;                                                        \
    int per_sm = 0;                                                                        \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kXbThreads, smem);       \
    if (e != cudaSuccess) return e;                                                        \
    if (per_sm < 1) return cudaErrorInvalidConfiguration;                                  \
    const int grid = std::min(n, per_sm * sm_count());                                     \
    k<<<grid, kXbThreads, smem, st>>>(runs, items, n, err);                                \
    return cudaGetLastError();                                                             \
  }
  MWF_XB_CASES(MWF_XF)
#undef MWF_XF
  return cudaErrorInvalidValue;
}

cudaError_t launch_x_inverse_batched(int MM, const RunDesc* runs, const WorkItem* items, int n, size_t smem,
                                     int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (smem > zb_smem_budget(kXiBlocks)) return cudaErrorInvalidValue;
#define MWF_XI(MM_)                                                                         \
  if (MM == MM_) {                                                                          \
    auto k = xi_batched_kernel<MM_, kXbThreads, kXiBlocks>;                                 \
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                         (int)zb_smem_budget(1));                          \
    if (e != cudaSuccess) return e;                                                        \
    k<<<n, kXbThreads, smem, st>>>(runs, items, err);                                       \
    return cudaGetLastError();                                                             \
  }
  MWF_XB_CASES(MWF_XI)
#undef MWF_XI
  return cudaErrorInvalidValue;
}

}  // namespace mwf
