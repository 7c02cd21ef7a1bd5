// The persistent FP32 step kernel (mwf_persist.cuh) and its launcher.
#include "mwf_persist.cuh"
#include "mwf_launch.h"

namespace mwf {

static_assert(sizeof(PersistItem) == 4 * sizeof(int), "PersistItem layout");

// Allow the kernel the device's whole opt-in shared memory less its static part.
static cudaError_t persistent_attr() {
  auto k = persistent_step_kernel<kZbThreads>;
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, k);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(zb_smem_budget(1) - fa.sharedSizeBytes));
}

int persistent_grid(size_t smem) {
  if (persistent_attr() != cudaSuccess) return -1;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_step_kernel<kZbThreads>, kZbThreads, smem) !=
      cudaSuccess)
    return -1;
  return sms * per_sm;
}

cudaError_t launch_persistent_step(const RunDesc* runs, const void* items, int n_items, int* counters, size_t smem,
                                   int grid, int* err, cudaStream_t st) {
  if (n_items <= 0) return cudaSuccess;
  if (grid <= 0) return cudaErrorInvalidValue;
  cudaError_t e = persistent_attr();
  if (e != cudaSuccess) return e;
  persistent_step_kernel<kZbThreads><<<grid, kZbThreads, smem, st>>>(
      runs, reinterpret_cast<const PersistItem*>(items), n_items, counters, err);
  return cudaGetLastError();
}

}  // namespace mwf
