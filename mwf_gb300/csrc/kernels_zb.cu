// Instantiations and launcher of the batched FP32 z pass (mwf_zbatch.cuh), one kernel per
// model (K0) and z line length NN = Q.
#include <algorithm>

#include "mwf_kernels.cuh"
#include "mwf_zbatch.cuh"
#include "mwf_launch.h"

namespace mwf {

bool zb_supported(int K0, int Q) {
  if (K0 != 4 && K0 != 6) return false;
  switch (Q) {
    case 32: case 48: case 64: case 96: case 128: case 192: case 256: break;
    default: return false;
  }
  return zb_smem_bytes(K0, Q, 1) <= zb_smem_budget(1);
}

int zb_blocks_per_sm(int K0, int Q) { return zb_minb(K0, Q); }

size_t zb_smem(int K0, int Q, int L) { return zb_smem_bytes(K0, Q, L); }

// SMs of the current device (the batched passes run one wave of resident CTAs over their items).
int sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 1;
  return sms > 0 ? sms : 1;
}

cudaError_t launch_z_batched(int K0, int Q, const RunDesc* runs, const WorkItem* items, int n, size_t smem,
                             int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
#define MWF_ZB(K0_, Q_)                                                                   \
  if (K0 == K0_ && Q == Q_) {                                                             \
    constexpr int minb = zb_minb(K0_, Q_);                                                \
    auto k = z_batched_kernel<K0_, Q_, kZbThreads, minb>;                                 \
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                         (int)zb_smem_budget(1));                        \
    if (e != cudaSuccess) return e;                                                      \
    if (smem > zb_smem_budget(minb)) return cudaErrorInvalidValue;                       \
    int per_sm = 0;                                                                      \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kZbThreads, smem);     \
    if (e != cudaSuccess) return e;                                                      \
    if (per_sm < 1) return cudaErrorInvalidConfiguration;                                \
    const int grid = std::min(n, per_sm * sm_count());                                   \
    k<<<grid, kZbThreads, smem, st>>>(runs, items, n, err);                              \
    return cudaGetLastError();                                                           \
  }
  MWF_ZB(4, 32) MWF_ZB(4, 48) MWF_ZB(4, 64) MWF_ZB(4, 96) MWF_ZB(4, 128) MWF_ZB(4, 192) MWF_ZB(4, 256)
  MWF_ZB(6, 32) MWF_ZB(6, 48) MWF_ZB(6, 64) MWF_ZB(6, 96) MWF_ZB(6, 128)
#undef MWF_ZB
  return cudaErrorInvalidValue;
}

}  // namespace mwf
