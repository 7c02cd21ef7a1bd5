// Instantiation of the pass kernels for one arithmetic type.  Included by kernels_f64.cu
// (MWF_T = double, MWF_SUF = f64) and kernels_f32.cu (float, f32).
#include "mwf_kernels.cuh"
#include "mwf_stateops.cuh"
#include "mwf_launch.h"

namespace mwf {

#define MWF_CAT2(a, b) a##b
#define MWF_CAT(a, b) MWF_CAT2(a, b)
#define MWF_FN(name) MWF_CAT(name, MWF_CAT(_, MWF_SUF))

// Allow `smem` bytes of dynamic shared memory for `kernel`.  Past 48 KB of static plus dynamic
// shared memory a kernel needs the opt-in attribute; it is set to the device's whole opt-in
// budget (minus the kernel's static part) rather than to this launch's size, so a launch
// recorded earlier with a larger size (in a CUDA graph) stays valid.
template <typename K>
static cudaError_t set_smem(K kernel, size_t smem) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  if (smem + fa.sharedSizeBytes <= 48 * 1024) return cudaSuccess;
  int dev = 0, optin = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  if (smem + fa.sharedSizeBytes > (size_t)optin) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}

cudaError_t MWF_FN(launch_x_forward)(int nt, const RunDesc* runs, const WorkItem* items, int n, size_t smem,
                                     int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e;
#define MWF_XF(NT_)                                                  \
  if (nt == NT_) {                                                   \
    auto k = x_forward_kernel<MWF_T, kXfVptOf<MWF_T>, NT_>;           \
    e = set_smem(k, smem);                                           \
    if (e != cudaSuccess) return e;                                  \
    k<<<n, NT_, smem, st>>>(runs, items, err);                       \
    return cudaGetLastError();                                       \
  }
  MWF_XF(kXfThreads)
  MWF_XF(kXThreadsSmall)
#undef MWF_XF
  return cudaErrorInvalidValue;
}

cudaError_t MWF_FN(launch_z_nonlinear)(int K0, int ppt, int nt, const RunDesc* runs, const WorkItem* items,
                                       int n, size_t smem, int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e;
#define MWF_ZL(K0_, PPT_, NT_)                                                              \
  if (K0 == K0_ && ppt == PPT_ && nt == NT_) {                                             \
    constexpr bool nls = zpass_smem_acc(sizeof(MWF_T) == 8 ? 0 : 1, PPT_);                  \
    constexpr int nb = (sizeof(MWF_T) == 8 && PPT_ == 2) ? 2 : 4;                          \
    auto k = z_nonlinear_kernel<MWF_T, K0_, PPT_, NT_, nb, nls, false, sizeof(MWF_T) == 4>; \
    e = set_smem(k, smem);                                                                 \
    if (e != cudaSuccess) return e;                                                        \
    k<<<n, NT_, smem, st>>>(runs, items, err);                                             \
    return cudaGetLastError();                                                             \
  }
  MWF_ZL(4, 1, kZThreads)
  MWF_ZL(4, 2, kZThreads)
  MWF_ZL(6, 1, kZThreads)
  MWF_ZL(6, 2, kZThreads)
  if constexpr (sizeof(MWF_T) == 4) {
    MWF_ZL(4, 1, kZThreadsSmall)
    MWF_ZL(6, 1, kZThreadsSmall)
  }
#undef MWF_ZL
  return cudaErrorInvalidValue;
}

cudaError_t MWF_FN(launch_z_diag)(int K0, int ppt, int nt, const RunDesc* runs, const WorkItem* items,
                                       int n, size_t smem, int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e;
#define MWF_ZL(K0_, PPT_, NT_)                                                              \
  if (K0 == K0_ && ppt == PPT_ && nt == NT_) {                                             \
    constexpr bool nls = zpass_smem_acc(sizeof(MWF_T) == 8 ? 0 : 1, PPT_);                  \
    constexpr int nb = (sizeof(MWF_T) == 8 && PPT_ == 2) ? 2 : 4;                          \
    auto k = z_nonlinear_kernel<MWF_T, K0_, PPT_, NT_, nb, nls, true, sizeof(MWF_T) == 4>;  \
    e = set_smem(k, smem);                                                                 \
    if (e != cudaSuccess) return e;                                                        \
    k<<<n, NT_, smem, st>>>(runs, items, err);                                             \
    return cudaGetLastError();                                                             \
  }
  MWF_ZL(4, 1, kZThreads)
  MWF_ZL(4, 2, kZThreads)
  MWF_ZL(6, 1, kZThreads)
  MWF_ZL(6, 2, kZThreads)
  if constexpr (sizeof(MWF_T) == 4) {
    MWF_ZL(4, 1, kZThreadsSmall)
    MWF_ZL(6, 1, kZThreadsSmall)
  }
#undef MWF_ZL
  return cudaErrorInvalidValue;
}

cudaError_t MWF_FN(launch_x_inverse)(int nt, const RunDesc* runs, const WorkItem* items, int n, size_t smem,
                                     int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e;
#define MWF_XI(NT_)                                                  \
  if (nt == NT_) {                                                   \
    auto k = x_inverse_kernel<MWF_T, kXiVpt, NT_>;                    \
    e = set_smem(k, smem);                                           \
    if (e != cudaSuccess) return e;                                  \
    k<<<n, NT_, smem, st>>>(runs, items, err);                       \
    return cudaGetLastError();                                       \
  }
  MWF_XI(kXiThreads)
  MWF_XI(kXThreadsSmall)
#undef MWF_XI
  return cudaErrorInvalidValue;
}

cudaError_t MWF_FN(launch_energy)(const RunDesc* runs, int run, double* partial, int nparts, double* out,
                                  cudaStream_t st) {
  energy_partial_kernel<MWF_T><<<nparts, 256, 0, st>>>(runs, run, partial);
  energy_final_kernel<<<1, 32, 0, st>>>(partial, nparts, out);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_ref_to_dev)(const double* re, const double* im, void* out, int K, int M, int NN,
                                      cudaStream_t st) {
  const size_t tot = (size_t)K * M * NN;
  const int blocks = (int)((tot + 255) / 256 < 152 * 16 ? (tot + 255) / 256 : 152 * 16);
  ref_to_dev_kernel<MWF_T><<<blocks, 256, 0, st>>>(re, im, reinterpret_cast<cx<MWF_T>*>(out), K, M, NN);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_dev_to_ref)(const void* in, double* re, double* im, int K, int M, int NN,
                                      cudaStream_t st) {
  const size_t tot = (size_t)K * M * NN;
  const int blocks = (int)((tot + 255) / 256 < 152 * 16 ? (tot + 255) / 256 : 152 * 16);
  dev_to_ref_kernel<MWF_T><<<blocks, 256, 0, st>>>(reinterpret_cast<const cx<MWF_T>*>(in), re, im, K, M, NN);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_imposesym)(const RunDesc* runs, int run, int mode, int M, int NN, cudaStream_t st) {
  const size_t tot = (size_t)M * NN;
  const int blocks = (int)((tot + 255) / 256 < 152 * 8 ? (tot + 255) / 256 : 152 * 8);
  imposesym_kernel<MWF_T><<<blocks, 256, 0, st>>>(runs, run, mode);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_nonfinite)(const RunDesc* runs, int run, int* flag, cudaStream_t st) {
  nonfinite_kernel<MWF_T><<<152 * 4, 256, 0, st>>>(runs, run, flag);
  return cudaGetLastError();
}

// ---- state operations and diagnostics outside the timestep (mwf_stateops.cuh) ----

static inline int grid_for(size_t tot, int cap) {
  const size_t b = (tot + 255) / 256;
  return (int)(b < (size_t)cap ? (b ? b : 1) : (size_t)cap);
}

cudaError_t MWF_FN(launch_phys_z)(const RunDesc* runs, int run, int X, int KK, const FftPlanDev& planZ,
                                  size_t smem, double* out, int* err, cudaStream_t st) {
  auto k = phys_z_kernel<MWF_T, kPhysVpt, kPhysThreads>;
  cudaError_t e = set_smem(k, smem);
  if (e != cudaSuccess) return e;
  k<<<X * ((KK + 1) / 2), kPhysThreads, smem, st>>>(runs, run, planZ, out, err);
  return cudaGetLastError();
}

// the stand-alone transforms: x lines of up to kTrXVpt * kTrXThreads points, z lines of up to
// kPhysVpt * kPhysThreads
constexpr int kTrXThreads = 512, kTrXVpt = 8;

cudaError_t MWF_FN(launch_spec_x_backward)(const RunDesc* runs, int run, int X, int KK, int NN, const void* sp,
                                           int* err, cudaStream_t st) {
  auto k = spec_x_backward_kernel<MWF_T, kTrXVpt, kTrXThreads>;
  const size_t smem = xpass_smem(sizeof(MWF_T) == 8 ? 0 : 1, (size_t)X);
  cudaError_t e = set_smem(k, smem);
  if (e != cudaSuccess) return e;
  k<<<KK * NN, kTrXThreads, smem, st>>>(runs, run, reinterpret_cast<const cx<MWF_T>*>(sp), err);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_phys_z_forward)(const RunDesc* runs, int run, int X, int KK, int Z, const FftPlanDev& planZ,
                                          const double* ph, int* err, cudaStream_t st) {
  auto k = phys_z_forward_kernel<MWF_T, kPhysVpt, kPhysThreads>;
  const size_t smem = xpass_smem(sizeof(MWF_T) == 8 ? 0 : 1, (size_t)Z);
  cudaError_t e = set_smem(k, smem);
  if (e != cudaSuccess) return e;
  k<<<X * ((KK + 1) / 2), kPhysThreads, smem, st>>>(runs, run, planZ, ph, err);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_spec_x_forward)(const RunDesc* runs, int run, int X, int KK, int NN, void* sp, int* err,
                                          cudaStream_t st) {
  auto k = spec_x_forward_kernel<MWF_T, kTrXVpt, kTrXThreads>;
  const size_t smem = xpass_smem(sizeof(MWF_T) == 8 ? 0 : 1, (size_t)X);
  cudaError_t e = set_smem(k, smem);
  if (e != cudaSuccess) return e;
  k<<<KK * NN, kTrXThreads, smem, st>>>(runs, run, reinterpret_cast<cx<MWF_T>*>(sp), err);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_spectrum)(const RunDesc* runs, int run, int M, int NN, unsigned long long* mx,
                                    cudaStream_t st) {
  const dim3 grid((M + 255) / 256, (NN + kSpecRows - 1) / kSpecRows);
  spectrum_kernel<MWF_T><<<grid, 256, 0, st>>>(runs, run, mx);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_probes)(const RunDesc* runs, int run, int K0, int NN, double2* g, const int* zs,
                                  int nprobe, double* out, cudaStream_t st) {
  if (K0 == 4) probe_sum_kernel<MWF_T, 11><<<NN, 256, 0, st>>>(runs, run, g);
  else if (K0 == 6) probe_sum_kernel<MWF_T, 17><<<NN, 256, 0, st>>>(runs, run, g);
  else return cudaErrorInvalidValue;
  const int warps = nprobe * (3 * K0 - 1);
  probe_eval_kernel<MWF_T><<<(warps + 7) / 8, 256, 0, st>>>(runs, run, g, zs, nprobe, out);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_remap_x)(const RunDesc* runs, int run, const void* src, size_t elems, int factor,
                                   cudaStream_t st) {
  remap_x_kernel<MWF_T><<<grid_for(elems, 152 * 16), 256, 0, st>>>(runs, run,
                                                                  reinterpret_cast<const cx<MWF_T>*>(src), factor);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_blend)(const RunDesc* runs, int run, int other, size_t elems, double d, cudaStream_t st) {
  blend_kernel<MWF_T><<<grid_for(elems, 152 * 16), 256, 0, st>>>(runs, run, other, d);
  return cudaGetLastError();
}

cudaError_t MWF_FN(launch_noise)(const RunDesc* runs, int run, size_t elems, double scale,
                                 unsigned long long seed, cudaStream_t st) {
  noise_kernel<MWF_T><<<grid_for(elems, 152 * 16), 256, 0, st>>>(runs, run, scale, seed);
  return cudaGetLastError();
}

}  // namespace mwf
