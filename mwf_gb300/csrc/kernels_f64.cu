#define MWF_T double
#define MWF_SUF f64
#include "kernels_inst.cuh"

namespace mwf {
// Arithmetic-peak probe: kFmaChains independent FMA chains per thread.
template <typename T>
__global__ void fma_probe_kernel(int iters, T* out) {
  T a[kFmaChains];
  const T m = T(0.999999), c = T(1e-7);
#pragma unroll
  for (int i = 0; i < kFmaChains; ++i) a[i] = T(threadIdx.x + i);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < kFmaChains; ++i) a[i] = fma(a[i], m, c);
  }
  T s = T(0);
#pragma unroll
  for (int i = 0; i < kFmaChains; ++i) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t launch_fma_probe(int which, int blocks, int threads, int iters, void* out, cudaStream_t st) {
  if (which == 0) fma_probe_kernel<double><<<blocks, threads, 0, st>>>(iters, reinterpret_cast<double*>(out));
  else fma_probe_kernel<float><<<blocks, threads, 0, st>>>(iters, reinterpret_cast<float*>(out));
  return cudaGetLastError();
}
}  // namespace mwf
