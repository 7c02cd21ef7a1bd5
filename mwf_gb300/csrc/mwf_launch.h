// Host-side launch entry points of the kernels (defined per precision in kernels_f64.cu and
// kernels_f32.cu so the two instantiation sets compile in parallel).
#pragma once
#include <cuda_runtime.h>
#include "mwf_common.cuh"

namespace mwf {

// Compile-time shapes shared by the host planner and the kernels.
constexpr int kXfThreads = 512;   // x-pass block size (FP64, and FP32 lines longer than 1536)
constexpr int kXThreadsSmall = 256;  // x-pass block size for lines up to 1536 (FP32: 4 CTAs per SM, FP64: 2)
constexpr int kXfVpt = 6;         // x-pass line capacity per thread that picks the block size
// x-forward complex values per thread (nb*X <= VPT*threads): twice the x-inverse tile, so fewer
// threads idle in the radix-12/16 stages (x forward 13 % faster on a 512-run FP32 ensemble,
// 3 % on the 1536^2 FP64 case; the x inverse, holding three fields, is faster at 6)
template <typename T> constexpr int kXfVptOf = 12;
inline int xf_vpt(int prec) { return prec == 0 ? kXfVptOf<double> : kXfVptOf<float>; }
constexpr int kXiThreads = 512;
constexpr int kXiVpt = 6;         // x-inverse values per thread and field: nb*X <= 6*threads

// Block size of the x passes for a run.
inline int xpass_threads(int prec, int X) { (void)prec; return X <= kXfVpt * kXThreadsSmall ? kXThreadsSmall : kXfThreads; }
constexpr int kZThreads = 512;    // z-pass block size (FP64, and FP32 lines longer than 256)
constexpr int kZThreadsSmall = 256;  // FP32 z-pass block size for NN <= 256 (3 CTAs per SM)
// z-pass variants: the nonlinear accumulators live in shared memory (FP64, and FP32 with one
// point per thread, where the registers go to the transforms) or in registers (FP32 with two
// points per thread, whose staging buffers fill shared memory); transforms in flight per
// batch: 4, or 2 for FP64 with 2 points per thread.  FP32 stages the next task's rows.
constexpr bool zpass_smem_acc(int prec, int ppt) { return prec == 0 || ppt == 1; }
inline int zpass_nb(int prec, int ppt) { return (prec == 0 && ppt == 2) ? 2 : 4; }
// FP32 z items run the three z-subsets of their lines in turn and sum them into one partial
// (the x-inverse pass, latency-bound on its HBM reads there, then reads a third as much: 1.44 ->
// 1.29 ms on a 512-run ensemble).  FP64 keeps one subset per item: on the 1536^2 M6 case the
// summed form cost the z pass 0.63 ms and saved the x inverse 0.14 ms.
constexpr bool zpass_summed(int prec) { return prec == 1; }
// FP32 M4 with one point per thread also holds a second transform buffer (out-of-place
// two-stage transforms); for M6 it would cost the third CTA per SM.
__host__ __device__ constexpr bool zpass_pingpong(int prec, int K0, int ppt) { return prec == 1 && K0 == 4 && ppt == 1; }

// Shared memory of the z pass for a CTA with ppt points per thread (1 or 2).
inline size_t zpass_smem(int prec, int K0, int ppt, int nt) {
  const size_t pts = (size_t)nt * ppt;
  const size_t rb = prec == 0 ? 8 : 4;
  const size_t kk = 3 * K0 - 1;
  const size_t nbuf = (size_t)zpass_nb(prec, ppt) * pts;
  const size_t bufb = prec == 0 ? 16 * padded_elems<double>(nbuf) : 8 * padded_elems<float>(nbuf);
  // FP32 prefetch buffers, starting on the next 16-byte boundary (bulk-copy destinations)
  const size_t stage = prec == 0 ? 0 : 2 * 2 * (size_t)zpass_nb(prec, ppt) * pts * 8 + 16;
  return bufb + rb * kk * pts + (zpass_smem_acc(prec, ppt) ? rb * kk * pts : 0) + stage +
         (zpass_pingpong(prec, K0, ppt) ? bufb : 0);
}

// Batched FP32 z pass (mwf_zbatch.cuh): every transform of a work item of L x lines and all
// three z-subsets in one batch, for the z line lengths with compile-time two-stage plans.  A
// CTA may use at most zb_smem_budget(b) bytes of dynamic shared memory when b CTAs share an SM
// (228 KB per SM, 1 KB of it reserved per CTA; at most 227 KB for one CTA).
#ifndef MWF_ZB_THREADS
#define MWF_ZB_THREADS 256
#endif
constexpr int kZbThreads = MWF_ZB_THREADS;
__host__ __device__ constexpr size_t zb_smem_budget(int blocks) {
  return blocks <= 1 ? (size_t)232448 : (size_t)233472 / blocks - 1024;
}
bool zb_supported(int K0, int Q);            // a kernel exists and one line fits one CTA
int zb_blocks_per_sm(int K0, int Q);         // CTAs per SM the kernel is compiled for
size_t zb_smem(int K0, int Q, int L);
int sm_count();                               // SMs of the current device        // dynamic shared memory of an item of L lines
cudaError_t launch_z_batched(int K0, int Q, const RunDesc* runs, const WorkItem* items, int n, size_t smem,
                             int* err, cudaStream_t st);

// FP32 x passes with the lines split into three subsets of length MM (mwf_xbatch.cuh), for the
// MM with compile-time two-stage plans: CTAs of kXbThreads threads, kXfBlocks (x forward) and
// kXiBlocks (x inverse) of them per SM.
constexpr int kXbThreads = 256;
#ifndef MWF_XF_BLOCKS
#define MWF_XF_BLOCKS 3
#endif
#ifndef MWF_XI_BLOCKS
#define MWF_XI_BLOCKS 4
#endif
constexpr int kXfBlocks = MWF_XF_BLOCKS;
constexpr int kXiBlocks = MWF_XI_BLOCKS;
bool xb_supported(int MM);
size_t xbf_smem(int MM, int nb);             // x forward item of nb columns (u_k, v_k, w_k of one mode k)
size_t xbi_smem(int MM, int nb);             // x inverse item of nb columns (one wall-normal mode)
cudaError_t launch_x_forward_batched(int MM, const RunDesc* runs, const WorkItem* items, int n, size_t smem,
                                     int* err, cudaStream_t st);
cudaError_t launch_x_inverse_batched(int MM, const RunDesc* runs, const WorkItem* items, int n, size_t smem,
                                     int* err, cudaStream_t st);

// Persistent FP32 step (mwf_persist.cuh): the passes of every run with batched forms of all
// three, in one launch of kZbThreads-thread CTAs taking items from a ticket counter.  Items are
// PersistItem; counters has 1 + 2 n_runs ints and must be zero at launch.  persistent_grid: how
// many CTAs with `smem` bytes of dynamic shared memory the device holds at once (-1 on error).
int persistent_grid(size_t smem);
cudaError_t launch_persistent_step(const RunDesc* runs, const void* items, int n_items, int* counters, size_t smem,
                                   int grid, int* err, cudaStream_t st);

// Physical-field z transform (one line of length Z <= kPhysVpt * kPhysThreads per CTA).
constexpr int kPhysThreads = 256;
constexpr int kPhysVpt = 12;

// Shared memory of an x pass holding n complex elements (padded layout).
inline size_t xpass_smem(int prec, size_t n) {
  return prec == 0 ? 16 * padded_elems<double>(n) : 8 * padded_elems<float>(n);
}

#define MWF_DECLARE_LAUNCHERS(SUF)                                                                   \
  cudaError_t launch_x_forward_##SUF(int nt, const RunDesc* runs, const WorkItem* items, int n,      \
                                     size_t smem, int* err, cudaStream_t st);                        \
  cudaError_t launch_z_nonlinear_##SUF(int K0, int ppt, int nt, const RunDesc* runs,                  \
                                       const WorkItem* items,                                         \
                                       int n, size_t smem, int* err, cudaStream_t st);               \
  cudaError_t launch_z_diag_##SUF(int K0, int ppt, int nt, const RunDesc* runs, const WorkItem* items,  \
                                  int n, size_t smem, int* err, cudaStream_t st);                    \
  cudaError_t launch_x_inverse_##SUF(int nt, const RunDesc* runs, const WorkItem* items, int n,      \
                                     size_t smem, int* err, cudaStream_t st);                        \
  cudaError_t launch_energy_##SUF(const RunDesc* runs, int run, double* partial, int nparts,         \
                                  double* out, cudaStream_t st);                                     \
  cudaError_t launch_ref_to_dev_##SUF(const double* re, const double* im, void* out, int K, int M,   \
                                      int NN, cudaStream_t st);                                      \
  cudaError_t launch_dev_to_ref_##SUF(const void* in, double* re, double* im, int K, int M, int NN,  \
                                      cudaStream_t st);                                              \
  cudaError_t launch_imposesym_##SUF(const RunDesc* runs, int run, int mode, int M, int NN,          \
                                     cudaStream_t st);                                               \
  cudaError_t launch_nonfinite_##SUF(const RunDesc* runs, int run, int* flag, cudaStream_t st);    \
  cudaError_t launch_phys_z_##SUF(const RunDesc* runs, int run, int X, int KK, const FftPlanDev& planZ, \
                                  size_t smem, double* out, int* err, cudaStream_t st);              \
  cudaError_t launch_spectrum_##SUF(const RunDesc* runs, int run, int M, int NN,                     \
                                    unsigned long long* mx, cudaStream_t st);                        \
  cudaError_t launch_probes_##SUF(const RunDesc* runs, int run, int K0, int NN, double2* g,          \
                                  const int* zs, int nprobe, double* out, cudaStream_t st);          \
  cudaError_t launch_remap_x_##SUF(const RunDesc* runs, int run, const void* src, size_t elems,      \
                                   int factor, cudaStream_t st);                                     \
  cudaError_t launch_blend_##SUF(const RunDesc* runs, int run, int other, size_t elems, double d,    \
                                 cudaStream_t st);                                                   \
  cudaError_t launch_noise_##SUF(const RunDesc* runs, int run, size_t elems, double scale,           \
                                 unsigned long long seed, cudaStream_t st);                         \
  cudaError_t launch_spec_x_backward_##SUF(const RunDesc* runs, int run, int X, int KK, int NN,       \
                                           const void* sp, int* err, cudaStream_t st);                \
  cudaError_t launch_phys_z_forward_##SUF(const RunDesc* runs, int run, int X, int KK, int Z,         \
                                          const FftPlanDev& planZ, const double* ph, int* err,        \
                                          cudaStream_t st);                                           \
  cudaError_t launch_spec_x_forward_##SUF(const RunDesc* runs, int run, int X, int KK, int NN, void* sp, \
                                          int* err, cudaStream_t st);

MWF_DECLARE_LAUNCHERS(f64)
constexpr int kFmaChains = 8;
// which = 0: FP64 FMA chains, 1: FP32 (defined in kernels_f64.cu)
cudaError_t launch_fma_probe(int which, int blocks, int threads, int iters, void* out, cudaStream_t st);
MWF_DECLARE_LAUNCHERS(f32)

}  // namespace mwf
