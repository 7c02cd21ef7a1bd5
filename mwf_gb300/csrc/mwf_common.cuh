// Shared device/host definitions for the MWF timestep kernels (sm_103a).
//
// Device layouts of one run (all interleaved complex, "m" = x-wavenumber slot 0..M-1 with
// slots > MM-1 holding negative m, exactly as the reference's spectral arrays):
//   c, onl   cx<T>[NN][K][M]     MPT state and previous nonlinear term (AB2 history)
//   inv_lhs, rhs  double[NN][K][M]  FP64 implicit-update tables (1/lhs and rhs); FP32 runs
//                 hold float tables of A = rhs/lhs (hi, lo) and B = (dt/2)/lhs there (RunDesc)
//   T        cx<T>[2KK][X][NN]   x-transformed u,v,w (KK fields) and d/dx of them (KK)
//   NLT      cx<T>[KK][X][NN]    z-transformed nonlinear term, before the inverse x pass
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define MWF_MAX_STAGES 16

template <typename T> struct CxOf;
template <> struct CxOf<double> { using type = double2; };
template <> struct CxOf<float> { using type = float2; };
template <typename T> using cx = typename CxOf<T>::type;

template <typename T> __host__ __device__ __forceinline__ cx<T> mk(T a, T b) {
  cx<T> r; r.x = a; r.y = b; return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {
  C r; r.x = a.x * b.x + a.y * b.y; r.y = a.y * b.x - a.x * b.y; return r;
}
// FP32: the roundings spelled out (a fused multiply-add over one rounded product), so that every
// kernel inlining the same item code rounds alike, whatever contraction the compiler would pick
// in its context (the per-pass and the persistent FP32 kernels are compared bitwise).
template <> __device__ __forceinline__ float2 cmul<float2>(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)), __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x)));
}
template <> __device__ __forceinline__ float2 cmulc<float2>(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, __fmul_rn(a.y, b.y)), __fmaf_rn(a.y, b.x, -__fmul_rn(a.x, b.y)));
}
template <typename C> __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }

// Division by a runtime divisor 1 <= d <= 2^16 of dividends 0 <= b < 2^16:
// q = umulhi(b, ceil(2^32 / d)) is exact in that range (the rounding error of the
// reciprocal times b stays below 2^-16 <= 1/d).  All index divisions of the passes fall in
// it (dividends are bounded by a CTA's element count, at most 18 * 512).
struct FastDiv {
  unsigned m;
  int d;
  __device__ __forceinline__ int div(int b) const { return d == 1 ? b : (int)__umulhi((unsigned)b, m); }
};
// ceil(2^32 / d) for d >= 2 is floor((2^32 - 1) / d) + 1: a 32-bit division (a 64-bit one is
// a long software sequence on the device, and kernels build their divisors per thread).
__host__ __device__ inline FastDiv make_fastdiv(int d) {
  FastDiv f;
  f.d = d;
  f.m = d == 1 ? 0u : 0xFFFFFFFFu / (unsigned)d + 1u;
  return f;
}

// Mixed-radix Stockham plan for one line length N = 2^a 3^b.
struct FftPlanDev {
  int N;
  int nst;
  int radix[MWF_MAX_STAGES];
  int ns[MWF_MAX_STAGES];       // product of the radices of the earlier stages
  FastDiv fnb[MWF_MAX_STAGES];  // division by N / radix
  FastDiv fns[MWF_MAX_STAGES];  // division by ns
};

// Shared-memory index of element i of an FFT buffer: one pad element after every 128
// bytes, so the radix-R strided accesses of the Stockham stages spread over all banks.
template <typename T>
__host__ __device__ __forceinline__ int pad_idx(int i) { return i + (i >> (sizeof(T) == 8 ? 3 : 4)); }
template <typename T>
__host__ __device__ inline size_t padded_elems(size_t n) { return n + (n >> (sizeof(T) == 8 ? 3 : 4)) + 1; }

// Wavenumber tables of the FP64 x-forward pass (static shared memory): x positions (the
// longest x line) and columns; the host planner leaves room for them in the tile choice.
constexpr int kXTabLen = 4096;
constexpr int kXTabCols = 64;
constexpr size_t kXTabBytes = (size_t)(kXTabLen + kXTabCols) * 8;

// Per-run descriptor, resident in device memory.
struct RunDesc {
  int K0, MM, NN, M, X, Z, K, KK;
  int prec;                     // 0 = FP64, 1 = FP32
  int xf_nb;                    // columns n per x-forward work item
  int xi_nb;                    // columns n per x-inverse work item
  int z_lx;                     // x lines per z-pass work item
  int z_sum;                    // 1: each z item runs the three z-subsets of its lines and sums
                                // their outputs into the first NLT partial (FP32); 0: one subset per item
  int zb_lx;                    // x lines per item of the batched FP32 z pass (0: the run uses
                                // z_nonlinear_kernel)
  int xbf_nb, xbi_nb;           // columns per item of the subset-split FP32 x passes (0: the run
                                // uses x_forward_kernel / x_inverse_kernel)
  int xbf_items, zb_items;      // the run's x-forward and z items per step (persistent step waits)
  double alpha, gamma, dt, cth, sth, scale;
  float alpha_f, gamma_f;       // FP32 copies for the FP32 kernels (no FP64 instructions there)
  void* c;
  void* onl;
  // Implicit-update tables, computed in FP64 on the host.  FP64 runs: 1/lhs and rhs as double.
  // FP32 runs: the update is c' = A c + B (3 nl - onl); the 1/lhs slot holds A = rhs/lhs as
  // two float arrays (hi, then lo = A - hi), the rhs slot B = (dt/2)/lhs as float.
  const double* inv_lhs;
  const double* rhs;
  void* T;
  void* NLT;
  const void* twX;              // e^{-2 pi i t / X}, t < X
  const void* twQ;              // e^{-2 pi i t / NN}
  const void* twZ;              // e^{-2 pi i t / Z}
  int* nst;                     // 1 -> next step is the Euler start (reference nst flag)
  int active;                   // 0 -> the passes skip this run (a finished request)
  // Test only (mwf_test_copy_timeout): the FP32 z pass of z_nonlinear_kernel arms each staging
  // barrier with this many bytes more than its copies carry, and waits at most test_wait_ns
  // (0: about a second) for a barrier phase, so its bounded wait runs out on purpose.
  unsigned test_tx_extra;
  unsigned long long test_wait_ns;
  double diag_ct;               // threshold of the physical-space diagnostic
  FftPlanDev planX, planQ;
};

// One CTA's share of a pass.
struct WorkItem {
  int run;
  int a;   // x-forward / x-inverse: first column n;  z-pass: first x line
  int b;   // x-forward: field (0..2KK-1); x-inverse: wall-normal mode k (0..K0-1); z: subset
           // 0..2, or 3 = all three summed (runs with z_sum)
  int pad; // x-forward: 1 = without the laminar base flow (diagnostics)
};

// One item of the persistent FP32 step (mwf_persist.cuh): a pass work item and its kind and size,
// code = kind << 8 | size index (kinds: 0 x forward, 1 z pass of M4, 2 z pass of M6, 3 x inverse;
// size index of MM or NN in {32, 48, 64, 96, 128, 192, 256}).
struct PersistItem {
  int run, a, b, code;
};

// Device-side error bits (the kernels never trap; they record and skip).
enum {
  MWF_DERR_FFT_CAPACITY = 1,
  MWF_DERR_OUTPUT_CAPACITY = 2,
  MWF_DERR_BAD_RADIX = 4,
  MWF_DERR_COPY_TIMEOUT = 8,   // a bulk copy into shared memory did not complete within the wait limit
  MWF_DERR_WAIT_TIMEOUT = 16,  // a persistent-step item waited for its prerequisites past the limit
};
