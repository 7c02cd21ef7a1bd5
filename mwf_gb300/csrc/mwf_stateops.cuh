// Device kernels of the state operations and diagnostics outside the timestep: the physical
// field of vel_mpt2phys, spectrum maxima (io_save_Uspec), velocity probes (vel_history),
// x-resolution remapping (var_doubleX / var_quadX), state blending (utils/interpstate.f90)
// and additive noise (var_randadd).
#pragma once
#include "mwf_kernels.cuh"

namespace mwf {

// ---------------------------------------------------------------------------------------
// Physical field, z direction (tra_spec2phys, transform.fftw5.f90:64-87, second half).
// Input: the x-forward output T[f][x][n] of the KK perturbation fields (no base flow).
// One CTA per (x line, field pair): the c2r of length Z of two real fields runs as one
// complex transform of their Hermitian extensions, a_f + i a_g; the real part of the result
// is field f and the imaginary part field g.  As FFTW's c2r, only the real part of the
// n = 0 coefficient enters.  Output in the reference's phys order (KK, 0:Z-1, 0:X-1):
// out[(x * Z + z) * KK + f], FP64.
// ---------------------------------------------------------------------------------------
template <typename T, int VPT, int NT>
__global__ void __launch_bounds__(NT) phys_z_kernel(const RunDesc* __restrict__ runs, int run, FftPlanDev planZ,
                                                     double* __restrict__ out, int* err) {
  using C = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const RunDesc& R = runs[run];
  const int X = R.X, Z = R.Z, NN = R.NN, KK = R.KK;
  const int npairs = (KK + 1) / 2;
  const int x = blockIdx.x / npairs;
  const int f = 2 * (blockIdx.x - x * npairs);
  const bool two = f + 1 < KK;
  if (Z > VPT * NT) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_FFT_CAPACITY);
    return;
  }
  const C* __restrict__ Tin = reinterpret_cast<const C*>(R.T);
  const C* __restrict__ la = Tin + ((size_t)f * X + x) * NN;
  const C* __restrict__ lb = Tin + ((size_t)(f + 1) * X + x) * NN;
  for (int z = threadIdx.x; z < Z; z += NT) buf[pad_idx<T>(z)] = mk<T>(T(0), T(0));
  __syncthreads();
  for (int n = threadIdx.x; n < NN; n += NT) {
    const C a = la[n];
    const C b = two ? lb[n] : mk<T>(T(0), T(0));
    // stored conjugated: the backward transform runs as conj(forward(conj(.)))
    if (n == 0) {
      buf[pad_idx<T>(0)] = mk<T>(a.x, -b.x);
    } else {
      buf[pad_idx<T>(n)] = cconj(mk<T>(a.x - b.y, a.y + b.x));          // a + i b
      buf[pad_idx<T>(Z - n)] = cconj(mk<T>(a.x + b.y, b.x - a.y));      // conj(a) + i conj(b)
    }
  }
  __syncthreads();
  fft_lines_inl<T, VPT, kXMaxRadix<T>>(buf, 0, 1, Z, planZ, reinterpret_cast<const C*>(R.twZ), false, err);
  double* o = out + (size_t)x * Z * KK;
  for (int z = threadIdx.x; z < Z; z += NT) {
    const C v = buf[pad_idx<T>(z)];
    o[(size_t)z * KK + f] = (double)v.x;
    if (two) o[(size_t)z * KK + f + 1] = -(double)v.y;
  }
}

// ---------------------------------------------------------------------------------------
// The stand-alone 2D transforms of the transform module (mwf_spec2phys / mwf_phys2spec), on
// fields the caller supplies.  Spectral fields are held as sp[n][f][ms] (f < KK, slot ms < M),
// x-transformed ones as W[f][x][n] (the layout of RunDesc::T).
// tra_spec2phys x part (transform.fftw5.f90:64-78): one CTA per (field f, column n); the line
// x = m mod X holds the coefficient of m for |m| <= MM-1 and zero elsewhere and is transformed
// backward (e^{+i}, unnormalised) as conj(forward(conj .)).  The z part is phys_z_kernel.
// ---------------------------------------------------------------------------------------
template <typename T, int VPT, int NT>
__global__ void __launch_bounds__(NT) spec_x_backward_kernel(const RunDesc* __restrict__ runs, int run,
                                                             const cx<T>* __restrict__ sp, int* err) {
  using C = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const RunDesc& R = runs[run];
  const int X = R.X, NN = R.NN, KK = R.KK, M = R.M, MM = R.MM;
  const int f = blockIdx.x / NN;
  const int n = blockIdx.x - f * NN;
  if (X > VPT * NT) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_FFT_CAPACITY);
    return;
  }
  for (int x = threadIdx.x; x < X; x += NT) buf[pad_idx<T>(x)] = mk<T>(T(0), T(0));
  __syncthreads();
  const C* __restrict__ row = sp + ((size_t)n * KK + f) * M;
  for (int ms = threadIdx.x; ms < M; ms += NT) {
    const int m = signed_m(ms, MM, M);
    buf[pad_idx<T>(m < 0 ? m + X : m)] = cconj(row[ms]);
  }
  __syncthreads();
  fft_lines_inl<T, VPT, kXMaxRadix<T>>(buf, 0, 1, X, R.planX, reinterpret_cast<const C*>(R.twX), false, err);
  C* __restrict__ W = reinterpret_cast<C*>(R.T);
  for (int x = threadIdx.x; x < X; x += NT) W[((size_t)f * X + x) * NN + n] = cconj(buf[pad_idx<T>(x)]);
}

// tra_phys2spec z part (transform.fftw5.f90:126-135): one CTA per (x line, pair of fields);
// the two real fields scaled by 1/(XZ) (as the reference scales before its r2c) form one complex
// line, transformed forward; the spectra of the two fields at n < NN are
// (Y[n] + conj Y[Z-n]) / 2 and (Y[n] - conj Y[Z-n]) / (2i).
template <typename T, int VPT, int NT>
__global__ void __launch_bounds__(NT) phys_z_forward_kernel(const RunDesc* __restrict__ runs, int run, FftPlanDev planZ,
                                                            const double* __restrict__ ph, int* err) {
  using C = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const RunDesc& R = runs[run];
  const int X = R.X, Z = R.Z, NN = R.NN, KK = R.KK;
  const int npairs = (KK + 1) / 2;
  const int x = blockIdx.x / npairs;
  const int f = 2 * (blockIdx.x - x * npairs);
  const bool two = f + 1 < KK;
  if (Z > VPT * NT) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_FFT_CAPACITY);
    return;
  }
  const T sc = T(R.scale);
  const double* __restrict__ line = ph + (size_t)x * Z * KK;
  for (int z = threadIdx.x; z < Z; z += NT) {
    const T a = T(line[(size_t)z * KK + f]) * sc;
    const T b = two ? T(line[(size_t)z * KK + f + 1]) * sc : T(0);
    buf[pad_idx<T>(z)] = mk<T>(a, b);
  }
  __syncthreads();
  fft_lines_inl<T, VPT, kXMaxRadix<T>>(buf, 0, 1, Z, planZ, reinterpret_cast<const C*>(R.twZ), false, err);
  C* __restrict__ W = reinterpret_cast<C*>(R.T);
  for (int n = threadIdx.x; n < NN; n += NT) {
    const C y = buf[pad_idx<T>(n)];
    const C yq = buf[pad_idx<T>(n == 0 ? 0 : Z - n)];
    W[((size_t)f * X + x) * NN + n] = mk<T>(T(0.5) * (y.x + yq.x), T(0.5) * (y.y - yq.y));
    if (two) W[((size_t)(f + 1) * X + x) * NN + n] = mk<T>(T(0.5) * (y.y + yq.y), T(0.5) * (yq.x - y.x));
  }
}

// tra_phys2spec x part (transform.fftw5.f90:136-144): one CTA per (field f, column n); the line
// W[f][x][n] over x is transformed forward and the kept wavenumbers |m| <= MM-1 are written to
// sp[n][f][ms].
template <typename T, int VPT, int NT>
__global__ void __launch_bounds__(NT) spec_x_forward_kernel(const RunDesc* __restrict__ runs, int run,
                                                            cx<T>* __restrict__ sp, int* err) {
  using C = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const RunDesc& R = runs[run];
  const int X = R.X, NN = R.NN, KK = R.KK, M = R.M, MM = R.MM;
  const int f = blockIdx.x / NN;
  const int n = blockIdx.x - f * NN;
  if (X > VPT * NT) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_FFT_CAPACITY);
    return;
  }
  const C* __restrict__ W = reinterpret_cast<const C*>(R.T);
  for (int x = threadIdx.x; x < X; x += NT) buf[pad_idx<T>(x)] = W[((size_t)f * X + x) * NN + n];
  __syncthreads();
  fft_lines_inl<T, VPT, kXMaxRadix<T>>(buf, 0, 1, X, R.planX, reinterpret_cast<const C*>(R.twX), false, err);
  C* __restrict__ row = sp + ((size_t)n * KK + f) * M;
  for (int ms = threadIdx.x; ms < M; ms += NT) {
    const int m = signed_m(ms, MM, M);
    row[ms] = buf[pad_idx<T>(m < 0 ? m + X : m)];
  }
}

// ---------------------------------------------------------------------------------------
// Spectrum maxima (io_save_Uspec, io.f90:345-372): for every (m, n) the largest modulus
// sqrt(re^2 + im^2) over the KK spectral coefficients of u, v, w (no base flow); folded
// into mx[0..MM-1] by |m| and mx[MM..MM+NN-1] by n.  The moduli are non-negative, so their
// bit patterns order like the values and one 64-bit atomicMax keeps each maximum.
// Grid: (ceil(M / 256), ceil(NN / kSpecRows)); one thread per column slot m.
// ---------------------------------------------------------------------------------------
constexpr int kSpecRows = 16;

template <typename T>
__global__ void __launch_bounds__(256) spectrum_kernel(const RunDesc* __restrict__ runs, int run,
                                                        unsigned long long* mx) {
  using C = cx<T>;
  const RunDesc& R = runs[run];
  const C* __restrict__ c = reinterpret_cast<const C*>(R.c);
  const int M = R.M, MM = R.MM, NN = R.NN, KK = R.KK;
  const int ms = blockIdx.x * 256 + threadIdx.x;
  const int n0 = blockIdx.y * kSpecRows;
  const bool live = ms < M;
  const int m = live ? signed_m(ms, MM, M) : 0;
  double mcol = 0.0;
  for (int r = 0; r < kSpecRows && n0 + r < NN; ++r) {
    const int n = n0 + r;
    double d = 0.0;
    if (live) {
      for (int fs = 0; fs < KK; ++fs) {
        const C v = mpt_to_field<T>(R, c, fs, m, n, false);
        const double re = (double)v.x, im = (double)v.y;
        d = fmax(d, sqrt(__dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im))));
      }
    }
    mcol = fmax(mcol, d);
    for (int o = 16; o > 0; o >>= 1) d = fmax(d, __shfl_xor_sync(0xffffffffu, d, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&mx[MM + n], (unsigned long long)__double_as_longlong(d));
  }
  if (live) atomicMax(&mx[m < 0 ? -m : m], (unsigned long long)__double_as_longlong(mcol));
}

// ---------------------------------------------------------------------------------------
// Velocity probes (vel_history, velocity.f90:164-180), step 1: g[f][n] = sum over the live
// x slots m of the spectral coefficient, the x transform evaluated at x = 0.
// One CTA per n; thread-strided over m, then a warp + shared-memory reduction per field.
// ---------------------------------------------------------------------------------------
template <typename T, int KK>
__global__ void __launch_bounds__(256) probe_sum_kernel(const RunDesc* __restrict__ runs, int run,
                                                         double2* __restrict__ g) {
  using C = cx<T>;
  const RunDesc& R = runs[run];
  const C* __restrict__ c = reinterpret_cast<const C*>(R.c);
  const int M = R.M, MM = R.MM, NN = R.NN;
  const int n = blockIdx.x;
  double ar[KK], ai[KK];
#pragma unroll
  for (int f = 0; f < KK; ++f) { ar[f] = 0.0; ai[f] = 0.0; }
  for (int ms = threadIdx.x; ms < M; ms += 256) {
    const int m = signed_m(ms, MM, M);
#pragma unroll
    for (int f = 0; f < KK; ++f) {
      const C v = mpt_to_field<T>(R, c, f, m, n, false);
      ar[f] += (double)v.x;
      ai[f] += (double)v.y;
    }
  }
  __shared__ double2 red[KK][8];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int f = 0; f < KK; ++f) {
    double a = ar[f], b = ai[f];
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) red[f][w] = make_double2(a, b);
  }
  __syncthreads();
  if (threadIdx.x < KK) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < 8; ++i) { a += red[threadIdx.x][i].x; b += red[threadIdx.x][i].y; }
    g[(size_t)threadIdx.x * NN + n] = make_double2(a, b);
  }
}

// Step 2: one warp per (probe j, field f): the c2r of length Z at z = zs[j],
// Re g(0) + 2 sum_{n >= 1} Re(g(n) e^{+2 pi i n z / Z}), with the twiddles of the transforms.
template <typename T>
__global__ void __launch_bounds__(256) probe_eval_kernel(const RunDesc* __restrict__ runs, int run,
                                                          const double2* __restrict__ g, const int* __restrict__ zs,
                                                          int nprobe, double* __restrict__ out) {
  using C = cx<T>;
  const RunDesc& R = runs[run];
  const int NN = R.NN, Z = R.Z, KK = R.KK;
  const int wid = (blockIdx.x * 256 + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (wid >= nprobe * KK) return;
  const int j = wid / KK, f = wid - j * KK;
  const long long z = zs[j];
  const C* __restrict__ twZ = reinterpret_cast<const C*>(R.twZ);
  const double2* __restrict__ gf = g + (size_t)f * NN;
  double s = 0.0;
  for (int n = 1 + lane; n < NN; n += 32) {
    const C w = twZ[(int)(((long long)n * z) % Z)];             // e^{-2 pi i n z / Z}
    const double2 a = gf[n];
    s += a.x * (double)w.x + a.y * (double)w.y;                  // Re(a * conj(w))
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[(size_t)j * KK + f] = gf[0].x + 2.0 * s;
}

// ---------------------------------------------------------------------------------------
// x-resolution remap (var_quadX, variables.f90:168-185, and var_doubleX 147-165 with the
// same mirror rule): the coefficient of x wavenumber m moves to factor*m.  Written as a
// gather into c from the copy src of the old state, in the reference's scatter order: slot
// mm <= MM-1 takes m = mm/factor when factor divides mm; slot mm > MM-1 takes the negative
// m with M - factor*(M - m) = mm.  The reference keeps negative targets down to slot MM-1
// (its test is mm < MM-1), so for factor > 1 and MM divisible by factor the wavenumber
// -MM lands in slot MM-1 and, coming later in the loop, overwrites the positive mode there.
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void remap_x_kernel(const RunDesc* __restrict__ runs, int run, const cx<T>* __restrict__ src,
                               int factor) {
  using C = cx<T>;
  const RunDesc& R = runs[run];
  C* __restrict__ c = reinterpret_cast<C*>(R.c);
  const int M = R.M, MM = R.MM, K = R.K;
  const size_t tot = (size_t)R.NN * K * M;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int mm = (int)(e % M);
    const size_t row = e / M;                     // n * K + k
    int from = -1;
    if (mm >= MM - 1 && (M - mm) % factor == 0) from = M - (M - mm) / factor;
    if (from < 0 && mm <= MM - 1 && mm % factor == 0) from = mm / factor;
    c[e] = from >= 0 ? src[row * M + from] : mk<T>(T(0), T(0));
  }
}

// State blend (utils/interpstate.f90:32-33): c := (1 - d) c + d c_other, rounded per
// operation as written (no fused multiply-add).
template <typename T>
__global__ void blend_kernel(const RunDesc* __restrict__ runs, int run, int other, double d) {
  using C = cx<T>;
  C* __restrict__ c = reinterpret_cast<C*>(runs[run].c);
  const C* __restrict__ o = reinterpret_cast<const C*>(runs[other].c);
  const size_t tot = (size_t)runs[run].NN * runs[run].K * runs[run].M;
  const double e = __dadd_rn(1.0, -d);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const C a = c[i], b = o[i];
    c[i] = mk<T>(T(__dadd_rn(__dmul_rn(e, (double)a.x), __dmul_rn(d, (double)b.x))),
                 T(__dadd_rn(__dmul_rn(e, (double)a.y), __dmul_rn(d, (double)b.y))));
  }
}

// Additive noise (var_randadd, variables.f90:253-269): every coefficient with m != 0 and
// n != 0 gets scale * r added to its real and its imaginary part, r uniform in [0, 1).
// The reference draws r from Fortran's RANDOM_NUMBER; here r comes from SplitMix64
// (Steele, Lea and Flood, OOPSLA 2014) of (seed, 2e) and (seed, 2e + 1), e the element's
// index in the reference order (k fastest, then m, then n), as the top 53 bits.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__device__ __forceinline__ double noise_u01(unsigned long long seed, unsigned long long i) {
  return (double)(splitmix64(seed ^ splitmix64(i)) >> 11) * 0x1.0p-53;
}

template <typename T>
__global__ void noise_kernel(const RunDesc* __restrict__ runs, int run, double scale, unsigned long long seed) {
  using C = cx<T>;
  const RunDesc& R = runs[run];
  C* __restrict__ c = reinterpret_cast<C*>(R.c);
  const int M = R.M, K = R.K;
  const size_t tot = (size_t)R.NN * K * M;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int m = (int)(e % M);
    const size_t row = e / M;
    const int n = (int)(row / K);
    const int k = (int)(row - (size_t)n * K);
    if (m == 0 || n == 0) continue;
    const unsigned long long ref = ((unsigned long long)n * M + m) * K + k;
    C v = c[e];
    v.x = T(__dadd_rn((double)v.x, __dmul_rn(scale, noise_u01(seed, 2 * ref))));
    v.y = T(__dadd_rn((double)v.y, __dmul_rn(scale, noise_u01(seed, 2 * ref + 1))));
    c[e] = v;
  }
}

}  // namespace mwf
