// The three passes of one MWF timestep (sm_103a), templated on the arithmetic type T
// (double for the plain FP64 path, float for the FP32 path) and on K0 (4 = M4, 6 = M6).
//
//   x_forward : MPT state -> u,v,w and d/dx u,v,w (var_mpt2spec + vel_addlam +
//               var_spec_grad, variables.f90:390-434,600-612, velocity.f90:76-82), padded
//               to 3MM and transformed in x (tra_spec2phys x part, transform.fftw5.f90:69-78)
//   z_nonlinear : c2r in z of u, du/dx, du/dz (transform.fftw5.f90:80-85), the pointwise
//               Galerkin u.grad(u) (modes.M4.f90:14-28 / modes.M6.f90:14-20), r2c in z and
//               truncation (transform.fftw5.f90:126-135) -- physical fields stay on chip
//   x_inverse : inverse x transform + truncation (transform.fftw5.f90:136-144), curl /
//               curl-curl projection to MPT (var_spec2mpt, variables.f90:440-480) and the
//               AB2 / implicit update (vel_TS, velocity.f90:21-41)
//
// The z pass works on the three interleaved z-subsets z = s + 3q (s = 0,1,2, q < NN)
// separately.  Because only n < NN is non-zero, the c2r restricted to subset s is
// Re(sum_n c_n X_n w^{ns} W_NN^{nq}) (c_0 = 1, c_n = 2, w = e^{2 pi i/Z}), a length-NN
// complex transform; two real fields share one transform through the Hermitian split.
// The r2c output n < NN is sum_s w^{-ns} DFT_NN(subset s)[n], accumulated in place.
#pragma once
#include "mwf_common.cuh"
#include "mwf_fft.cuh"
#include "mwf_launch.h"
#include "nl_gen.cuh"

namespace mwf {

constexpr double kBeta = 1.5707963267948966;   // pi/2, program/parameters.f90:55

// Wavenumbers alpha*m, gamma*n and the wall-normal factor (-1)^k k beta (var_precompute,
// variables.f90:520-532).  The FP64 path forms them in FP64 as the reference's tables do; the
// FP32 path multiplies FP32 copies, so the FP32 kernels issue no FP64 instruction (GB300's
// FP64 pipe runs at 1/64 of FP32 and would otherwise bound them).
template <typename T>
__device__ __forceinline__ T wavenum(double f, float ff, int i) {
  if constexpr (sizeof(T) == 8) return f * i;
  else return ff * (float)i;
}
template <typename T>
__device__ __forceinline__ T kbeta(int k) {
  if constexpr (sizeof(T) == 8) return (k & 1) ? -k * kBeta : k * kBeta;
  else return (float)((k & 1) ? -k : k) * (float)kBeta;
}

template <int K0, typename T, typename P, typename NL>
__device__ __forceinline__ void nl_y(const P& p, NL&& nl) {
  if constexpr (K0 == 4) nl_y_4<T>(p, nl); else nl_y_6<T>(p, nl);
}
template <int K0, int J, typename T, typename P, typename NL>
__device__ __forceinline__ void nl_xz(const P& p, T px, T pz, NL&& nl) {
  if constexpr (K0 == 4) nl_xz_4<J, T>(p, px, pz, nl); else nl_xz_6<J, T>(p, px, pz, nl);
}

// Field index J known only after loop unrolling: the switch folds away once J is constant.
template <int K0, typename T, typename P, typename NL>
__device__ __forceinline__ void nl_xz_rt(int J, const P& p, T px, T pz, NL&& nl) {
#define MWF_CASE(j) case j: if constexpr (j < 3 * K0 - 1) nl_xz<K0, j, T>(p, px, pz, nl); break;
  switch (J) {
    MWF_CASE(0) MWF_CASE(1) MWF_CASE(2) MWF_CASE(3) MWF_CASE(4) MWF_CASE(5) MWF_CASE(6) MWF_CASE(7)
    MWF_CASE(8) MWF_CASE(9) MWF_CASE(10) MWF_CASE(11) MWF_CASE(12) MWF_CASE(13) MWF_CASE(14)
    MWF_CASE(15) MWF_CASE(16)
    default: break;
  }
#undef MWF_CASE
}

// Asynchronous global -> shared copies (cp.async): 8 or 16 bytes per call, grouped and
// waited for with commit/wait_group; the registers are not involved.
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (BYTES == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
  else asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// One-dimensional bulk copies global -> shared through the TMA unit (cp.async.bulk), which
// signal their bytes to an mbarrier: both addresses 16-byte aligned, size a multiple of 16.
// One thread issues a whole task's rows; the others only wait on the barrier's phase.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
// Orders this thread's earlier generic-proxy accesses of shared memory before later bulk copies.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned done;
  asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  return done != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
// Completes `bytes` of the barrier's expected transaction count from this thread (used only
// when a test armed the barrier with more bytes than its copies carry).
__device__ __forceinline__ void mbar_complete_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Waits for the phase of the given parity to complete; false once limit_ns has passed (about a
// second unless a test shortens it; each try_wait suspends the thread for at most a short,
// hardware-chosen time), so a copy that never lands cannot hang the CTA.
constexpr unsigned long long kMbarWaitNs = 1000000000ull;
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity,
                                          unsigned long long limit_ns = kMbarWaitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (global_ns() - t0 < limit_ns)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Largest radix of the transforms (the staging registers of a radix-R stage are R complex
// values per thread): x passes 12 in FP64 and 16 in FP32, z pass 8 in FP64 and 12 in FP32.
// The host planner uses the same caps (mwf_host.cu, make_plan).
template <typename T> constexpr int kXMaxRadix = sizeof(T) == 8 ? 12 : 16;
template <typename T> constexpr int kZMaxRadix = sizeof(T) == 8 ? 8 : 12;

// Signed x wavenumber of slot ms (0..M-1): slots above MM-1 hold m - M.
__device__ __forceinline__ int signed_m(int ms, int MM, int M) { return ms < MM ? ms : ms - M; }

// ---------------------------------------------------------------------------------------
// u,v,w (field f of the KK spectral fields) at (m, n) from the MPT state: the formulas of
// var_mpt2spec with the mean-mode rule and the laminar base flow, in the run's precision.
// ---------------------------------------------------------------------------------------
// Wall-normal index k of spectral field fs (u_k: fs < K0, v_k: next K0-1, w_k: last K0).
__device__ __forceinline__ int field_k(int fs, int K0) {
  return fs < K0 ? fs : (fs < 2 * K0 - 1 ? fs - K0 + 1 : fs - (2 * K0 - 1));
}

// The same with the wavenumbers m1 = alpha m, n1 = gamma n and k1 = (-1)^k k beta supplied by
// the caller (the x-forward pass reads them from per-block tables).
template <typename T>
__device__ __forceinline__ cx<T> mpt_to_field_w(const RunDesc& R, const cx<T>* __restrict__ c,
                                                int fs, int m, int n, bool addlam, T m1, T n1, T k1);

template <typename T>
__device__ __forceinline__ cx<T> mpt_to_field(const RunDesc& R, const cx<T>* __restrict__ c,
                                              int fs, int m, int n, bool addlam) {
  return mpt_to_field_w<T>(R, c, fs, m, n, addlam, wavenum<T>(R.alpha, R.alpha_f, m),
                           wavenum<T>(R.gamma, R.gamma_f, n), kbeta<T>(field_k(fs, R.K0)));
}

template <typename T>
__device__ __forceinline__ cx<T> mpt_to_field_w(const RunDesc& R, const cx<T>* __restrict__ c,
                                                int fs, int m, int n, bool addlam, T m1, T n1, T k1) {
  const int K0 = R.K0, K = R.K, M = R.M;
  int comp, k;
  if (fs < K0) { comp = 0; k = fs; }
  else if (fs < 2 * K0 - 1) { comp = 1; k = fs - K0 + 1; }
  else { comp = 2; k = fs - (2 * K0 - 1); }
  const int ms = m < 0 ? m + M : m;
  const cx<T>* col = c + (size_t)n * K * M;
  T re, im;
  if (m == 0 && n == 0) {
    // mean flows: u_k = psi_k, w_k = phi_k (k >= 1), u_0 = w_0 = 0, v = -phi*0
    re = T(0); im = T(0);
    if (comp == 0 && k >= 1) { cx<T> a = col[(size_t)k * M]; re = a.x; im = a.y; }
    if (comp == 2 && k >= 1) { cx<T> a = col[(size_t)(k + K0 - 1) * M]; re = a.x; im = a.y; }
    if (addlam && k == 1) {
      if (comp == 0) re += T(R.cth);
      if (comp == 2) re += T(R.sth);
    }
    return mk<T>(re, im);
  }
  if (comp == 1) {
    const cx<T> phi = col[(size_t)(k + K0 - 1) * M + ms];
    const T H = -m1 * m1 - n1 * n1;
    re = -phi.x * H;
    im = -phi.y * H;
  } else {
    const cx<T> psi = col[(size_t)k * M + ms];
    const cx<T> phi = (k >= 1) ? col[(size_t)(k + K0 - 1) * M + ms] : mk<T>(T(0), T(0));
    if (comp == 0) {
      re = -(-psi.y * n1 + phi.y * k1 * m1);
      im = -psi.x * n1 + phi.x * k1 * m1;
    } else {
      re = -(psi.y * m1 + phi.y * k1 * n1);
      im = psi.x * m1 + phi.x * k1 * n1;
    }
  }
  return mk<T>(re, im);
}

// FP32 x transforms of the usual runs (X = 3MM for MM = 32 ... 512, 2^a 3^b) with
// compile-time plans, the planner's default radices for FP32; returns false for other lengths.
template <typename T, int NT, int VPT>
__device__ __forceinline__ bool fft_x_fixed(cx<T>* buf, int base, int L, int X, const cx<T>* __restrict__ tw,
                                            int* err) {
  if constexpr (sizeof(T) == 4) {
    switch (X) {
      case 96: fft_lines_fixed<T, 96, 12, 8, 1, NT, VPT>(buf, base, L, tw, err); return true;
      case 144: fft_lines_fixed<T, 144, 12, 12, 1, NT, VPT>(buf, base, L, tw, err); return true;
      case 192: fft_lines_fixed<T, 192, 12, 16, 1, NT, VPT>(buf, base, L, tw, err); return true;
      case 288: fft_lines_fixed<T, 288, 12, 12, 2, NT, VPT>(buf, base, L, tw, err); return true;
      case 384: fft_lines_fixed<T, 384, 12, 8, 4, NT, VPT>(buf, base, L, tw, err); return true;
      case 576: fft_lines_fixed<T, 576, 12, 12, 4, NT, VPT>(buf, base, L, tw, err); return true;
      case 768: fft_lines_fixed<T, 768, 12, 8, 8, NT, VPT>(buf, base, L, tw, err); return true;
      case 1152: fft_lines_fixed<T, 1152, 12, 12, 8, NT, VPT>(buf, base, L, tw, err); return true;
      case 1536: fft_lines_fixed<T, 1536, 12, 16, 8, NT, VPT>(buf, base, L, tw, err); return true;
      default: break;
    }
  }
  return false;
}

// FP32 z lines (Q = NN) with compile-time plans; the two-stage ones run out of place through
// buf2 when PP (one barrier per stage).  Returns false for other lengths.
template <typename T, int NT, int VPT, bool PP>
__device__ __forceinline__ bool fft_z_fixed(cx<T>* buf, cx<T>* buf2, int L, int Q, const cx<T>* __restrict__ tw,
                                            int* err) {
#define MWF_Z2(N, R1, R2)                                                        \
  case N:                                                                        \
    if constexpr (PP) fft_lines_fixed_pp<T, N, R1, R2, NT, VPT>(buf, buf2, 0, L, tw, err); \
    else fft_lines_fixed<T, N, R1, R2, 1, NT, VPT>(buf, 0, L, tw, err);          \
    return true;
  switch (Q) {
    MWF_Z2(32, 8, 4)
    MWF_Z2(48, 12, 4)
    MWF_Z2(64, 8, 8)
    MWF_Z2(96, 12, 8)
    MWF_Z2(128, 16, 8)
    MWF_Z2(192, 12, 16)
    MWF_Z2(256, 16, 16)
    case 384: fft_lines_fixed<T, 384, 12, 8, 4, NT, VPT>(buf, 0, L, tw, err); return true;
    case 512: fft_lines_fixed<T, 512, 8, 8, 8, NT, VPT>(buf, 0, L, tw, err); return true;
    default: return false;
  }
#undef MWF_Z2
}

// ---------------------------------------------------------------------------------------
// Pass 1: x forward.  Work item = (run, first column n0, field f in 0..2KK-1).
// ---------------------------------------------------------------------------------------
template <typename T, int VPT, int NT>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 1024 / NT : 512 / NT) x_forward_kernel(const RunDesc* __restrict__ runs, const WorkItem* __restrict__ items,
                                 int* err) {
  using C = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const WorkItem wi = items[blockIdx.x];
  const RunDesc& R = runs[wi.run];
  if (!R.active) return;
  const int X = R.X, MM = R.MM, NN = R.NN, KK = R.KK;
  const int n0 = wi.a;
  const int nb = min(R.xf_nb, NN - n0);
  const int f = wi.b;
  const bool deriv = f >= KK;
  const int fs = deriv ? f - KK : f;
  const C* __restrict__ c = reinterpret_cast<const C*>(R.c);
  const int S = X;
  const FastDiv fX = make_fastdiv(X), fNB = make_fastdiv(nb);
  // FP64: the block's wavenumbers alpha m (per x position) and gamma n (per column) go to
  // shared-memory tables first, so the fill spends the FP64 pipe, which bounds this pass, on the
  // field formulas alone (same products as computed in place: the results are identical)
  constexpr bool kTab = sizeof(T) == 8;
  __shared__ T mtab[kTab ? kXTabLen : 1];
  __shared__ T ntab[kTab ? kXTabCols : 1];
  const bool tab = kTab && X <= kXTabLen && nb <= kXTabCols;
  if (tab) {
    for (int x = threadIdx.x; x < X; x += blockDim.x)
      mtab[x] = wavenum<T>(R.alpha, R.alpha_f, x < MM ? x : (x > X - MM ? x - X : 0));
    for (int l = threadIdx.x; l < nb; l += blockDim.x) ntab[l] = wavenum<T>(R.gamma, R.gamma_f, n0 + l);
    __syncthreads();
  }
  const T k1 = kbeta<T>(field_k(fs, R.K0));
  // fill: line l = column n0+l, position x = m mod X
  for (int e = threadIdx.x; e < nb * X; e += blockDim.x) {
    const int l = fX.div(e);
    const int x = e - l * X;
    C v = mk<T>(T(0), T(0));
    int m = 0;
    bool live = false;
    if (x < MM) { m = x; live = true; }
    else if (x > X - MM) { m = x - X; live = true; }
    if (live) {
      const T m1 = tab ? mtab[x] : wavenum<T>(R.alpha, R.alpha_f, m);
      const T n1 = tab ? ntab[l] : wavenum<T>(R.gamma, R.gamma_f, n0 + l);
      v = mpt_to_field_w<T>(R, c, fs, m, n0 + l, wi.pad == 0, m1, n1, k1);
      if (deriv) v = mk<T>(-v.y * m1, v.x * m1);
    }
    buf[pad_idx<T>(l * S + x)] = cconj(v);
  }
  // backward transform (e^{+i}) as conj(forward(conj(.))): the conjugates are folded into the
  // fill above and the store below, so the transforms run forward-only codelets
  if (!fft_x_fixed<T, NT, VPT>(buf, 0, nb, X, reinterpret_cast<const C*>(R.twX), err))
    fft_lines_inl<T, VPT, kXMaxRadix<T>>(buf, 0, nb, S, R.planX, reinterpret_cast<const C*>(R.twX), false, err);
  // store T[f][x][n0 + l], consecutive threads -> consecutive n
  C* __restrict__ out = reinterpret_cast<C*>(R.T) + (size_t)f * X * NN;
  for (int e = threadIdx.x; e < nb * X; e += blockDim.x) {
    const int x = fNB.div(e);
    const int l = e - x * nb;
    out[(size_t)x * NN + n0 + l] = cconj(buf[pad_idx<T>(l * S + x)]);
  }
}

// ---------------------------------------------------------------------------------------
// Pass 2: z transforms + nonlinear term for the z-subsets of L x lines.
// Work item = (run, first x line x0, subset s), or s = 3 for FP32 runs (RunDesc::z_sum): the
// three subsets in turn.  For subset s the CTA owns the L*NN points z = s + 3q of its lines,
// and work runs as a sequence of tasks sharing one transform:
//   A: u,v,w of the points, two fields per complex transform, NB transforms at a time,
//      stored in shared memory (pv);
//   (then v d/dy terms into the accumulators nl)
//   C: (d/dx f_J, d/dz f_J) pairs; each adds u d/dx f_J + w d/dz f_J into nl;
//   D: the KK products, two per forward transform, Hermitian split, w^{-ns} and the
//      1/(X Z) scale, written to this subset's partial output NLT_s (z_sum: added to NLT_0).
// ---------------------------------------------------------------------------------------

template <typename T>
struct PView {
  const T* base;
  int stride;
  __device__ __forceinline__ T operator[](int i) const { return base[i * stride]; }
};
template <typename T>
struct NLView {
  T* base;
  int stride;
  __device__ __forceinline__ T& operator[](int i) const { return base[i * stride]; }
};

// Hermitian part of one field for subset s (see the header comment):
//   n = 0 : Re X_0 ;  n > 0 : X_n w^{ns} + conj(X_{Q-n}) w^{-(Q-n)s}
template <typename T>
__device__ __forceinline__ cx<T> herm(cx<T> xn, cx<T> xqn, int n, int Q, int s, const cx<T>* __restrict__ twZ) {
  if (n == 0) return mk<T>(xn.x, T(0));
  if (s == 0) return cadd(xn, cconj(xqn));
  const cx<T> a = cmulc(xn, __ldg(&twZ[n * s]));
  const cx<T> b = cmul(cconj(xqn), __ldg(&twZ[(Q - n) * s]));
  return cadd(a, b);
}

template <int K0, typename T>
__device__ __forceinline__ void nl_pair_rt(int k, const T (&nl)[3 * K0 - 1], T& a, T& b) {
  constexpr int KK = 3 * K0 - 1;
#define MWF_PC(j) case j: if constexpr (2 * j < KK) { a = nl[2 * j]; b = (2 * j + 1 < KK) ? nl[(2 * j + 1) % KK] : T(0); } break;
  switch (k) {
    MWF_PC(0) MWF_PC(1) MWF_PC(2) MWF_PC(3) MWF_PC(4) MWF_PC(5) MWF_PC(6) MWF_PC(7) MWF_PC(8)
    default: a = T(0); b = T(0); break;
  }
#undef MWF_PC
}

// NLS: keep the nonlinear accumulators in shared memory (FP64, where registers are needed for
// occupancy and the FP64 pipe, not shared memory, is the limit, and FP32 with one point per
// thread, whose registers go to the compile-time transforms) or in registers.
// PF (FP32): the input rows of the next task are copied into a shared-memory staging
// buffer while the current task computes (double buffered); the fill then reads shared
// memory.  Staging slot q of a task holds one field's rows for the CTA's lines, which are
// contiguous in T ([f][x][n] with the lines x0..x0+L-1 adjacent), so with NN even each slot
// is one bulk copy of L*NN complex values issued by thread 0 (TMA, completing on the
// buffer's mbarrier); odd NN falls back to per-element cp.async.
// DIAG: physical-space diagnostics instead of the nonlinear term -- only the u,v,w tasks run
// (on x-transformed fields without the base flow), then each point's epos (y-mean of
// u^2+v^2+w^2, velocity.f90:115-126) is compared with RunDesc::diag_ct; the CTA writes
// (number of points above, sum of epos) as two doubles to the run's NLT scratch at
// 2*blockIdx.x (diagnostic launches hold one run's items only).
template <typename T, int K0, int PPT, int NT, int NB, bool NLS, bool DIAG = false, bool PF = !NLS>
__global__ void __launch_bounds__(NT, NT > 256 ? 1 : (sizeof(T) == 8 ? 2 : 3)) z_nonlinear_kernel(const RunDesc* __restrict__ runs,
                                                           const WorkItem* __restrict__ items, int* err) {
  using C = cx<T>;
  constexpr int KK = 3 * K0 - 1;
  constexpr int NPAIR = (KK + 1) / 2;
  constexpr int NTA = (NPAIR + NB - 1) / NB;
  constexpr int NTC = (KK + NB - 1) / NB;
  constexpr int NTASK = DIAG ? NTA : 2 * NTA + NTC;
  constexpr int PTS = NT * PPT;           // point capacity of the CTA
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);                       // NB * PTS complex
  T* pv = reinterpret_cast<T*>(smem_raw + sizeof(C) * padded_elems<T>(NB * PTS));  // KK * PTS reals
  T* nlv = pv + (size_t)KK * PTS;                                  // KK * PTS reals if NLS
  // PF: 2 x 2NB x PTS complex, from a 16-byte boundary (bulk-copy destinations)
  C* stage = reinterpret_cast<C*>(smem_raw + ((sizeof(C) * padded_elems<T>(NB * PTS) +
                                               sizeof(T) * (NLS ? 2 : 1) * KK * PTS + 15) & ~size_t(15)));
  __shared__ __align__(8) unsigned long long stage_bar[2];        // PF: one mbarrier per buffer
  // PP (FP32 M4, one point per thread): a second transform buffer after the staging buffers,
  // so the two-stage transforms run out of place (M6 keeps three CTAs per SM without it)
  constexpr bool PP = zpass_pingpong(sizeof(T) == 8 ? 0 : 1, K0, PPT);
  C* buf2 = stage + (PF ? 4 * NB * PTS : 0);
  const WorkItem wi = items[blockIdx.x];
  const RunDesc& R = runs[wi.run];
  if (!R.active) return;
  const int X = R.X, NN = R.NN, Q = R.NN;
  const int x0 = wi.a;
  // z-subsets of this item: wi.b alone, or (wi.b = 3, RunDesc::z_sum) all three in turn, each
  // adding its output to the first partial in the order the x-inverse pass would sum them
  // (FP32 only: for FP64 the subset loop folds away at compile time)
  constexpr bool kSum = sizeof(T) == 4 && !DIAG;
  const bool sum3 = kSum && wi.b == 3;
  const int s0 = sum3 ? 0 : wi.b, nsub = sum3 ? 3 : 1;
  const int L = min(R.z_lx, X - x0);
  const int npts = L * Q;
  if (npts > PTS) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_OUTPUT_CAPACITY);
    return;
  }
  const size_t fstride = (size_t)X * NN;
  const FastDiv fN = make_fastdiv(npts);
  const int Qh = Q / 2 + 1;                       // pairs (n, Q-n), n = 0..Q/2, per line
  const FastDiv fQh = make_fastdiv(Qh), fLQh = make_fastdiv(L * Qh);
  const C* __restrict__ Tin = reinterpret_cast<const C*>(R.T) + (size_t)x0 * NN;
  C* __restrict__ NLT = reinterpret_cast<C*>(R.NLT) + (size_t)(sum3 ? 0 : s0) * KK * fstride + (size_t)x0 * NN;
  const C* __restrict__ twZ = reinterpret_cast<const C*>(R.twZ);
  const C* __restrict__ twQ = reinterpret_cast<const C*>(R.twQ);
  const T gam = T(R.gamma);
  const T hscale = T(0.5 * R.scale);      // 1/2 of the Hermitian split times 1/(XZ)

  T nl[NLS ? 1 : PPT][KK];

  // field held by staging slot q of a task (kind 0: the pair's two fields; kind 1: d/dx f_J
  // in the even slot and f_J in the odd slot); -1 = none
  auto slot_field = [&](int kind_, int g_, int q) -> int {
    const int b = q >> 1;
    if (kind_ == 0) { const int f = 2 * (g_ + b) + (q & 1); return f < KK ? f : -1; }
    return (q & 1) ? g_ + b : KK + g_ + b;
  };
  // tasks t = 0..NCOPY-1 (kinds 0 and 1) of each subset read staged rows.  Over the item's
  // flattened task sequence u = si*NTASK + t, copy task c = si*NCOPY + t uses buffer c&1, and
  // its (c>>1)-th use completes phase c>>1 of that buffer's mbarrier.
  constexpr int NCOPY = DIAG ? NTA : NTA + NTC;
  const int ntot = kSum ? nsub * NTASK : NTASK;
  const bool bulk = PF && (NN % 2 == 0);   // every slot's rows start and end on 16-byte boundaries
  const unsigned long long wait_ns = R.test_wait_ns ? R.test_wait_ns : kMbarWaitNs;
  if constexpr (PF) {
    if (bulk) {
      if (threadIdx.x == 0) {
        mbar_init(&stage_bar[0], 1);
        mbar_init(&stage_bar[1], 1);
        mbar_init_fence();
      }
      __syncthreads();
    }
  }
  auto issue = [&](int u) {
    if constexpr (PF) {
      const int su = kSum ? u / NTASK : 0, tt = u - su * NTASK, c = su * NCOPY + tt;
      if (u < ntot && tt < NCOPY) {
        const int kind_ = tt < NTA ? 0 : 1;
        const int g_ = (kind_ == 0 ? tt : tt - NTA) * NB;
        const int nbk_ = kind_ == 1 ? min(NB, KK - g_) : min(NB, NPAIR - g_);
        C* sb = stage + (size_t)(c & 1) * 2 * NB * PTS;
        if (bulk) {
          if (threadIdx.x == 0) {
            int nslot = 0;
            for (int q = 0; q < 2 * nbk_; ++q) nslot += slot_field(kind_, g_, q) >= 0;
            const unsigned bytes = (unsigned)(npts * sizeof(C));
            // the buffer was last read by the fill of copy task c-2, which every thread finished
            // before that task's transform barriers; order those reads before the async writes
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&stage_bar[c & 1], bytes * nslot + R.test_tx_extra);
            for (int q = 0; q < 2 * nbk_; ++q) {
              const int f = slot_field(kind_, g_, q);
              if (f >= 0) bulk_copy_g2s(sb + q * PTS, Tin + (size_t)f * fstride, bytes, &stage_bar[c & 1]);
            }
          }
        } else {
          for (int e = threadIdx.x; e < 2 * nbk_ * npts; e += NT) {
            const int q = fN.div(e);
            const int r = e - q * npts;
            const int f = slot_field(kind_, g_, q);
            if (f >= 0) cp_async<sizeof(C)>(sb + q * PTS + r, Tin + (size_t)f * fstride + r);
          }
        }
      }
      if (!bulk) cp_async_commit();
    }
  };
  issue(0);

  for (int u = 0; u < ntot; ++u) {
    const int si = kSum ? u / NTASK : 0, t = u - si * NTASK;
    const int s = s0 + si;
    const int cb = si * NCOPY + t;           // copy-task index while t < NCOPY
    const int kind = t < NTA ? 0 : (t < NTA + NTC ? 1 : 2);
    const int g = (kind == 0 ? t : (kind == 1 ? t - NTA : t - NTA - NTC)) * NB;
    const int nbk = kind == 1 ? min(NB, KK - g) : min(NB, NPAIR - g);
    bool staged = true;
    if constexpr (PF) {
      issue(u + 1);
      if (!bulk) cp_async_wait<1>();     // everything but the group just issued: task u's rows are in
      else if (t < NCOPY) staged = mbar_wait(&stage_bar[cb & 1], (cb >> 1) & 1, wait_ns);
    }
    if (t == NTA) {
      // all u,v,w of the points are in pv: v d/dy terms
      __syncthreads();
#pragma unroll
      for (int i = 0; i < PPT; ++i) {
        const int e = threadIdx.x + i * NT;
        if (e < npts) {
          if constexpr (NLS) nl_y<K0, T>(PView<T>{pv + e, PTS}, NLView<T>{nlv + e, PTS});
          else nl_y<K0, T>(PView<T>{pv + e, PTS}, nl[i]);
        }
      }
    }
    if (__syncthreads_or(!staged)) {
      // a bulk copy did not land within the wait limit: flag it, give the copies in flight one
      // more bounded wait, and leave this work item
      if (threadIdx.x == 0) {
        atomicOr(err, MWF_DERR_COPY_TIMEOUT);
        // a test that armed the barriers with extra bytes completes them here, so the wait below
        // ends when the real copies have landed
        if (R.test_tx_extra) mbar_complete_tx(&stage_bar[cb & 1], R.test_tx_extra);
        mbar_wait(&stage_bar[cb & 1], (cb >> 1) & 1, wait_ns);
        // the copy issued for the next task, if that is a copy task
        const int un = u + 1, sn = un / NTASK, tn = un - sn * NTASK, cn = sn * NCOPY + tn;
        if (un < ntot && tn < NCOPY) {
          if (R.test_tx_extra) mbar_complete_tx(&stage_bar[cn & 1], R.test_tx_extra);
          mbar_wait(&stage_bar[cn & 1], (cn >> 1) & 1, wait_ns);
        }
      }
      return;
    }
    // ---- fill nbk lines-groups of the transform buffer ----
    // One item per Hermitian pair (n, Q-n) of a line: with w = w^{ns} and eps = e^{-2 pi i s/3},
    //   H[n]   = w (X_n + eps conj X_{Q-n}),   H[Q-n] = conj(eps w) (X_{Q-n} + eps conj X_n),
    // so four loads give both outputs of both packed fields.  n = 0: H = Re X_0.
    if (kind < 2) {
      for (int e = threadIdx.x; e < nbk * L * Qh; e += NT) {
        const int b = fLQh.div(e);
        const int r = e - b * L * Qh;
        const int l = fQh.div(r);
        const int n = r - l * Qh;
        const int nq = (n == 0) ? 0 : Q - n;
        const C* pa;   // the row of the first packed field (kind 0: f_a; kind 1: d/dx f_J)
        const C* pb;   // kind 0: f_b (null past KK); kind 1: f_J, differentiated in z below
        if constexpr (PF) {
          const C* sb = stage + (size_t)(cb & 1) * 2 * NB * PTS + (size_t)l * Q;
          pa = sb + (2 * b) * PTS;
          pb = (kind == 0 && 2 * (g + b) + 1 >= KK) ? nullptr : sb + (2 * b + 1) * PTS;
        } else {
          const size_t row = (size_t)l * NN;
          if (kind == 0) {
            const int fa = 2 * (g + b);
            pa = Tin + (size_t)fa * fstride + row;
            pb = (fa + 1 < KK) ? Tin + (size_t)(fa + 1) * fstride + row : nullptr;
          } else {
            pa = Tin + (size_t)(KK + g + b) * fstride + row;
            pb = Tin + (size_t)(g + b) * fstride + row;
          }
        }
        C* yrow = buf;
        const int ybase = b * npts + l * Q;
        const C Pa = pa[n], Ra = pa[nq];
        const C Pb = pb ? pb[n] : mk<T>(T(0), T(0));
        const C Rb = pb ? pb[nq] : mk<T>(T(0), T(0));
        // kinds 0 and 1 need the backward transform (e^{+i}); it runs as conj(forward(conj(H))),
        // so the fill stores conj(H) and the consumers read the conjugate of the result
        if (n == 0) {       // kind 1: the z derivative of the n = 0 coefficient is zero
          yrow[pad_idx<T>(ybase)] = mk<T>(Pa.x, kind == 1 ? T(0) : -Pb.x);
          continue;
        }
        // The packed lines a + i b at n and at Q-n, and the conjugate-side terms:
        //   U  = P_a + i P_b,       V  = conj(R_a) + i conj(R_b)   (R = the row at Q-n)
        //   U' = R_a + i R_b,       V' = conj(P_a) + i conj(P_b)
        // so that H[n] = w U + (eps w) V and H[Q-n] = conj(eps w) U' + conj(w) V'.  Kind 1's
        // second field is the z derivative i gamma n f_J, folded in as real factors.
        C U, V, U2, V2;
        if (kind == 1) {
          const T gn = gam * T(n), gq = gam * T(nq);
          U = mk<T>(Pa.x - gn * Pb.x, Pa.y - gn * Pb.y);
          V = mk<T>(Ra.x + gq * Rb.x, -Ra.y - gq * Rb.y);
          U2 = mk<T>(Ra.x - gq * Rb.x, Ra.y - gq * Rb.y);
          V2 = mk<T>(Pa.x + gn * Pb.x, -Pa.y - gn * Pb.y);
        } else {
          U = mk<T>(Pa.x - Pb.y, Pa.y + Pb.x);
          V = mk<T>(Ra.x + Rb.y, Rb.x - Ra.y);
          U2 = mk<T>(Ra.x - Rb.y, Ra.y + Rb.x);
          V2 = mk<T>(Pa.x + Pb.y, Pb.x - Pa.y);
        }
        C Yn, Yq;
        if (s == 0) {
          Yn = cadd(U, V);
          Yq = cadd(U2, V2);
        } else {
          const C w = cconj(__ldg(&twZ[n * s]));          // w^{ns} = e^{+2 pi i ns / Z}
          const C ew = __ldg(&twZ[(Q - n) * s]);          // eps w = e^{-2 pi i s (Q-n) / Z}
          Yn = cadd(cmul(w, U), cmul(ew, V));
          Yq = cadd(cmulc(U2, ew), cmulc(V2, w));
        }
        yrow[pad_idx<T>(ybase + n)] = cconj(Yn);
        if (nq != n) yrow[pad_idx<T>(ybase + nq)] = cconj(Yq);
      }
    } else {
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        if (b < nbk) {
#pragma unroll
          for (int i = 0; i < PPT; ++i) {
            const int e = threadIdx.x + i * NT;
            if (e < npts) {
              T va, vb;
              if constexpr (NLS) {
                const int ka = 2 * (g + b);
                va = nlv[ka * PTS + e];
                vb = (ka + 1 < KK) ? nlv[(ka + 1) * PTS + e] : T(0);
              } else {
                nl_pair_rt<K0, T>(g + b, nl[i], va, vb);
              }
              buf[pad_idx<T>(b * npts + e)] = mk<T>(va, vb);
            }
          }
        }
      }
    }
    if constexpr (sizeof(T) == 4 && PPT == 1) {
      // FP32 runs up to NN = 512: compile-time transforms for the usual line lengths
      if (!fft_z_fixed<T, NT, NB * PPT, PP>(buf, buf2, nbk * L, Q, twQ, err))
        fft_lines_inl<T, NB * PPT, kZMaxRadix<T>>(buf, 0, nbk * L, Q, R.planQ, twQ, false, err);
    } else {
      fft_lines_inl<T, NB * PPT, kZMaxRadix<T>>(buf, 0, nbk * L, Q, R.planQ, twQ, false, err);
    }
    // ---- consume ----
    if (kind == 0) {
      for (int e = threadIdx.x; e < nbk * npts; e += NT) {
        const int b = fN.div(e);
        const int r = e - b * npts;
        const int fa = 2 * (g + b);
        const C v = buf[pad_idx<T>(e)];
        pv[fa * PTS + r] = v.x;
        if (fa + 1 < KK) pv[(fa + 1) * PTS + r] = -v.y;      // Im of the conjugated result
      }
    } else if (kind == 1) {
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        if (b < nbk) {
#pragma unroll
          for (int i = 0; i < PPT; ++i) {
            const int e = threadIdx.x + i * NT;
            if (e < npts) {
              const C v = buf[pad_idx<T>(b * npts + e)];
              if constexpr (NLS) nl_xz_rt<K0, T>(g + b, PView<T>{pv + e, PTS}, v.x, -v.y, NLView<T>{nlv + e, PTS});
              else nl_xz_rt<K0, T>(g + b, PView<T>{pv + e, PTS}, v.x, -v.y, nl[i]);
            }
          }
        }
      }
    } else {
      // one item per pair (n, Q-n): A = (G_n + conj G_{Q-n})/2 and B = (G_n - conj G_{Q-n})/(2i)
      // are the spectra of the two real products at n; at Q-n they are conj(A), conj(B).
      // Each is scaled by 1/(XZ) and by w^{-ns} at n, w^{-(Q-n)s} at Q-n (both from the table).
      for (int e = threadIdx.x; e < nbk * L * Qh; e += NT) {
        const int b = fLQh.div(e);
        const int r = e - b * L * Qh;
        const int l = fQh.div(r);
        const int n = r - l * Qh;
        const int nq = (n == 0) ? 0 : Q - n;
        const int ybase = b * npts + l * Q;
        const C gg = buf[pad_idx<T>(ybase + n)];
        const C gm = buf[pad_idx<T>(ybase + nq)];
        // A, B with the 1/2 of the split and the 1/(XZ) scale folded in
        const C A = mk<T>(hscale * (gg.x + gm.x), hscale * (gg.y - gm.y));
        const C B = mk<T>(hscale * (gg.y + gm.y), hscale * (gm.x - gg.x));
        const int ka = 2 * (g + b), kb = ka + 1;
        const size_t o = (size_t)l * NN;
        if (s == 0) {
          NLT[(size_t)ka * fstride + o + n] = A;
          if (kb < KK) NLT[(size_t)kb * fstride + o + n] = B;
          if (nq != n) {
            NLT[(size_t)ka * fstride + o + nq] = cconj(A);
            if (kb < KK) NLT[(size_t)kb * fstride + o + nq] = cconj(B);
          }
        } else {
          // summed items add to what this thread stored for the earlier subsets (same item
          // mapping in every subset): ((s0 + s1) + s2), as the x-inverse pass adds partials
          auto put = [&](size_t i, C v) {
            if (kSum && sum3) NLT[i] = cadd(NLT[i], v);
            else NLT[i] = v;
          };
          const C tz = __ldg(&twZ[n * s]);                // w^{-ns}
          put((size_t)ka * fstride + o + n, cmul(A, tz));
          if (kb < KK) put((size_t)kb * fstride + o + n, cmul(B, tz));
          if (nq != n) {
            const C tq = __ldg(&twZ[(Q - n) * s]);        // w^{-(Q-n)s}
            put((size_t)ka * fstride + o + nq, cmul(cconj(A), tq));
            if (kb < KK) put((size_t)kb * fstride + o + nq, cmul(cconj(B), tq));
          }
        }
      }
    }
  }
  if constexpr (DIAG) {
    __syncthreads();
    double cnt = 0.0, sum = 0.0;
#pragma unroll
    for (int i = 0; i < PPT; ++i) {
      const int e = threadIdx.x + i * NT;
      if (e < npts) {
        double ep = 0.0;
#pragma unroll
        for (int f = 0; f < KK; ++f) {
          const double v = (double)pv[f * PTS + e];
          ep += ((f == 0 || f == 2 * K0 - 1) ? 1.0 : 0.5) * v * v;
        }
        sum += ep;
        cnt += (ep > R.diag_ct) ? 1.0 : 0.0;
      }
    }
    double* red = reinterpret_cast<double*>(smem_raw);
    __syncthreads();
    red[threadIdx.x] = cnt;
    red[NT + threadIdx.x] = sum;
    __syncthreads();
    for (int h = NT / 2; h > 0; h >>= 1) {
      if ((int)threadIdx.x < h) {
        red[threadIdx.x] += red[threadIdx.x + h];
        red[NT + threadIdx.x] += red[NT + threadIdx.x + h];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      double* out = reinterpret_cast<double*>(R.NLT);
      out[2 * blockIdx.x] = red[0];
      out[2 * blockIdx.x + 1] = red[NT];
    }
  }
}

// ---------------------------------------------------------------------------------------
// Pass 3: x inverse + projection + AB2/implicit update.
// Work item = (run, first column n0, wall-normal mode k).  The fields u_k, v_k (k >= 1)
// and w_k of nb columns are loaded as 3*nb lines and transformed; each output (column, m)
// then reads its three spectral values and produces psi_k (and phi_k for k >= 1).
// ---------------------------------------------------------------------------------------
template <typename T, int VPT, int NT>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 1024 / NT : 512 / NT) x_inverse_kernel(const RunDesc* __restrict__ runs, const WorkItem* __restrict__ items,
                                 int* err) {
  using C = cx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const WorkItem wi = items[blockIdx.x];
  const RunDesc& R = runs[wi.run];
  if (!R.active) return;
  const int X = R.X, MM = R.MM, NN = R.NN, M = R.M, K0 = R.K0, K = R.K;
  const int n0 = wi.a;
  const int nb = min(R.xi_nb, NN - n0);
  const int k = wi.b;
  const int S = X;
  const C* __restrict__ NLT = reinterpret_cast<const C*>(R.NLT);
  const size_t fstride = (size_t)X * NN;
  // line (comp, l) at buf[(comp*nb + l)*S]; comp 0 = u_k, 1 = v_k, 2 = w_k
  const int fu = k, fv = K0 + k - 1, fw = 2 * K0 - 1 + k;
  const FastDiv fNX = make_fastdiv(nb * X), fNB = make_fastdiv(nb), fM = make_fastdiv(M);
  for (int e = threadIdx.x; e < 3 * nb * X; e += blockDim.x) {
    const int comp = fNX.div(e);
    const int r = e - comp * nb * X;
    const int x = fNB.div(r);
    const int l = r - x * nb;
    C v = mk<T>(T(0), T(0));
    if (!(comp == 1 && k == 0)) {
      const int fs = comp == 0 ? fu : (comp == 1 ? fv : fw);
      const size_t o = (size_t)fs * fstride + (size_t)x * NN + n0 + l;
      const size_t ss = (size_t)R.KK * fstride;        // the three z-subset partials (z_sum: summed in the first)
      v = R.z_sum ? NLT[o] : cadd(cadd(NLT[o], NLT[o + ss]), NLT[o + 2 * ss]);
    }
    buf[pad_idx<T>((comp * nb + l) * S + x)] = v;
  }
  // the three fields one after the other (a third of the registers of one 3*nb-line call)
  // (the compile-time x plans of the x-forward pass measured slower here: the three fields'
  // buffers leave less room for their registers)
  for (int comp = 0; comp < 3; ++comp)
    fft_lines_inl<T, VPT, kXMaxRadix<T>>(buf, comp * nb * S, nb, S, R.planX, reinterpret_cast<const C*>(R.twX),
                                         false, err);

  C* __restrict__ c = reinterpret_cast<C*>(R.c);
  C* __restrict__ onl = reinterpret_cast<C*>(R.onl);
  if constexpr (sizeof(T) == 4) {
    // FP32 runs: var_spec2mpt in FP32 and the update c' = A c + B (3 nl - onl), A = rhs/lhs and
    // B = (dt/2)/lhs formed in FP64 by the host, with no FP64 instruction in the pass.  A is a
    // float pair (hi + lo, ~48 bits), A_hi c is split exactly into ph + pl with an FMA, and
    // everything below ph is summed first, so c' is rounded once, as the FP64 update rounds
    // it once to FP32.  (Rounding the decayed state A c on its own before adding the
    // nonlinear increment biases slowly varying modes: -2e-6 relative energy after 50 steps
    // on a 3072^2 grid.)
    const size_t csz = (size_t)NN * K * M;
    const float* __restrict__ a_hi = reinterpret_cast<const float*>(R.inv_lhs);
    const float* __restrict__ a_lo = a_hi + csz;
    const float* __restrict__ bnl = reinterpret_cast<const float*>(R.rhs);
    const bool first32 = *R.nst != 0;
    const float kb1 = kbeta<float>(k);
    for (int o = threadIdx.x; o < nb * M; o += blockDim.x) {
      const int l = fM.div(o);
      const int ms = o - l * M;
      const int n = n0 + l;
      const int m = signed_m(ms, MM, M);
      const int xi = m < 0 ? m + X : m;
      const C su = buf[pad_idx<T>((0 * nb + l) * S + xi)];
      const C sv = buf[pad_idx<T>((1 * nb + l) * S + xi)];
      const C sw = buf[pad_idx<T>((2 * nb + l) * S + xi)];
      const float m1 = wavenum<float>(R.alpha, R.alpha_f, m);
      const float n1 = wavenum<float>(R.gamma, R.gamma_f, n);
      const float H = -(m1 * m1) - n1 * n1;
      float2 nphi, npsi;
      nphi.x = -(su.y * m1 * kb1 + sw.y * n1 * kb1) + sv.x * H;
      nphi.y = (su.x * m1 * kb1 + sw.x * n1 * kb1) + sv.y * H;
      npsi.x = sw.y * m1 - su.y * n1;
      npsi.y = -(sw.x * m1 - su.x * n1);
      if (ms == 0 && n == 0) {
        if (k == 0) npsi = make_float2(0.f, 0.f);
        else {
          npsi = make_float2(-su.x, -su.y);
          nphi = make_float2(-sw.x, -sw.y);
        }
      }
#pragma unroll
      for (int which = 0; which < 2; ++which) {
        if (which == 1 && k == 0) continue;
        const int slot = which == 0 ? k : k + K0 - 1;
        const float2 nlv = which == 0 ? npsi : nphi;
        const size_t idx = ((size_t)n * K + slot) * M + ms;
        const C cold = c[idx];
        const float2 ov = first32 ? nlv : onl[idx];
        const float ah = a_hi[idx], al = a_lo[idx], b = bnl[idx];
        auto update = [&](float cv, float nv, float onv) {
          const float ph = __fmul_rn(ah, cv);              // not contracted: ph + pl = ah*cv exactly
          const float pl = fmaf(ah, cv, -ph);
          const float r = fmaf(b, fmaf(3.f, nv, -onv), fmaf(al, cv, pl));
          return __fadd_rn(ph, r);
        };
        float cx_ = update(cold.x, nlv.x, ov.x);
        const float cy_ = update(cold.y, nlv.y, ov.y);
        if (slot == 0 && ms == 0 && n == 0) cx_ = 0.f;
        c[idx] = mk<T>(cx_, cy_);
        onl[idx] = mk<T>(nlv.x, nlv.y);
      }
    }
    return;
  }
  const double* __restrict__ ilhs = R.inv_lhs;
  const double* __restrict__ rhs = R.rhs;
  const bool first = *R.nst != 0;
  const double hdt = R.dt / 2.0;
  const double kb1 = (k & 1) ? -k * kBeta : k * kBeta;
  for (int o = threadIdx.x; o < nb * M; o += blockDim.x) {
    const int l = fM.div(o);
    const int ms = o - l * M;
    const int n = n0 + l;
    const int m = signed_m(ms, MM, M);
    const int xi = m < 0 ? m + X : m;
    const C su = buf[pad_idx<T>((0 * nb + l) * S + xi)];
    const C sv = buf[pad_idx<T>((1 * nb + l) * S + xi)];
    const C sw = buf[pad_idx<T>((2 * nb + l) * S + xi)];
    const double m1 = R.alpha * m;
    const double n1 = R.gamma * n;
    const double H = (-R.alpha * m * R.alpha * m) + (-R.gamma * n * R.gamma * n);
    // var_spec2mpt (variables.f90:455-464)
    double2 nphi, npsi;
    nphi.x = -((double)su.y * m1 * kb1 + (double)sw.y * n1 * kb1) + (double)sv.x * H;
    nphi.y = ((double)su.x * m1 * kb1 + (double)sw.x * n1 * kb1) + (double)sv.y * H;
    npsi.x = (double)sw.y * m1 - (double)su.y * n1;
    npsi.y = -((double)sw.x * m1 - (double)su.x * n1);
    if (ms == 0 && n == 0) {   // mean modes (variables.f90:467-479)
      if (k == 0) npsi = make_double2(0.0, 0.0);
      else {
        npsi = make_double2(-(double)su.x, -(double)su.y);
        nphi = make_double2(-(double)sw.x, -(double)sw.y);
      }
    }
    // AB2 / implicit update (velocity.f90:24-40); onl <- nl
#pragma unroll
    for (int which = 0; which < 2; ++which) {
      if (which == 1 && k == 0) continue;
      const int slot = which == 0 ? k : k + K0 - 1;
      const double2 nlv = which == 0 ? npsi : nphi;
      const size_t idx = ((size_t)n * K + slot) * M + ms;
      const C cold = c[idx];
      double2 ov;
      if (first) ov = nlv; else { const C t = onl[idx]; ov = make_double2((double)t.x, (double)t.y); }
      const double rr = rhs[idx], il = ilhs[idx];
      double cx_ = rr * (double)cold.x + hdt * (3.0 * nlv.x - ov.x);
      double cy_ = rr * (double)cold.y + hdt * (3.0 * nlv.y - ov.y);
      cx_ *= il;
      cy_ *= il;
      if (slot == 0 && ms == 0 && n == 0) cx_ = 0.0;
      c[idx] = mk<T>(T(cx_), T(cy_));
      onl[idx] = mk<T>(T(nlv.x), T(nlv.y));
    }
  }
}

// ---------------------------------------------------------------------------------------
// Perturbation energy of vel_energy (velocity.f90:144-162) by Parseval on the spectral
// u,v,w (no base flow):  E = sum_f w_f [ sum_m |h_f(m,0)|^2 + 2 sum_{n>=1,m} |s_f(m,n)|^2 ],
// h = Hermitian part of the n = 0 column (the c2r keeps only Re of the x-transformed DC),
// w_f = 1 for u_0, w_0 and 1/2 otherwise (epos, velocity.f90:115-126).  FP64 with
// Neumaier-compensated per-thread sums and a pairwise tree across the block.
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void energy_partial_kernel(const RunDesc* __restrict__ runs, int run, double* partial) {
  using C = cx<T>;
  const RunDesc& R = runs[run];
  const C* __restrict__ c = reinterpret_cast<const C*>(R.c);
  const int M = R.M, NN = R.NN, KK = R.KK, K0 = R.K0, MM = R.MM;
  const size_t npt = (size_t)NN * M;
  double sum = 0.0, comp = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < npt; e += (size_t)gridDim.x * blockDim.x) {
    const int n = (int)(e / M);
    const int ms = (int)(e - (size_t)n * M);
    const int m = signed_m(ms, MM, M);
    for (int fs = 0; fs < KK; ++fs) {
      const double w = (fs == 0 || fs == 2 * K0 - 1) ? 1.0 : 0.5;
      const C v = mpt_to_field<T>(R, c, fs, m, n, false);
      double t;
      if (n == 0) {
        const C vm = mpt_to_field<T>(R, c, fs, -m, 0, false);
        const double hx = 0.5 * ((double)v.x + (double)vm.x);
        const double hy = 0.5 * ((double)v.y - (double)vm.y);
        t = w * (hx * hx + hy * hy);
      } else {
        t = 2.0 * w * ((double)v.x * v.x + (double)v.y * v.y);
      }
      const double y = sum + t;
      comp += (fabs(sum) >= fabs(t)) ? (sum - y) + t : (t - y) + sum;
      sum = y;
    }
  }
  __shared__ double red[1024];
  red[threadIdx.x] = sum + comp;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

static __global__ void energy_final_kernel(const double* partial, int nparts, double* out) {
  if (threadIdx.x != 0) return;
  double sum = 0.0, comp = 0.0;
  for (int i = 0; i < nparts; ++i) {
    const double t = partial[i];
    const double y = sum + t;
    comp += (fabs(sum) >= fabs(t)) ? (sum - y) + t : (t - y) + sum;
    sum = y;
  }
  *out = sum + comp;
}

// ---------------------------------------------------------------------------------------
// Layout conversion between the reference's split Re/Im (K, M, NN) column-major arrays and
// the device's interleaved [NN][K][M].
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void ref_to_dev_kernel(const double* __restrict__ re, const double* __restrict__ im,
                                  cx<T>* __restrict__ out, int K, int M, int NN) {
  const size_t tot = (size_t)K * M * NN;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    // e enumerates the device layout [n][k][m]
    const int m = (int)(e % M);
    const size_t r = e / M;
    const int k = (int)(r % K);
    const int n = (int)(r / K);
    const size_t src = ((size_t)n * M + m) * K + k;
    out[e] = mk<T>(T(re[src]), T(im[src]));
  }
}

template <typename T>
__global__ void dev_to_ref_kernel(const cx<T>* __restrict__ in, double* __restrict__ re,
                                  double* __restrict__ im, int K, int M, int NN) {
  const size_t tot = (size_t)K * M * NN;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    // e enumerates the reference layout (k fastest, then m, then n)
    const int k = (int)(e % K);
    const size_t r = e / K;
    const int m = (int)(r % M);
    const int n = (int)(r / M);
    const cx<T> v = in[((size_t)n * K + k) * M + m];
    re[e] = (double)v.x;
    im[e] = (double)v.y;
  }
}

// ---------------------------------------------------------------------------------------
// Symmetry masks of vel_imposesym (velocity.f90:68-74), for K0 = 4 as in the reference
// (variables.f90:42-131 hard-code K = 7).  mode 0 = var_reflect, 1 = var_uvreflect,
// 2 = var_wreflect.  One thread per (n, m) column; the three masks run as separate
// launches in the reference's order because uvreflect/wreflect read the column M-m.
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void imposesym_kernel(const RunDesc* __restrict__ runs, int run, int mode) {
  using C = cx<T>;
  const RunDesc& R = runs[run];
  C* c = reinterpret_cast<C*>(R.c);
  const int M = R.M, NN = R.NN, MM = R.MM, K = R.K;
  const size_t tot = (size_t)M * NN;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int n = (int)(e / M);
    const int m = (int)(e - (size_t)n * M);
    C* col = c + (size_t)n * K * M;
    auto at = [&](int k, int mm) -> C& { return col[(size_t)k * M + mm]; };
    if (mode == 0) {
      if (m == 0 && n == 0) {
        at(0, m).x = T(0); at(2, m).x = T(0); at(5, m).x = T(0);
      } else {
        at(0, m).y = T(0); at(1, m).x = T(0); at(2, m).y = T(0); at(3, m).x = T(0);
        at(4, m).x = T(0); at(5, m).y = T(0); at(6, m).x = T(0);
      }
    } else if (mode == 1) {
      if (m == 0) {
        for (int k = 0; k < 7; k += 2) {
          at(k, m).x = T(0);
          if (n != 0) at(k, m).y = T(0);
        }
      } else if (m > MM - 1) {
        const int mm = M - m;
        for (int k = 0; k < 7; ++k) {
          const C v = at(k, mm);
          at(k, m) = (k % 2 == 0) ? mk<T>(-v.x, -v.y) : v;
        }
      }
    } else {
      if (n == 0) {
        if (m == 0) { for (int k = 4; k < 7; ++k) at(k, m).x = T(0); }
        else { for (int k = 0; k < 4; ++k) at(k, m) = mk<T>(T(0), T(0)); }
      } else if (m > MM - 1) {
        const int mm = M - m;
        for (int k = 0; k < 7; ++k) {
          const C v = at(k, mm);
          at(k, m) = (k < 4) ? mk<T>(-v.x, v.y) : mk<T>(v.x, -v.y);
        }
      }
    }
  }
}

// Non-finite check of a run's state: sets *flag to 1 if any coefficient is NaN/Inf.
template <typename T>
__global__ void nonfinite_kernel(const RunDesc* __restrict__ runs, int run, int* flag) {
  using C = cx<T>;
  const RunDesc& R = runs[run];
  const C* c = reinterpret_cast<const C*>(R.c);
  const size_t tot = (size_t)R.K * R.M * R.NN;
  int bad = 0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const C v = c[e];
    if (!isfinite((double)v.x) || !isfinite((double)v.y)) bad = 1;
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

}  // namespace mwf
