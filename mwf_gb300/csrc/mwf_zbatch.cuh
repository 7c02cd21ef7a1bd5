// FP32 z pass with every transform of a work item in one batch (sm_103a).
//
// The work item is (run, first x line x0): the CTA owns L x lines and all three z-subsets
// z = s + 3q (s = 0, 1, 2, q < NN) of them, i.e. every physical point of those lines.  It does
// the same arithmetic as z_nonlinear_kernel (tra_spec2phys z part, transform.fftw5.f90:80-85;
// udotgradu, modes.M4.f90:14-28 / modes.M6.f90:14-20; tra_phys2spec z part,
// transform.fftw5.f90:126-135), organised for fewer barriers and no shared-memory round trips
// of the coupling accumulators:
//   P0  the item's 2KK x-transformed rows (L NN complex values each, contiguous in T) arrive
//       by asynchronous 16-byte copies at the end of the CTA's shared memory (zb_rows_off);
//       then the fill: for every packed pair of the NTR = NPAIR + KK transforms of a subset
//       (NPAIR pairs of u,v,w fields, then KK pairs (d/dx f_J, d/dz f_J)) and every Hermitian
//       pair (n, NN-n), one thread's four shared-memory loads give the two inputs of all three
//       subsets;
//   P1  the 3 NTR L backward transforms of length NN in one batch, each Stockham stage out of
//       place between two shared-memory buffers (one barrier per stage);
//   P2  per point: u,v,w and the derivative pairs are read once, the coupling is formed in
//       registers, and the KK products are written back over the point's first NPAIR slots;
//   P3  the 3 NPAIR L forward transforms in one batch;
//   P4  per Hermitian pair and field pair: the three subsets' spectra are split, twiddled and
//       summed in registers ((s0 + s1) + s2) and the KK fields of the nonlinear term are
//       written once to the first NLT partial (RunDesc::z_sum = 1).
// Line (t, s, l) of the buffers is ((t * 3 + s) * L + l), so the forward transforms' lines
// (t < NPAIR) come first.  Backward transforms run as conj(forward(conj .)): the fill stores
// conjugates and P2 reads the conjugate of the result, as in z_nonlinear_kernel.
// The line count L is a compile-time parameter of the item body (every count an item can hold,
// dispatched at run time), so the row and line offsets are constants.  The launch is one wave
// of resident CTAs that take the items in turn; each CTA issues the copies of its next item's
// rows once P1 is done, into the part of its shared memory that P2-P4 leave free.
#pragma once
#include "mwf_common.cuh"
#include "mwf_fft.cuh"
#include "mwf_launch.h"
#include "nl_gen.cuh"

namespace mwf {

// Compile-time two-stage plan of the batched z pass for NN = Q: radices R1 (first stage) and R2.
template <int Q> struct ZbPlan;
template <> struct ZbPlan<32> { static constexpr int R1 = 8, R2 = 4; };
template <> struct ZbPlan<48> { static constexpr int R1 = 12, R2 = 4; };
template <> struct ZbPlan<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct ZbPlan<96> { static constexpr int R1 = 12, R2 = 8; };
template <> struct ZbPlan<128> { static constexpr int R1 = 16, R2 = 8; };
template <> struct ZbPlan<192> { static constexpr int R1 = 12, R2 = 16; };
template <> struct ZbPlan<256> { static constexpr int R1 = 16, R2 = 16; };

__device__ __forceinline__ unsigned dyn_smem_bytes() {
  unsigned r;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(r));
  return r;
}

// One Stockham stage (radix R, span NS) of `nlines` lines of length N, out of place: each
// butterfly is read from `in`, twiddled, transformed and written to `out` before the next one
// is read, so no butterfly is held across the barrier that ends the stage.  tw[t * TWS] =
// e^{-2 pi i t / N} (TWS = 3 reads the length-3N table of the x lines).
// The first (NT / B) B threads work, each on one butterfly index j of a line and on every
// (NT / B)-th line, so j, the twiddles and the in-line offsets are fixed per thread; N is a
// multiple of 16, so the padded index of element x of line l is l (N + N/16) + pad_idx(x).  The
// thread's R - 1 twiddles are read once, before its lines.
template <int N, int R, int NS, int NT, int TWS = 1>
__device__ __forceinline__ void zb_stage(const float2* __restrict__ in, float2* __restrict__ out, int nlines,
                                         const float2* __restrict__ tw) {
  constexpr int B = N / R, TSTEP = N / (NS * R) * TWS;
  static_assert(N % 16 == 0 && B <= NT, "line length and block size of the batched stages");
  constexpr int LPP = NT / B;               // lines per pass of the CTA
  constexpr int LS = N + N / 16;            // padded line stride
  if (threadIdx.x < LPP * B) {
    const int j = threadIdx.x % B;
    const int k = j % NS;
    const int jo = (j - k) * R + k;
    float2 w[R];                            // this thread's twiddles, loaded once per stage
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) w[r] = __ldg(&tw[r * k * TSTEP]);
    }
    for (int line = threadIdx.x / B; line < nlines; line += LPP) {
      const float2* src = in + line * LS;
      float2* dst = out + line * LS;
      float2 v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = src[pad_idx<float>(j + r * B)];
      if constexpr (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[r] = cmul(v[r], w[r]);
      }
      dftR<float, R>(v, false);
#pragma unroll
      for (int r = 0; r < R; ++r) dst[pad_idx<float>(jo + r * NS)] = v[r];
    }
  }
  __syncthreads();
}

// Complex products of the fill and of P4 with every rounding spelled out (fused multiply-adds),
// so that each kernel that inlines the item -- the per-pass launch and the persistent step --
// rounds them alike, whatever contraction the compiler would choose in its context.
__device__ __forceinline__ float2 zb_mul(float2 a, float2 b) {          // a b
  return make_float2(__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)), __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float2 zb_mac(float2 c, float2 a, float2 b) {  // c + a b
  return make_float2(__fmaf_rn(a.x, b.x, __fmaf_rn(-a.y, b.y, c.x)), __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, c.y)));
}

// Shared memory of one batched z item: two buffers of 3 NTR L lines of Q complex floats, the
// second starting on a 16-byte boundary (asynchronous 16-byte copy destinations).
__host__ __device__ constexpr size_t zb_buf_elems(int K0, int Q, int L) {
  return ((size_t)3 * ((3 * K0 - 1 + 1) / 2 + 3 * K0 - 1) * L * Q +
          ((size_t)3 * ((3 * K0 - 1 + 1) / 2 + 3 * K0 - 1) * L * Q >> 4) + 2) & ~(size_t)1;
}
__host__ __device__ constexpr size_t zb_smem_bytes(int K0, int Q, int L) { return 2 * 8 * zb_buf_elems(K0, Q, L); }

// CTAs per SM of the batched z pass for (K0, NN = Q), and the most lines an item can then hold.
__host__ __device__ constexpr int zb_minb(int K0, int Q) { return zb_smem_bytes(K0, Q, 1) <= zb_smem_budget(2) ? 2 : 1; }
__host__ __device__ constexpr int zb_lmax(int K0, int Q) {
  int L = 1;
  while (zb_smem_bytes(K0, Q, L + 1) <= zb_smem_budget(zb_minb(K0, Q))) ++L;
  return L;
}

// Lines of work item wi of run R in a CTA with smem_bytes of shared memory: L >= 1, 0 for an
// inactive run, -1 if the item does not fit (an internal error).
template <int K0, int Q>
__device__ __forceinline__ int zb_item_lines(const RunDesc& R, const WorkItem& wi, unsigned smem_bytes) {
  if (!R.active) return 0;
  const int L = min(R.zb_lx, R.X - wi.a);
  if (R.NN != Q || L < 1 || L > zb_lmax(K0, Q) || zb_smem_bytes(K0, Q, L) > smem_bytes) return -1;
  return L;
}

// Complex offset of the staged input rows of an item of L lines: the last 2KK L Q complex values
// of the CTA's shared memory, from a 16-byte boundary.  For any two items of at most the lines
// that fit (2 zb_buf_elems(L) complex values), the rows of the second lie beyond the first
// buffer and the part of the second that P3 uses (3 NPAIR L lines), because 2 NN < 3 (NN + NN/16).
__device__ __forceinline__ size_t zb_rows_off(unsigned smem_bytes, int KK, int Q, int L) {
  return ((size_t)(smem_bytes / 8) - (size_t)2 * KK * L * Q) & ~(size_t)1;
}

// Issue the asynchronous 16-byte copies of the 2KK input rows of the item at x line x0 (L lines)
// of run R: rows of field f, T[f][x0 .. x0+L-1][0 .. NN-1], are L NN complex values from a
// 16-byte boundary (NN even, T 256-byte aligned), copied to rows[f L Q ..]; one commit group.
template <int K0, int Q, int NT>
__device__ __forceinline__ void zb_stage_rows(const RunDesc& R, int x0, int L, float2* rows) {
  constexpr int KK = 3 * K0 - 1;
  constexpr int CH = 2;                                 // complex values per 16-byte copy
  const float2* __restrict__ Tin = reinterpret_cast<const float2*>(R.T) + (size_t)x0 * Q;
  const size_t fstride = (size_t)R.X * Q;
  const int rowc = L * Q / CH;
  const FastDiv fL = make_fastdiv(L);
  for (int e = threadIdx.x; e < 2 * KK * rowc; e += NT) {
    const int f = fL.div(e / (Q / CH));
    const int c = e - f * rowc;
    cp_async<16>(rows + (size_t)f * L * Q + c * CH, Tin + (size_t)f * fstride + c * CH);
  }
  cp_async_commit();
}

// One work item of L x lines (a compile-time count, so every shared-memory offset of a field
// pair is a constant) of the batched z pass, run by the whole CTA (NT threads) in smem_raw (16-byte
// aligned, smem_bytes in all), whose input rows are in flight (zb_stage_rows, the CTA's only
// open commit group) at zb_rows_off.  If Rn is not null, the rows of the next item (run *Rn,
// line x0n, Ln lines) are prefetched once P1 is done, into the space the rest of the item
// leaves free.  The caller synchronises the CTA before it reuses the shared memory otherwise.
template <int K0, int Q, int NT, int L>
__device__ __forceinline__ void z_batched_body(const RunDesc& R, int x0, unsigned char* smem_raw,
                                               unsigned smem_bytes, const RunDesc* Rn, int x0n, int Ln,
                                               int* err) {
  using C = float2;
  constexpr int KK = 3 * K0 - 1;
  constexpr int NPAIR = (KK + 1) / 2;
  constexpr int NTR = NPAIR + KK;
  constexpr int R1 = ZbPlan<Q>::R1, R2 = ZbPlan<Q>::R2;
  static_assert(R1 * R2 == Q, "two-stage plan");
  const int X = R.X, NN = Q;
  const int nlines = 3 * NTR * L;
  C* A = reinterpret_cast<C*>(smem_raw);
  C* Bf = A + zb_buf_elems(K0, Q, L);
  const size_t fstride = (size_t)X * NN;
  const C* __restrict__ twZ = reinterpret_cast<const C*>(R.twZ);
  const C* __restrict__ twQ = reinterpret_cast<const C*>(R.twQ);
  const float gam = R.gamma_f;
  const float hscale = (float)(0.5 * R.scale);      // 1/2 of the Hermitian split times 1/(XZ)
  auto line = [&](int t, int s, int l) { return (t * 3 + s) * L + l; };

  // ---- P0: the staged input rows, then the fill ----
  cp_async_wait<0>();
  __syncthreads();
  // Fill and P4 give each thread one Hermitian pair (n, NN-n) of every (line, field pair) row
  // it visits: slot 0 takes n = NN/2 (its own partner), slots 1 .. NN/2-1 take n = slot, and
  // n = 0 has a short loop of its own.  The twiddles, the gamma n factors and the padded offsets
  // are then fixed per thread.
  constexpr int S = Q / 2;                          // pair slots per row
  constexpr int RPP = NT / S;                       // rows per pass of the CTA
  constexpr int LS = Q + Q / 16;                    // padded line stride
  static_assert(RPP >= 1 && Q % 16 == 0, "pair slots of the batched z pass");
  const int slot = threadIdx.x % S;
  const int n = slot == 0 ? S : slot;
  const int nq = Q - n;
  const int pn = pad_idx<float>(n), pq = pad_idx<float>(nq);
  const C tz1 = __ldg(&twZ[n]), tq1 = __ldg(&twZ[Q - n]);                 // w^{-ns}, w^{-(NN-n)s}
  const C tz2 = __ldg(&twZ[2 * n]), tq2 = __ldg(&twZ[2 * (Q - n)]);
  const bool worker = threadIdx.x < RPP * S;
  const C* __restrict__ St = A + zb_rows_off(smem_bytes, KK, Q, L);
  if (worker) {
    const float gn = gam * (float)n, gq = gam * (float)nq;
    for (int row = threadIdx.x / S; row < NTR * L; row += RPP) {
      const int t = row / L;
      const int l = row - t * L;
      const bool kind1 = t >= NPAIR;
      const C* pa;
      const C* pb;
      if (!kind1) {
        const int fa = 2 * t;
        pa = St + (fa * L + l) * Q;
        pb = (fa + 1 < KK) ? St + ((fa + 1) * L + l) * Q : nullptr;
      } else {
        const int J = t - NPAIR;
        pa = St + ((KK + J) * L + l) * Q;
        pb = St + (J * L + l) * Q;
      }
      const C Pa = pa[n], Ra = pa[nq];
      const C Pb = pb ? pb[n] : mk<float>(0.f, 0.f);
      const C Rb = pb ? pb[nq] : mk<float>(0.f, 0.f);
      // packed lines at n and NN-n (see z_nonlinear_kernel): H[n] = w U + (eps w) V and
      // H[NN-n] = conj(eps w) U' + conj(w) V', with w = w^{ns}, eps w = e^{-2 pi i s (NN-n)/Z}
      C U, V, U2, V2;
      if (kind1) {
        U = mk<float>(__fmaf_rn(-gn, Pb.x, Pa.x), __fmaf_rn(-gn, Pb.y, Pa.y));
        V = mk<float>(__fmaf_rn(gq, Rb.x, Ra.x), -__fmaf_rn(gq, Rb.y, Ra.y));
        U2 = mk<float>(__fmaf_rn(-gq, Rb.x, Ra.x), __fmaf_rn(-gq, Rb.y, Ra.y));
        V2 = mk<float>(__fmaf_rn(gn, Pb.x, Pa.x), -__fmaf_rn(gn, Pb.y, Pa.y));
      } else {
        U = mk<float>(Pa.x - Pb.y, Pa.y + Pb.x);
        V = mk<float>(Ra.x + Rb.y, Rb.x - Ra.y);
        U2 = mk<float>(Ra.x - Rb.y, Ra.y + Rb.x);
        V2 = mk<float>(Pa.x + Pb.y, Pb.x - Pa.y);
      }
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        C Yn, Yq;
        if (s == 0) {
          Yn = cadd(U, V);
          Yq = cadd(U2, V2);
        } else {
          const C tz = s == 1 ? tz1 : tz2;              // conj(w)
          const C tq = s == 1 ? tq1 : tq2;              // eps w
          Yn = zb_mac(zb_mul(cconj(tz), U), tq, V);
          Yq = zb_mac(zb_mul(U2, cconj(tq)), V2, tz);
        }
        C* dst = A + line(t, s, l) * LS;
        dst[pn] = cconj(Yn);
        if (nq != n) dst[pq] = cconj(Yq);
      }
    }
  }
  // n = 0: H = Re X_0 in every subset; the z derivative of n = 0 is zero
  for (int row = threadIdx.x; row < NTR * L; row += NT) {
    const int t = row / L;
    const int l = row - t * L;
    const bool kind1 = t >= NPAIR;
    C v;
    if (!kind1) {
      const int fa = 2 * t;
      const float pbx = (fa + 1 < KK) ? St[((fa + 1) * L + l) * Q].x : 0.f;
      v = mk<float>(St[(fa * L + l) * Q].x, -pbx);
    } else {
      v = mk<float>(St[((KK + t - NPAIR) * L + l) * Q].x, 0.f);
    }
#pragma unroll
    for (int s = 0; s < 3; ++s) A[line(t, s, l) * LS] = v;
  }
  __syncthreads();

  // ---- P1: backward transforms of every line ----
  zb_stage<Q, R1, 1, NT>(A, Bf, nlines, twQ);
  zb_stage<Q, R2, R1, NT>(Bf, A, nlines, twQ);
  // the second buffer is free: prefetch the next item's rows beyond the part P3 uses
  if (Rn != nullptr) {
    const size_t off = zb_rows_off(smem_bytes, KK, Q, Ln);
    if (off >= (size_t)zb_buf_elems(K0, Q, L) + (size_t)3 * NPAIR * L * (Q + Q / 16))
      zb_stage_rows<K0, Q, NT>(*Rn, x0n, Ln, A + off);
    else if (threadIdx.x == 0)
      atomicOr(err, MWF_DERR_OUTPUT_CAPACITY);
  }

  // ---- P2: the coupling term per point, in registers ----
  const int npts = 3 * L * Q;
  constexpr int L3 = 3 * L;
  for (int e = threadIdx.x; e < npts; e += NT) {
    const int sl = e / Q;                 // s * L + l
    const int q = e - sl * Q;
    float pv[KK], nl[KK];
#pragma unroll
    for (int t = 0; t < NPAIR; ++t) {
      const C v = A[pad_idx<float>((t * L3 + sl) * Q + q)];
      pv[2 * t] = v.x;
      if (2 * t + 1 < KK) pv[2 * t + 1] = -v.y;     // Im of the conjugated result
    }
    if constexpr (K0 == 4) nl_y_4<float>(pv, nl); else nl_y_6<float>(pv, nl);
#pragma unroll
    for (int J = 0; J < KK; ++J) {
      const C v = A[pad_idx<float>(((NPAIR + J) * L3 + sl) * Q + q)];
      nl_xz_rt<K0, float>(J, pv, v.x, -v.y, nl);
    }
#pragma unroll
    for (int t = 0; t < NPAIR; ++t)
      A[pad_idx<float>((t * L3 + sl) * Q + q)] = mk<float>(nl[2 * t], 2 * t + 1 < KK ? nl[2 * t + 1] : 0.f);
  }
  __syncthreads();

  // ---- P3: forward transforms of the products ----
  const int nfl = 3 * NPAIR * L;
  zb_stage<Q, R1, 1, NT>(A, Bf, nfl, twQ);
  zb_stage<Q, R2, R1, NT>(Bf, A, nfl, twQ);

  // ---- P4: split, twiddle, sum over the subsets, write ----
  C* __restrict__ NLT = reinterpret_cast<C*>(R.NLT) + (size_t)x0 * NN;
  auto store = [&](int t, int l, int nn, C a, C b) {
    const size_t o = (size_t)l * NN + nn;
    NLT[(size_t)(2 * t) * fstride + o] = a;
    if (2 * t + 1 < KK) NLT[(size_t)(2 * t + 1) * fstride + o] = b;
  };
  if (worker) {
    for (int row = threadIdx.x / S; row < NPAIR * L; row += RPP) {
      const int t = row / L;
      const int l = row - t * L;
      C An, Bn, Aq, Bq;
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const C* src = A + line(t, s, l) * LS;
        const C gg = src[pn];
        const C gm = src[pq];
        const C As = mk<float>(hscale * (gg.x + gm.x), hscale * (gg.y - gm.y));
        const C Bs = mk<float>(hscale * (gg.y + gm.y), hscale * (gm.x - gg.x));
        if (s == 0) {
          An = As; Bn = Bs; Aq = cconj(As); Bq = cconj(Bs);
        } else {
          const C tz = s == 1 ? tz1 : tz2;
          const C tq = s == 1 ? tq1 : tq2;
          An = zb_mac(An, As, tz);
          Bn = zb_mac(Bn, Bs, tz);
          Aq = zb_mac(Aq, cconj(As), tq);
          Bq = zb_mac(Bq, cconj(Bs), tq);
        }
      }
      store(t, l, n, An, Bn);
      if (nq != n) store(t, l, nq, Aq, Bq);
    }
  }
  // n = 0
  const C tz0 = __ldg(&twZ[0]);
  for (int row = threadIdx.x; row < NPAIR * L; row += NT) {
    const int t = row / L;
    const int l = row - t * L;
    C An, Bn;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const C gg = A[line(t, s, l) * LS];
      const C As = mk<float>(hscale * (gg.x + gg.x), hscale * (gg.y - gg.y));
      const C Bs = mk<float>(hscale * (gg.y + gg.y), hscale * (gg.x - gg.x));
      if (s == 0) {
        An = As; Bn = Bs;
      } else {
        An = zb_mac(An, As, tz0);
        Bn = zb_mac(Bn, Bs, tz0);
      }
    }
    store(t, l, 0, An, Bn);
  }
}

// z_batched_body for the run-time line count L (1 <= L <= zb_lmax).
template <int K0, int Q, int NT, int LT = 1>
__device__ __forceinline__ void z_batched_body_l(int L, const RunDesc& R, int x0, unsigned char* smem_raw,
                                                 unsigned smem_bytes, const RunDesc* Rn, int x0n, int Ln, int* err) {
  if constexpr (LT < zb_lmax(K0, Q)) {
    if (L != LT) {
      z_batched_body_l<K0, Q, NT, LT + 1>(L, R, x0, smem_raw, smem_bytes, Rn, x0n, Ln, err);
      return;
    }
  }
  z_batched_body<K0, Q, NT, LT>(R, x0, smem_raw, smem_bytes, Rn, x0n, Ln, err);
}

// One work item with no prefetch (the persistent step's form).
template <int K0, int Q, int NT>
__device__ __forceinline__ void z_batched_item(const RunDesc& R, const WorkItem& wi, unsigned char* smem_raw,
                                               unsigned smem_bytes, int* err) {
  const int L = zb_item_lines<K0, Q>(R, wi, smem_bytes);
  if (L == 0) return;
  if (L < 0) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_OUTPUT_CAPACITY);
    return;
  }
  zb_stage_rows<K0, Q, NT>(R, wi.a, L,
                           reinterpret_cast<float2*>(smem_raw) + zb_rows_off(smem_bytes, 3 * K0 - 1, Q, L));
  z_batched_body_l<K0, Q, NT>(L, R, wi.a, smem_raw, smem_bytes, nullptr, 0, 0, err);
}

// The batched z pass over n items: each CTA takes items blockIdx.x, + gridDim.x, ... and
// prefetches the input rows of its next item while it works on the current one.
template <int K0, int Q, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) z_batched_kernel(const RunDesc* __restrict__ runs,
                                                             const WorkItem* __restrict__ items, int n, int* err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const unsigned sb = dyn_smem_bytes();
  // the first item at or after `it` that has work (skipping inactive runs, flagging misfits)
  auto next_item = [&](int it, int& L) {
    for (; it < n; it += gridDim.x) {
      L = zb_item_lines<K0, Q>(runs[items[it].run], items[it], sb);
      if (L > 0) break;
      if (L < 0 && threadIdx.x == 0) atomicOr(err, MWF_DERR_OUTPUT_CAPACITY);
    }
    return it;
  };
  int L = 0;
  int it = next_item(blockIdx.x, L);
  if (it >= n) return;
  {
    const WorkItem wi = items[it];
    zb_stage_rows<K0, Q, NT>(runs[wi.run], wi.a, L,
                             reinterpret_cast<float2*>(smem_raw) + zb_rows_off(sb, 3 * K0 - 1, Q, L));
  }
  while (it < n) {
    const WorkItem wi = items[it];
    int Ln = 0;
    const int nx = next_item(it + gridDim.x, Ln);
    const RunDesc* Rn = nx < n ? &runs[items[nx].run] : nullptr;
    z_batched_body_l<K0, Q, NT>(L, runs[wi.run], wi.a, smem_raw, sb, Rn, nx < n ? items[nx].a : 0, Ln, err);
    it = nx;
    L = Ln;
  }
}

}  // namespace mwf
