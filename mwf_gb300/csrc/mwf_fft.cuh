// Shared-memory mixed-radix (2/3/4/8/12/16) Stockham FFT over a batch of lines.
//
// A CTA holds L lines of length N in shared memory (line stride S complex elements, element
// i stored at pad_idx(i)) and transforms them in place.  Each stage loads the radix-R butterfly inputs of this thread
// into registers, synchronises, and writes the butterfly outputs to their auto-sorted
// positions, so no second buffer is needed.  Twiddles come from a per-length table
// tw[t] = exp(-2 pi i t / N) computed on the host in extended precision.
//
// Direction: inv = false gives sum_j x_j e^{-2 pi i jk/N} (FFTW "forward", sign -1);
//            inv = true  gives sum_j x_j e^{+2 pi i jk/N} (FFTW "backward", sign +1).
// Both are unnormalised, like the reference's FFTW plans (transform.fftw5.f90:33-59).
#pragma once
#include "mwf_common.cuh"

namespace mwf {

// x * (-i) for the forward transform, x * (+i) for the inverse.
template <typename C> __device__ __forceinline__ C rot90(C a, bool inv) {
  C r;
  if (inv) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; }
  return r;
}

template <typename T, typename C> __device__ __forceinline__ void dft2(C* v) {
  C a = v[0];
  v[0] = cadd(a, v[1]);
  v[1] = csub(a, v[1]);
}

template <typename T, typename C> __device__ __forceinline__ void dft3(C* v, bool inv) {
  // y1,y2 = a - (b+c)/2 +- i s (b - c),  s = -sqrt(3)/2 forward, +sqrt(3)/2 inverse
  const T s = inv ? T(0.86602540378443864676) : T(-0.86602540378443864676);
  C t1 = cadd(v[1], v[2]);
  C t2 = csub(v[1], v[2]);
  C m;
  if constexpr (sizeof(T) == 4) {         // FP32: explicit rounding (see cmul<float2>)
    m.x = __fmaf_rn(-0.5f, t1.x, v[0].x);
    m.y = __fmaf_rn(-0.5f, t1.y, v[0].y);
  } else {
    m.x = v[0].x - T(0.5) * t1.x;
    m.y = v[0].y - T(0.5) * t1.y;
  }
  C j;
  j.x = -s * t2.y;
  j.y = s * t2.x;
  v[0] = cadd(v[0], t1);
  v[1] = cadd(m, j);
  v[2] = csub(m, j);
}

template <typename T, typename C> __device__ __forceinline__ void dft4(C* v, bool inv) {
  C t0 = cadd(v[0], v[2]);
  C t1 = csub(v[0], v[2]);
  C t2 = cadd(v[1], v[3]);
  C t3 = rot90(csub(v[1], v[3]), inv);
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

// multiply by exp(-+ i pi/4) = (1 -+ i)/sqrt(2)
template <typename T, typename C> __device__ __forceinline__ C w8(C a, bool inv) {
  const T h = T(0.70710678118654752440);
  C r;
  if (inv) { r.x = h * (a.x - a.y); r.y = h * (a.x + a.y); }
  else     { r.x = h * (a.x + a.y); r.y = h * (a.y - a.x); }
  return r;
}

template <typename T, typename C> __device__ __forceinline__ void dft8(C* v, bool inv) {
  C e[4] = {v[0], v[2], v[4], v[6]};
  C o[4] = {v[1], v[3], v[5], v[7]};
  dft4<T>(e, inv);
  dft4<T>(o, inv);
  o[1] = w8<T>(o[1], inv);
  o[2] = rot90(o[2], inv);
  o[3] = rot90(w8<T>(o[3], inv), inv);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}

// multiply by (c - i s) forward or (c + i s) inverse: the twiddle e^{-+ i theta}, c = cos, s = sin
template <typename T, typename C> __device__ __forceinline__ C wmul(C a, T c, T s, bool inv) {
  const T sn = inv ? s : -s;
  C r;
  if constexpr (sizeof(T) == 4) {         // FP32: explicit rounding (see cmul<float2>)
    r.x = __fmaf_rn(a.x, c, -__fmul_rn(a.y, sn));
    r.y = __fmaf_rn(a.x, sn, __fmul_rn(a.y, c));
  } else {
    r.x = a.x * c - a.y * sn;
    r.y = a.x * sn + a.y * c;
  }
  return r;
}

// 16 = 4 x 4: four length-4 transforms over n1 (x[4 n1 + n2]), twiddles W16^{n2 k1}, four
// length-4 transforms over n2; output X[k1 + 4 k2] in natural order.
template <typename T, typename C> __device__ __forceinline__ void dft16(C* v, bool inv) {
  const T c1 = T(0.92387953251128675613), s1 = T(0.38268343236508977173);   // cos, sin(pi/8)
  const T h = T(0.70710678118654752440);
  C y[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    C t[4] = {v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]};
    dft4<T>(t, inv);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) y[n2][k1] = t[k1];
  }
  // twiddles W16^{n2 k1}: exponents 1,2,3 (n2=1), 2,4,6 (n2=2), 3,6,9 (n2=3)
  y[1][1] = wmul<T>(y[1][1], c1, s1, inv);
  y[1][2] = wmul<T>(y[1][2], h, h, inv);
  y[1][3] = wmul<T>(y[1][3], s1, c1, inv);
  y[2][1] = wmul<T>(y[2][1], h, h, inv);
  y[2][2] = rot90(y[2][2], inv);
  y[2][3] = wmul<T>(y[2][3], -h, h, inv);
  y[3][1] = wmul<T>(y[3][1], s1, c1, inv);
  y[3][2] = wmul<T>(y[3][2], -h, h, inv);
  y[3][3] = wmul<T>(y[3][3], -c1, -s1, inv);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    C t[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
    dft4<T>(t, inv);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
  }
}

// 12 = 3 x 4: four length-3 transforms over n1 (x[4 n1 + n2]), twiddles W12^{n2 k1}, three
// length-4 transforms over n2; output X[k1 + 3 k2] in natural order.
template <typename T, typename C> __device__ __forceinline__ void dft12(C* v, bool inv) {
  const T r3 = T(0.86602540378443864676);
  C y[4][3];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    C t[3] = {v[n2], v[n2 + 4], v[n2 + 8]};
    dft3<T>(t, inv);
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) y[n2][k1] = t[k1];
  }
  // W12^1 = (r3, 1/2), W12^2 = (1/2, r3), W12^3 = -i, W12^4 = (-1/2, r3), W12^6 = -1
  y[1][1] = wmul<T>(y[1][1], r3, T(0.5), inv);
  y[1][2] = wmul<T>(y[1][2], T(0.5), r3, inv);
  y[2][1] = wmul<T>(y[2][1], T(0.5), r3, inv);
  y[2][2] = wmul<T>(y[2][2], T(-0.5), r3, inv);
  y[3][1] = rot90(y[3][1], inv);
  y[3][2] = mk<T>(-y[3][2].x, -y[3][2].y);
#pragma unroll
  for (int k1 = 0; k1 < 3; ++k1) {
    C t[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
    dft4<T>(t, inv);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 3 * k2] = t[k2];
  }
}

template <typename T, int R> __device__ __forceinline__ void dftR(cx<T>* v, bool inv) {
  if constexpr (R == 2) dft2<T>(v);
  else if constexpr (R == 3) dft3<T>(v, inv);
  else if constexpr (R == 4) dft4<T>(v, inv);
  else if constexpr (R == 8) dft8<T>(v, inv);
  else if constexpr (R == 12) dft12<T>(v, inv);
  else dft16<T>(v, inv);
}

// One Stockham stage of radix R over L lines.  IT = butterflies per thread (compile time).
// The caller guarantees L*N/R <= IT*blockDim.
template <typename T, int R, int IT>
__device__ __forceinline__ void fft_stage(cx<T>* buf, int base, int L, int S, int N, int Ns, FastDiv fnb,
                                          FastDiv fns, const cx<T>* __restrict__ tw, bool inv) {
  using C = cx<T>;
  const int nb = N / R;
  const int total = L * nb;
  const int tstep = N / (Ns * R);
  C v[IT][R];
  int dst[IT];
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    const int b = threadIdx.x + it * blockDim.x;
    dst[it] = -1;
    if (b < total) {
      const int line = fnb.div(b);
      const int j = b - line * nb;
      const int src = base + line * S + j;
#pragma unroll
      for (int r = 0; r < R; ++r) v[it][r] = buf[pad_idx<T>(src + r * nb)];
      const int k = j - fns.div(j) * Ns;
      if (Ns > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          C w = __ldg(&tw[k * r * tstep]);
          v[it][r] = inv ? cmulc(v[it][r], w) : cmul(v[it][r], w);
        }
      }
      dftR<T, R>(v[it], inv);
      dst[it] = base + line * S + (j - k) * R + k;
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    if (dst[it] >= 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) buf[pad_idx<T>(dst[it] + r * Ns)] = v[it][r];
    }
  }
  __syncthreads();
}

// Transform L lines of length pl.N in place, line l starting at element base + l*S.
// VPT = complex values per thread the caller
// guarantees: L*N <= VPT*blockDim.  A radix-R stage then needs ceil(VPT/R) butterflies per
// thread.  On a capacity violation the lines are left untransformed and *err gets a flag.
template <typename T, int VPT, int MAXR = 16>
__device__ __forceinline__ void fft_lines_inl(cx<T>* buf, int base, int L, int S, const FftPlanDev& pl,
                                              const cx<T>* __restrict__ tw, bool inv, int* err) {
  __syncthreads();
  if (L * pl.N > VPT * (int)blockDim.x) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_FFT_CAPACITY);
    return;
  }
  for (int s = 0; s < pl.nst; ++s) {
    const int R = pl.radix[s];
    const int Ns = pl.ns[s];
    switch (R) {
      case 16:
        if constexpr (MAXR >= 16) { fft_stage<T, 16, (VPT + 15) / 16>(buf, base, L, S, pl.N, Ns, pl.fnb[s], pl.fns[s], tw, inv); break; }
        else { if (threadIdx.x == 0) atomicOr(err, MWF_DERR_BAD_RADIX); return; }
      case 12:
        if constexpr (MAXR >= 12) { fft_stage<T, 12, (VPT + 11) / 12>(buf, base, L, S, pl.N, Ns, pl.fnb[s], pl.fns[s], tw, inv); break; }
        else { if (threadIdx.x == 0) atomicOr(err, MWF_DERR_BAD_RADIX); return; }
      case 8: fft_stage<T, 8, (VPT + 7) / 8>(buf, base, L, S, pl.N, Ns, pl.fnb[s], pl.fns[s], tw, inv); break;
      case 4: fft_stage<T, 4, (VPT + 3) / 4>(buf, base, L, S, pl.N, Ns, pl.fnb[s], pl.fns[s], tw, inv); break;
      case 3: fft_stage<T, 3, (VPT + 2) / 3>(buf, base, L, S, pl.N, Ns, pl.fnb[s], pl.fns[s], tw, inv); break;
      case 2: fft_stage<T, 2, (VPT + 1) / 2>(buf, base, L, S, pl.N, Ns, pl.fnb[s], pl.fns[s], tw, inv); break;
      default:
        if (threadIdx.x == 0) atomicOr(err, MWF_DERR_BAD_RADIX);
        return;
    }
  }
}

// One Stockham stage with compile-time length N, radix R and span NS (the product of the
// earlier radices): every index division, the twiddle stride N/(NS R) and the loop bounds are
// constants.  L lines of stride N starting at element base; NT = block size.  As in fft_stage,
// each thread first loads all of its IT = ceil(VPT/R) butterflies, then the block synchronises,
// then the outputs are stored (the stage is in place); the caller guarantees L N <= VPT NT.
template <typename T, int N, int R, int NS, int NT, int VPT>
__device__ __forceinline__ void fixed_stage(cx<T>* buf, int base, int L, const cx<T>* __restrict__ tw) {
  using C = cx<T>;
  constexpr int B = N / R, TSTEP = N / (NS * R), IT = (VPT + R - 1) / R;
  const int tot = L * B;
  C v[IT][R];
  int dst[IT];
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    const int b = threadIdx.x + it * NT;
    dst[it] = -1;
    if (b < tot) {
      const int line = b / B, j = b - line * B;
      const int k = j % NS;
      const int src = base + line * N + j;
#pragma unroll
      for (int r = 0; r < R; ++r) v[it][r] = buf[pad_idx<T>(src + r * B)];
      if constexpr (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[it][r] = cmul(v[it][r], __ldg(&tw[r * k * TSTEP]));
      }
      dftR<T, R>(v[it], false);
      dst[it] = base + line * N + (j - k) * R + k;
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    if (dst[it] >= 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) buf[pad_idx<T>(dst[it] + r * NS)] = v[it][r];
    }
  }
  __syncthreads();
}

// Forward transform of L lines of compile-time length N = R1 R2 R3 (R3 = 1: two stages; line
// stride N, from element base) as compile-time Stockham stages: the same butterflies as
// fft_lines_inl with the plan {R1, R2, R3} (identical results) in about two thirds of the
// instructions.  NT = block size, VPT = values per thread the caller's buffer holds at most
// (L N <= VPT NT; otherwise the lines are left untransformed and *err gets a flag).
template <typename T, int N, int R1, int R2, int R3, int NT, int VPT>
__device__ __forceinline__ void fft_lines_fixed(cx<T>* buf, int base, int L, const cx<T>* __restrict__ tw, int* err) {
  static_assert(N == R1 * R2 * R3, "N = R1 R2 R3");
  __syncthreads();
  if (L * N > VPT * NT) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_FFT_CAPACITY);
    return;
  }
  fixed_stage<T, N, R1, 1, NT, VPT>(buf, base, L, tw);
  fixed_stage<T, N, R2, R1, NT, VPT>(buf, base, L, tw);
  if constexpr (R3 > 1) fixed_stage<T, N, R3, R1 * R2, NT, VPT>(buf, base, L, tw);
}

// fixed_stage out of place: butterflies read from `in` and are written to `out` one at a
// time (no registers held across a barrier), then the block synchronises once.
template <typename T, int N, int R, int NS, int NT, int VPT>
__device__ __forceinline__ void fixed_stage_oop(const cx<T>* in, cx<T>* out, int base, int L,
                                                const cx<T>* __restrict__ tw) {
  using C = cx<T>;
  constexpr int B = N / R, TSTEP = N / (NS * R), IT = (VPT + R - 1) / R;
  const int tot = L * B;
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    const int b = threadIdx.x + it * NT;
    if (b < tot) {
      const int line = b / B, j = b - line * B;
      const int k = j % NS;
      const int src = base + line * N + j;
      C v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = in[pad_idx<T>(src + r * B)];
      if constexpr (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(&tw[r * k * TSTEP]));
      }
      dftR<T, R>(v, false);
      const int dst = base + line * N + (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) out[pad_idx<T>(dst + r * NS)] = v[r];
    }
  }
  __syncthreads();
}

// Two-stage compile-time transform (N = R1 R2) through a second buffer: a -> b -> a, the
// result back in a, with one barrier per stage where the in-place form needs two.  b holds
// as many padded elements as a; same results as fft_lines_fixed<T, N, R1, R2, 1, ...>.
template <typename T, int N, int R1, int R2, int NT, int VPT>
__device__ __forceinline__ void fft_lines_fixed_pp(cx<T>* a, cx<T>* b, int base, int L, const cx<T>* __restrict__ tw,
                                                   int* err) {
  static_assert(N == R1 * R2, "N = R1 R2");
  __syncthreads();
  if (L * N > VPT * NT) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_FFT_CAPACITY);
    return;
  }
  fixed_stage_oop<T, N, R1, 1, NT, VPT>(a, b, base, L, tw);
  fixed_stage_oop<T, N, R2, R1, NT, VPT>(b, a, base, L, tw);
}

// Out-of-line copy for kernels that call the transform from many places.
template <typename T, int VPT, int MAXR = 16>
__device__ __noinline__ void fft_lines(cx<T>* buf, int L, int S, const FftPlanDev& pl,
                                       const cx<T>* __restrict__ tw, bool inv, int* err) {
  fft_lines_inl<T, VPT, MAXR>(buf, 0, L, S, pl, tw, inv, err);
}

}  // namespace mwf
