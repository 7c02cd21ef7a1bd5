// FP32 x passes with the x transforms split into three interleaved subsets (sm_103a).
//
// An x line holds X = 3MM points.  Its spectrum is non-zero only for |m| <= MM-1, so the
// backward transform of the x-forward pass (tra_spec2phys x part, transform.fftw5.f90:69-78)
// restricted to the points x = s + 3q (s = 0, 1, 2, q < MM) is a length-MM transform:
//   X_{s+3q} = sum_j D_j^(s) e^{+2 pi i jq/MM},
//   D_j^(s) = c_j e^{+2 pi i js/X} + c_{j-MM} e^{+2 pi i (j-MM)s/X}   (j >= 1;  D_0^(s) = c_0),
// and the forward transform of the x-inverse pass (tra_phys2spec x part,
// transform.fftw5.f90:136-144) is, for the kept wavenumbers |m| <= MM-1,
//   Y_m = sum_s e^{-2 pi i ms/X} F_s[m mod MM],   F_s = forward length-MM transform of x = s + 3q.
// So both passes run length-MM transforms, whose plans for the usual sizes are two compile-time
// stages (the length-3MM lines need three), out of place between two shared-memory buffers with
// one barrier per stage.  Inputs are staged in shared memory by asynchronous copies, all in
// flight at once, before any arithmetic.  The column count of an item is a compile-time
// parameter of its body (every count an item can hold, dispatched at run time).  The x-forward
// launch is one wave of resident CTAs, kXfBlocks per SM, that copy their next item's MPT rows
// while they transform the current one; the x inverse runs one CTA per item, kXiBlocks per SM.
//
// x forward: item (run, first column n0, wall-normal mode k < K0): the fields u_k, v_k (k >= 1),
//   w_k (var_mpt2spec + vel_addlam, variables.f90:390-434, velocity.f90:76-82) and their x
//   derivatives (var_spec_grad, variables.f90:600-612) for nb columns, one after the other from
//   one staged copy of the MPT rows psi_k, phi_k; writes T[fs] and T[KK + fs] of each.
// x inverse: item (run, first column n0, wall-normal mode k): u_k, v_k, w_k of nb columns, then
//   var_spec2mpt (variables.f90:440-480) and the AB2 / implicit update (vel_TS, velocity.f90:21-41)
//   as in x_inverse_kernel's FP32 form.
#pragma once
#include "mwf_common.cuh"
#include "mwf_fft.cuh"
#include "mwf_zbatch.cuh"

namespace mwf {

// Padded element count of a buffer of n complex values, rounded to an even count so the next
// buffer starts on a 16-byte boundary.
__host__ __device__ constexpr size_t xb_pad_elems(size_t n) { return (n + (n >> 4) + 2) & ~(size_t)1; }

// x forward: A, B of 6 nb lines of MM (field and derivative, three subsets each) and the staged
// MPT rows (two slots of nb columns of M = 2MM-1 values).
__host__ __device__ constexpr size_t xbf_smem_bytes(int MM, int nb) {
  return 8 * (2 * xb_pad_elems((size_t)6 * nb * MM) + (size_t)2 * nb * (2 * MM - 1));
}
// x inverse: A, B of 9 nb lines of MM (three fields, three subsets each); the rows of the
// nonlinear term are staged straight into A.
__host__ __device__ constexpr size_t xbi_smem_bytes(int MM, int nb) { return 8 * 2 * xb_pad_elems((size_t)9 * nb * MM); }

// The most columns an x-forward / x-inverse item holds at kXfBlocks / kXiBlocks CTAs per SM (at
// most 8).
__host__ __device__ constexpr int xbf_nbmax(int MM) {
  int nb = 1;
  while (nb < 8 && xbf_smem_bytes(MM, nb + 1) <= zb_smem_budget(kXfBlocks)) ++nb;
  return nb;
}
__host__ __device__ constexpr int xbi_nbmax(int MM) {
  int nb = 1;
  while (nb < 8 && xbi_smem_bytes(MM, nb + 1) <= zb_smem_budget(kXiBlocks)) ++nb;
  return nb;
}

// Columns of x-forward item wi of run R in a CTA with smem_bytes of shared memory: nb >= 1, 0 for
// an inactive run, -1 if the item does not fit (an internal error).
template <int MM>
__device__ __forceinline__ int xf_item_cols(const RunDesc& R, const WorkItem& wi, unsigned smem_bytes) {
  if (!R.active) return 0;
  const int nb = min(R.xbf_nb, R.NN - wi.a);
  if (R.MM != MM || nb < 1 || nb > xbf_nbmax(MM) || wi.b >= R.K0 || xbf_smem_bytes(MM, nb) > smem_bytes) return -1;
  return nb;
}

// An x-forward item (column block, wall-normal mode k) writes the fields u_k, v_k (k >= 1) and w_k
// (var_mpt2spec order; x-forward field index k, K0 - 1 + k and 2 K0 - 1 + k) and their x
// derivatives, all from one staged copy of the MPT slots psi_k (q = 0) and, for k >= 1, phi_k
// (q = 1): v reads phi_k; u and w read psi_k and phi_k.

// Complex offset of the staged MPT rows of an x-forward item of nb columns: the last 2 nb M
// complex values of the CTA's shared memory (8-byte copies), beyond both buffers of any item
// that fits.
__device__ __forceinline__ size_t xf_rows_off(unsigned smem_bytes, int M, int nb) {
  return (size_t)(smem_bytes / 8) - (size_t)2 * nb * M;
}

// Issue the asynchronous copies of the MPT rows c[n0 + l][slot][0 .. M-1] of x-forward item wi
// (nb columns; slot k, then k + K0 - 1 for k >= 1) to S[(q nb + l) M + ms]; one commit group.
template <int MM, int NT>
__device__ __forceinline__ void xf_stage_rows(const RunDesc& R, const WorkItem& wi, int nb, float2* S) {
  constexpr int M = 2 * MM - 1;
  const int K = R.K, K0 = R.K0, n0 = wi.a, k = wi.b;
  const float2* __restrict__ c = reinterpret_cast<const float2*>(R.c);
  for (int q = 0; q < (k >= 1 ? 2 : 1); ++q) {
    const int slot = q ? k + K0 - 1 : k;
    for (int e = threadIdx.x; e < nb * M; e += NT) {
      const int l = e / M;
      const int ms = e - l * M;
      cp_async<8>(S + (q * nb + l) * M + ms, c + ((size_t)(n0 + l) * K + slot) * M + ms);
    }
  }
  cp_async_commit();
}

// One x-forward work item (nb columns), run by the whole CTA (NT threads) in smem_raw
// (smem_bytes in all), whose MPT rows are in flight (xf_stage_rows, the CTA's only open commit
// group) at xf_rows_off.  If Rn is not null, the rows of the next item (run *Rn, item *win, nbn
// columns) are prefetched once the last field's fill is done.  The caller synchronises the CTA before it
// reuses the shared memory otherwise.
template <int MM, int NT, int nb>
__device__ __forceinline__ void xf_batched_body(const RunDesc& R, const WorkItem& wi, unsigned char* smem_raw,
                                                unsigned smem_bytes, const RunDesc* Rn, const WorkItem* win,
                                                int nbn, int* err) {
  using C = float2;
  constexpr int X = 3 * MM, M = 2 * MM - 1;
  constexpr int R1 = ZbPlan<MM>::R1, R2 = ZbPlan<MM>::R2;
  const int NN = R.NN, KK = R.KK, K0 = R.K0;
  const int n0 = wi.a;
  const int k = wi.b;
  constexpr int nl = 6 * nb;                  // line (d, s, l) = (d * 3 + s) * nb + l; d = 1: derivative
  C* A = reinterpret_cast<C*>(smem_raw);
  C* Bf = A + xb_pad_elems((size_t)nl * MM);
  const C* S = A + xf_rows_off(smem_bytes, M, nb);
  cp_async_wait<0>();
  __syncthreads();

  const C* __restrict__ twX = reinterpret_cast<const C*>(R.twX);
  const float k1 = kbeta<float>(k);
  const bool addlam = wi.pad == 0;
  const int ncomp = k >= 1 ? 3 : 2;           // v_0 does not exist
  for (int ci = 0; ci < ncomp; ++ci) {
    const int comp = (k == 0 && ci == 1) ? 2 : ci;
    const int fs = comp == 0 ? k : (comp == 1 ? K0 - 1 + k : 2 * K0 - 1 + k);
    const int aq = comp == 1 ? 1 : 0;           // v reads phi_k, u and w psi_k (and phi_k as b)
    const bool hasb = comp != 1 && k >= 1;
    // fill: one unit per (column l, folded index j); two field values give the three subsets'
    // inputs of the field and of its derivative.  ep[s-1] = e^{+2 pi i js/X} and
    // en[s-1] = e^{+2 pi i (j-MM)s/X} (conjugates of the table at js and at X + (j-MM)s, i.e.
    // 2MM + j for s = 1 and MM + 2j for s = 2).
    auto unit = [&](int l, int j, float m1p, float m1n, const C (&ep)[2], const C (&en)[2]) {
      const int n = n0 + l;
      const float n1 = wavenum<float>(R.gamma, R.gamma_f, n);
      auto field = [&](int m, float m1) -> C {
        const int ms = m < 0 ? m + M : m;
        const C a = S[(aq * nb + l) * M + ms];
        const C b = hasb ? S[(nb + l) * M + ms] : mk<float>(0.f, 0.f);
        float re, im;
        if (m == 0 && n == 0) {             // mean flows: u_k = psi_k, w_k = phi_k (k >= 1)
          re = 0.f; im = 0.f;
          if (comp == 0 && k >= 1) { re = a.x; im = a.y; }
          if (comp == 2 && k >= 1) { re = b.x; im = b.y; }
          if (addlam && k == 1) {
            if (comp == 0) re += (float)R.cth;
            if (comp == 2) re += (float)R.sth;
          }
          return mk<float>(re, im);
        }
        // (roundings spelled out, see cmul<float2>)
        if (comp == 1) {
          const float H = __fmaf_rn(-m1, m1, -__fmul_rn(n1, n1));
          re = -a.x * H;
          im = -a.y * H;
        } else if (comp == 0) {
          re = -__fmaf_rn(-a.y, n1, __fmul_rn(__fmul_rn(b.y, k1), m1));
          im = __fmaf_rn(-a.x, n1, __fmul_rn(__fmul_rn(b.x, k1), m1));
        } else {
          re = -__fmaf_rn(a.y, m1, __fmul_rn(__fmul_rn(b.y, k1), n1));
          im = __fmaf_rn(a.x, m1, __fmul_rn(__fmul_rn(b.x, k1), n1));
        }
        return mk<float>(re, im);
      };
      const C v = field(j, m1p);
      const C dv = mk<float>(-v.y * m1p, v.x * m1p);
      if (j == 0) {
#pragma unroll
        for (int s = 0; s < 3; ++s) {
          A[pad_idx<float>((s * nb + l) * MM)] = cconj(v);
          A[pad_idx<float>(((3 + s) * nb + l) * MM)] = cconj(dv);
        }
        return;
      }
      const C w = field(j - MM, m1n);
      const C dw = mk<float>(-w.y * m1n, w.x * m1n);
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        C D, dD;
        if (s == 0) {
          D = cadd(v, w);
          dD = cadd(dv, dw);
        } else {
          D = cadd(cmul(v, ep[s - 1]), cmul(w, en[s - 1]));
          dD = cadd(cmul(dv, ep[s - 1]), cmul(dw, en[s - 1]));
        }
        // backward transform as conj(forward(conj .)): store the conjugate
        A[pad_idx<float>((s * nb + l) * MM + j)] = cconj(D);
        A[pad_idx<float>(((3 + s) * nb + l) * MM + j)] = cconj(dD);
      }
    };
    auto twiddles = [&](int j, C (&ep)[2], C (&en)[2]) {
      ep[0] = cconj(__ldg(&twX[j]));
      ep[1] = cconj(__ldg(&twX[2 * j]));
      en[0] = cconj(__ldg(&twX[2 * MM + j]));
      en[1] = cconj(__ldg(&twX[MM + 2 * j]));
    };
    if constexpr (NT % MM == 0) {
      // a thread keeps one j, its wavenumbers and twiddles, over the columns it visits
      const int j = threadIdx.x % MM;
      const float m1p = wavenum<float>(R.alpha, R.alpha_f, j);
      const float m1n = wavenum<float>(R.alpha, R.alpha_f, j - MM);
      C ep[2], en[2];
      twiddles(j, ep, en);
      for (int l = threadIdx.x / MM; l < nb; l += NT / MM) unit(l, j, m1p, m1n, ep, en);
    } else {
      for (int e = threadIdx.x; e < nb * MM; e += NT) {
        const int l = e / MM;
        const int j = e - l * MM;
        C ep[2], en[2];
        twiddles(j, ep, en);
        unit(l, j, wavenum<float>(R.alpha, R.alpha_f, j), wavenum<float>(R.alpha, R.alpha_f, j - MM), ep, en);
      }
    }
    __syncthreads();
    // after the last field's fill the staged rows are consumed: prefetch the next item's beyond
    // both buffers
    if (ci == ncomp - 1 && Rn != nullptr) {
      const size_t off = xf_rows_off(smem_bytes, M, nbn);
      if (off >= 2 * xb_pad_elems((size_t)nl * MM))
        xf_stage_rows<MM, NT>(*Rn, *win, nbn, A + off);
      else if (threadIdx.x == 0)
        atomicOr(err, MWF_DERR_OUTPUT_CAPACITY);
    }
    zb_stage<MM, R1, 1, NT, 3>(A, Bf, nl, twX);
    zb_stage<MM, R2, R1, NT, 3>(Bf, A, nl, twX);
    // store T[d KK + fs][s + 3q][n0 + l]: consecutive threads -> consecutive columns, then
    // consecutive q of one subset s, so the shared-memory reads of a half-warp fall on distinct
    // banks or at most two ways (the lines of the three subsets share a bank offset)
    C* __restrict__ out = reinterpret_cast<C*>(R.T);
    const size_t fstride = (size_t)X * NN;
    for (int e = threadIdx.x; e < X * nb; e += NT) {
      const int sq = e / nb;                      // s MM + q
      const int l = e - sq * nb;
      const int s = sq / MM;
      const int q = sq - s * MM;
      const int x = s + 3 * q;
#pragma unroll
      for (int d = 0; d < 2; ++d)
        out[(size_t)(d * KK + fs) * fstride + (size_t)x * NN + n0 + l] = cconj(A[pad_idx<float>(((d * 3 + s) * nb + l) * MM + q)]);
    }
    if (ci < ncomp - 1) __syncthreads();       // the next field's fill overwrites A
  }
}

// xf_batched_body for the run-time column count nb (1 <= nb <= xbf_nbmax).
template <int MM, int NT, int NBT = 1>
__device__ __forceinline__ void xf_batched_body_nb(int nb, const RunDesc& R, const WorkItem& wi, unsigned char* smem_raw,
                                                   unsigned smem_bytes, const RunDesc* Rn, const WorkItem* win,
                                                   int nbn, int* err) {
  if constexpr (NBT < xbf_nbmax(MM)) {
    if (nb != NBT) {
      xf_batched_body_nb<MM, NT, NBT + 1>(nb, R, wi, smem_raw, smem_bytes, Rn, win, nbn, err);
      return;
    }
  }
  xf_batched_body<MM, NT, NBT>(R, wi, smem_raw, smem_bytes, Rn, win, nbn, err);
}

// One x-forward work item with no prefetch (the persistent step's form).
template <int MM, int NT>
__device__ __forceinline__ void xf_batched_item(const RunDesc& R, const WorkItem& wi, unsigned char* smem_raw,
                                                unsigned smem_bytes, int* err) {
  const int nb = xf_item_cols<MM>(R, wi, smem_bytes);
  if (nb == 0) return;
  if (nb < 0) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_OUTPUT_CAPACITY);
    return;
  }
  xf_stage_rows<MM, NT>(R, wi, nb, reinterpret_cast<float2*>(smem_raw) + xf_rows_off(smem_bytes, 2 * MM - 1, nb));
  xf_batched_body_nb<MM, NT>(nb, R, wi, smem_raw, smem_bytes, nullptr, nullptr, 0, err);
}

// The first item at or after `it` (stride gridDim.x) with work, its width in w; items of
// inactive runs are skipped and items that do not fit are flagged.
template <typename F>
__device__ __forceinline__ int xb_next_item(int it, int n, int& w, F width, int* err) {
  for (; it < n; it += gridDim.x) {
    w = width(it);
    if (w > 0) break;
    if (w < 0 && threadIdx.x == 0) atomicOr(err, MWF_DERR_OUTPUT_CAPACITY);
  }
  return it;
}

// The x-forward pass over n items: each CTA takes items blockIdx.x, + gridDim.x, ... and
// prefetches the MPT rows of its next item while it transforms the current one.
template <int MM, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) xf_batched_kernel(const RunDesc* __restrict__ runs,
                                                              const WorkItem* __restrict__ items, int n, int* err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const unsigned sb = dyn_smem_bytes();
  auto width = [&](int i) { return xf_item_cols<MM>(runs[items[i].run], items[i], sb); };
  int nb = 0;
  int it = xb_next_item(blockIdx.x, n, nb, width, err);
  if (it >= n) return;
  {
    const WorkItem wi = items[it];
    xf_stage_rows<MM, NT>(runs[wi.run], wi, nb, reinterpret_cast<float2*>(smem_raw) + xf_rows_off(sb, 2 * MM - 1, nb));
  }
  while (it < n) {
    const WorkItem wi = items[it];
    int nbn = 0;
    const int nx = xb_next_item(it + gridDim.x, n, nbn, width, err);
    WorkItem win{};
    if (nx < n) win = items[nx];
    xf_batched_body_nb<MM, NT>(nb, runs[wi.run], wi, smem_raw, sb, nx < n ? &runs[win.run] : nullptr, &win, nbn, err);
    it = nx;
    nb = nbn;
  }
}

// Columns of x-inverse item wi of run R (see xf_item_cols); the nonlinear term must be the summed
// z output (one partial).
template <int MM>
__device__ __forceinline__ int xi_item_cols(const RunDesc& R, const WorkItem& wi, unsigned smem_bytes) {
  if (!R.active) return 0;
  const int nb = min(R.xbi_nb, R.NN - wi.a);
  if (R.MM != MM || nb < 1 || nb > xbi_nbmax(MM) || wi.b >= R.K0 || !R.z_sum || xbi_smem_bytes(MM, nb) > smem_bytes)
    return -1;
  return nb;
}

// Issue the asynchronous copies of the rows NLT[f][x][n0 .. n0+nb-1] of the three fields u_k,
// v_k, w_k of x-inverse item wi straight into the subset lines of the first buffer:
// A[(comp, s, l)][q] = row (comp, x = s + 3q), column l, at its padded index (v_0 does not exist:
// its lines are zeroed); one commit group.  (Staging the update's operands, c, onl and the tables, the same way measured slower:
// they narrow the item to fit three CTAs per SM, and their small copies cost more than the
// latency they hide.)
template <int MM, int NT, int nb>
__device__ __forceinline__ void xi_stage_rows(const RunDesc& R, const WorkItem& wi, float2* A) {
  constexpr int X = 3 * MM;
  const int NN = R.NN, K0 = R.K0, k = wi.b, n0 = wi.a;
  const float2* __restrict__ NLT = reinterpret_cast<const float2*>(R.NLT);
  const size_t fstride = (size_t)X * NN;
  for (int e = threadIdx.x; e < 3 * X * nb; e += NT) {
    const int row = e / nb;
    const int l = e - row * nb;
    const int comp = row / X;
    const int x = row - comp * X;
    const int q = x / 3;
    const int s = x - 3 * q;
    float2* dst = A + pad_idx<float>(((comp * 3 + s) * nb + l) * MM + q);
    if (comp == 1 && k == 0) {
      *dst = make_float2(0.f, 0.f);
      continue;
    }
    const int f = comp == 0 ? k : (comp == 1 ? K0 + k - 1 : 2 * K0 - 1 + k);   // u_k, v_k, w_k
    cp_async<8>(dst, NLT + (size_t)f * fstride + (size_t)x * NN + n0 + l);
  }
  cp_async_commit();
}

// One x-inverse work item (nb columns), run by the whole CTA (NT threads) in smem_raw
// (smem_bytes in all), whose inputs are in flight (xi_stage_rows, the CTA's only open commit
// group).  The caller synchronises the CTA before it reuses the shared memory.
template <int MM, int NT, int nb>
__device__ __forceinline__ void xi_batched_body(const RunDesc& R, const WorkItem& wi, unsigned char* smem_raw) {
  using C = float2;
  constexpr int X = 3 * MM, M = 2 * MM - 1;
  constexpr int R1 = ZbPlan<MM>::R1, R2 = ZbPlan<MM>::R2;
  const int NN = R.NN, K0 = R.K0, K = R.K;
  const int n0 = wi.a;
  const int k = wi.b;
  constexpr int nl = 9 * nb;                  // line (comp, s, l) = (comp * 3 + s) * nb + l
  C* A = reinterpret_cast<C*>(smem_raw);
  C* Bf = A + xb_pad_elems((size_t)nl * MM);
  cp_async_wait<0>();
  __syncthreads();
  const C* __restrict__ twX = reinterpret_cast<const C*>(R.twX);
  zb_stage<MM, R1, 1, NT, 3>(A, Bf, nl, twX);
  zb_stage<MM, R2, R1, NT, 3>(Bf, A, nl, twX);

  // combine the subsets, var_spec2mpt and the update c' = A c + B (3 nl - onl) with A = rhs/lhs
  // (a float pair) and B = (dt/2)/lhs formed in FP64 by the host (see x_inverse_kernel)
  C* __restrict__ c = reinterpret_cast<C*>(R.c);
  C* __restrict__ onl = reinterpret_cast<C*>(R.onl);
  const size_t csz = (size_t)NN * K * M;
  const float* __restrict__ a_hi = reinterpret_cast<const float*>(R.inv_lhs);
  const float* __restrict__ a_lo = a_hi + csz;
  const float* __restrict__ bnl = reinterpret_cast<const float*>(R.rhs);
  const bool first32 = *R.nst != 0;
  const float kb1 = kbeta<float>(k);
  // the wavenumber scales in registers: the loop's stores to c and onl could alias the run
  // descriptor as far as the compiler knows, so reading them there reloads them every output
  const float alpha_f = R.alpha_f, gamma_f = R.gamma_f;
  // one output per (column l, slot ms): per column the row offsets of both MPT slots are fixed,
  // and the column's subset lines sit at constant offsets from its element j (MM is a multiple
  // of 16, so the padded index of line L, element j is L LS + pad_idx(j))
  constexpr int LS = MM + MM / 16;
  const int slot0 = k, slot1 = k + K0 - 1;
  auto output = [&](int l, int ms) {
    const int n = n0 + l;
    const size_t r0 = ((size_t)n * K + slot0) * M, r1 = ((size_t)n * K + slot1) * M;
    const float n1 = wavenum<float>(0.0, gamma_f, n);
    const C* __restrict__ Al = A + l * LS;
    const int m = signed_m(ms, MM, M);
    // the state, history and tables of both slots first, so their loads overlap the rest
    const size_t i0 = r0 + ms;
    const size_t i1 = r1 + ms;
    const C c0 = c[i0], o0 = onl[i0];
    const float ah0 = a_hi[i0], al0 = a_lo[i0], b0 = bnl[i0];
    C c1 = mk<float>(0.f, 0.f), o1 = c1;
    float ah1 = 0.f, al1 = 0.f, b1 = 0.f;
    if (k > 0) {
      c1 = c[i1]; o1 = onl[i1];
      ah1 = a_hi[i1]; al1 = a_lo[i1]; b1 = bnl[i1];
    }
    const int j = m >= 0 ? m : m + MM;
    const C w1 = __ldg(&twX[m >= 0 ? m : m + X]);              // e^{-2 pi i m/X}
    const C w2 = __ldg(&twX[m >= 0 ? 2 * m : 2 * m + X]);      // e^{-2 pi i 2m/X}
    const C* __restrict__ Aj = Al + pad_idx<float>(j);
    C sp[3];
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      const C F0 = Aj[(comp * 3 * nb) * LS];
      const C F1 = Aj[(comp * 3 * nb + nb) * LS];
      const C F2 = Aj[(comp * 3 * nb + 2 * nb) * LS];
      sp[comp] = cadd(cadd(F0, cmul(F1, w1)), cmul(F2, w2));
    }
    const C su = sp[0], sv = sp[1], sw = sp[2];
    const float m1 = wavenum<float>(0.0, alpha_f, m);
    // (roundings spelled out, see cmul<float2>)
    const float H = __fmaf_rn(-m1, m1, -__fmul_rn(n1, n1));
    float2 nphi, npsi;
    nphi.x = __fmaf_rn(sv.x, H, -__fadd_rn(__fmul_rn(__fmul_rn(su.y, m1), kb1), __fmul_rn(__fmul_rn(sw.y, n1), kb1)));
    nphi.y = __fmaf_rn(sv.y, H, __fadd_rn(__fmul_rn(__fmul_rn(su.x, m1), kb1), __fmul_rn(__fmul_rn(sw.x, n1), kb1)));
    npsi.x = __fmaf_rn(sw.y, m1, -__fmul_rn(su.y, n1));
    npsi.y = -__fmaf_rn(sw.x, m1, -__fmul_rn(su.x, n1));
    if (ms == 0 && n == 0) {
      if (k == 0) npsi = make_float2(0.f, 0.f);
      else {
        npsi = make_float2(-su.x, -su.y);
        nphi = make_float2(-sw.x, -sw.y);
      }
    }
    auto update = [&](float ah, float al, float b, float cv, float nv, float onv) {
      const float ph = __fmul_rn(ah, cv);              // not contracted: ph + pl = ah*cv exactly
      const float pl = fmaf(ah, cv, -ph);
      const float r = fmaf(b, fmaf(3.f, nv, -onv), fmaf(al, cv, pl));
      return __fadd_rn(ph, r);
    };
    {
      const float2 ov = first32 ? npsi : o0;
      float cx_ = update(ah0, al0, b0, c0.x, npsi.x, ov.x);
      const float cy_ = update(ah0, al0, b0, c0.y, npsi.y, ov.y);
      if (slot0 == 0 && ms == 0 && n == 0) cx_ = 0.f;
      c[i0] = mk<float>(cx_, cy_);
      onl[i0] = npsi;
    }
    if (k > 0) {
      const float2 ov = first32 ? nphi : o1;
      const float cx_ = update(ah1, al1, b1, c1.x, nphi.x, ov.x);
      const float cy_ = update(ah1, al1, b1, c1.y, nphi.y, ov.y);
      c[i1] = mk<float>(cx_, cy_);
      onl[i1] = nphi;
    }
  };
  if constexpr (M <= NT) {
    // NT / M columns at a time, one slot per thread
    constexpr int P = NT / M;
    const int lg = threadIdx.x / M;
    const int ms = threadIdx.x - lg * M;
    if (lg < P) {
#pragma unroll 1
      for (int l = lg; l < nb; l += P) output(l, ms);
    }
  } else {
    for (int l = 0; l < nb; ++l)
      for (int ms = threadIdx.x; ms < M; ms += NT) output(l, ms);
  }
}

// Stage and run x-inverse item wi of nb columns (1 <= nb <= xbi_nbmax), nb fixed at compile time.
template <int MM, int NT, int NBT = 1>
__device__ __forceinline__ void xi_batched_nb(int nb, const RunDesc& R, const WorkItem& wi, unsigned char* smem_raw) {
  if constexpr (NBT < xbi_nbmax(MM)) {
    if (nb != NBT) {
      xi_batched_nb<MM, NT, NBT + 1>(nb, R, wi, smem_raw);
      return;
    }
  }
  xi_stage_rows<MM, NT, NBT>(R, wi, reinterpret_cast<float2*>(smem_raw));
  xi_batched_body<MM, NT, NBT>(R, wi, smem_raw);
}

// One x-inverse work item.
template <int MM, int NT>
__device__ __forceinline__ void xi_batched_item(const RunDesc& R, const WorkItem& wi, unsigned char* smem_raw,
                                                unsigned smem_bytes, int* err) {
  const int nb = xi_item_cols<MM>(R, wi, smem_bytes);
  if (nb == 0) return;
  if (nb < 0) {
    if (threadIdx.x == 0) atomicOr(err, MWF_DERR_OUTPUT_CAPACITY);
    return;
  }
  xi_batched_nb<MM, NT>(nb, R, wi, smem_raw);
}

// The x-inverse pass: one item per CTA.  (Resident CTAs that take items in turn and prefetch
// the next item's rows, as the x-forward and z passes do, measured slower here: the update's
// own loads dominate, and the items' uneven costs are better balanced by the block scheduler.)
template <int MM, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) xi_batched_kernel(const RunDesc* __restrict__ runs,
                                                              const WorkItem* __restrict__ items, int* err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const WorkItem wi = items[blockIdx.x];
  xi_batched_item<MM, NT>(runs[wi.run], wi, smem_raw, dyn_smem_bytes(), err);
}

}  // namespace mwf
