// Generated by gen_nl.py -- do not edit.  Galerkin coupling of Model Waleffe Flow.
#pragma once
#define MWF_BETA 1.5707963267948966

// ---- K0 = 4 (KK = 11) ----
template <typename T> __device__ __forceinline__ void nl_y_4(const T (&p)[11], T (&nl)[11]) {
  nl[0] = (T(0.5 * MWF_BETA) * p[4]) * p[1];
  nl[0] = fma(T(-1.0 * MWF_BETA) * p[5], p[2], nl[0]);
  nl[0] = fma(T(1.5 * MWF_BETA) * p[6], p[3], nl[0]);
  nl[1] = (T(-1.0 * MWF_BETA) * p[4]) * p[2];
  nl[1] = fma(T(0.5 * MWF_BETA) * p[5], p[1], nl[1]);
  nl[1] = fma(T(-1.5 * MWF_BETA) * p[5], p[3], nl[1]);
  nl[1] = fma(T(1.0 * MWF_BETA) * p[6], p[2], nl[1]);
  nl[2] = (T(0.5 * MWF_BETA) * p[4]) * p[1];
  nl[2] = fma(T(1.5 * MWF_BETA) * p[4], p[3], nl[2]);
  nl[2] = fma(T(0.5 * MWF_BETA) * p[6], p[1], nl[2]);
  nl[3] = (T(-1.0 * MWF_BETA) * p[4]) * p[2];
  nl[3] = fma(T(0.5 * MWF_BETA) * p[5], p[1], nl[3]);
  nl[4] = (T(1.0 * MWF_BETA) * p[4]) * p[5];
  nl[4] = fma(T(-0.5 * MWF_BETA) * p[5], p[4], nl[4]);
  nl[4] = fma(T(-1.5 * MWF_BETA) * p[5], p[6], nl[4]);
  nl[4] = fma(T(1.0 * MWF_BETA) * p[6], p[5], nl[4]);
  nl[5] = (T(-0.5 * MWF_BETA) * p[4]) * p[4];
  nl[5] = fma(T(-1.5 * MWF_BETA) * p[4], p[6], nl[5]);
  nl[5] = fma(T(0.5 * MWF_BETA) * p[6], p[4], nl[5]);
  nl[6] = (T(1.0 * MWF_BETA) * p[4]) * p[5];
  nl[6] = fma(T(0.5 * MWF_BETA) * p[5], p[4], nl[6]);
  nl[7] = (T(0.5 * MWF_BETA) * p[4]) * p[8];
  nl[7] = fma(T(-1.0 * MWF_BETA) * p[5], p[9], nl[7]);
  nl[7] = fma(T(1.5 * MWF_BETA) * p[6], p[10], nl[7]);
  nl[8] = (T(-1.0 * MWF_BETA) * p[4]) * p[9];
  nl[8] = fma(T(0.5 * MWF_BETA) * p[5], p[8], nl[8]);
  nl[8] = fma(T(-1.5 * MWF_BETA) * p[5], p[10], nl[8]);
  nl[8] = fma(T(1.0 * MWF_BETA) * p[6], p[9], nl[8]);
  nl[9] = (T(0.5 * MWF_BETA) * p[4]) * p[8];
  nl[9] = fma(T(1.5 * MWF_BETA) * p[4], p[10], nl[9]);
  nl[9] = fma(T(0.5 * MWF_BETA) * p[6], p[8], nl[9]);
  nl[10] = (T(-1.0 * MWF_BETA) * p[4]) * p[9];
  nl[10] = fma(T(0.5 * MWF_BETA) * p[5], p[8], nl[10]);
}
template <int J, typename T> __device__ __forceinline__ void nl_xz_4(const T (&p)[11], T px, T pz, T (&nl)[11]) {
  const T hx = T(0.5) * px, hz = T(0.5) * pz;
  if constexpr (J == 0) {  // u_0
    nl[0] = fma(p[0], px, nl[0]); nl[0] = fma(p[7], pz, nl[0]);
    nl[1] = fma(p[1], px, nl[1]); nl[1] = fma(p[8], pz, nl[1]);
    nl[2] = fma(p[2], px, nl[2]); nl[2] = fma(p[9], pz, nl[2]);
    nl[3] = fma(p[3], px, nl[3]); nl[3] = fma(p[10], pz, nl[3]);
  }
  else if constexpr (J == 1) {  // u_1
    nl[0] = fma(p[1], hx, nl[0]); nl[0] = fma(p[8], hz, nl[0]);
    nl[1] = fma(p[0], px, nl[1]); nl[1] = fma(p[7], pz, nl[1]);
    nl[1] = fma(-p[2], hx, nl[1]); nl[1] = fma(-p[9], hz, nl[1]);
    nl[2] = fma(-p[1], hx, nl[2]); nl[2] = fma(-p[8], hz, nl[2]);
    nl[2] = fma(p[3], hx, nl[2]); nl[2] = fma(p[10], hz, nl[2]);
    nl[3] = fma(p[2], hx, nl[3]); nl[3] = fma(p[9], hz, nl[3]);
  }
  else if constexpr (J == 2) {  // u_2
    nl[0] = fma(p[2], hx, nl[0]); nl[0] = fma(p[9], hz, nl[0]);
    nl[1] = fma(-p[1], hx, nl[1]); nl[1] = fma(-p[8], hz, nl[1]);
    nl[1] = fma(p[3], hx, nl[1]); nl[1] = fma(p[10], hz, nl[1]);
    nl[2] = fma(p[0], px, nl[2]); nl[2] = fma(p[7], pz, nl[2]);
    nl[3] = fma(p[1], hx, nl[3]); nl[3] = fma(p[8], hz, nl[3]);
  }
  else if constexpr (J == 3) {  // u_3
    nl[0] = fma(p[3], hx, nl[0]); nl[0] = fma(p[10], hz, nl[0]);
    nl[1] = fma(p[2], hx, nl[1]); nl[1] = fma(p[9], hz, nl[1]);
    nl[2] = fma(p[1], hx, nl[2]); nl[2] = fma(p[8], hz, nl[2]);
    nl[3] = fma(p[0], px, nl[3]); nl[3] = fma(p[7], pz, nl[3]);
  }
  else if constexpr (J == 4) {  // v_1
    nl[4] = fma(p[0], px, nl[4]); nl[4] = fma(p[7], pz, nl[4]);
    nl[4] = fma(p[2], hx, nl[4]); nl[4] = fma(p[9], hz, nl[4]);
    nl[5] = fma(p[1], hx, nl[5]); nl[5] = fma(p[8], hz, nl[5]);
    nl[5] = fma(p[3], hx, nl[5]); nl[5] = fma(p[10], hz, nl[5]);
    nl[6] = fma(p[2], hx, nl[6]); nl[6] = fma(p[9], hz, nl[6]);
  }
  else if constexpr (J == 5) {  // v_2
    nl[4] = fma(p[1], hx, nl[4]); nl[4] = fma(p[8], hz, nl[4]);
    nl[4] = fma(p[3], hx, nl[4]); nl[4] = fma(p[10], hz, nl[4]);
    nl[5] = fma(p[0], px, nl[5]); nl[5] = fma(p[7], pz, nl[5]);
    nl[6] = fma(-p[1], hx, nl[6]); nl[6] = fma(-p[8], hz, nl[6]);
  }
  else if constexpr (J == 6) {  // v_3
    nl[4] = fma(p[2], hx, nl[4]); nl[4] = fma(p[9], hz, nl[4]);
    nl[5] = fma(-p[1], hx, nl[5]); nl[5] = fma(-p[8], hz, nl[5]);
    nl[6] = fma(p[0], px, nl[6]); nl[6] = fma(p[7], pz, nl[6]);
  }
  else if constexpr (J == 7) {  // w_0
    nl[7] = fma(p[0], px, nl[7]); nl[7] = fma(p[7], pz, nl[7]);
    nl[8] = fma(p[1], px, nl[8]); nl[8] = fma(p[8], pz, nl[8]);
    nl[9] = fma(p[2], px, nl[9]); nl[9] = fma(p[9], pz, nl[9]);
    nl[10] = fma(p[3], px, nl[10]); nl[10] = fma(p[10], pz, nl[10]);
  }
  else if constexpr (J == 8) {  // w_1
    nl[7] = fma(p[1], hx, nl[7]); nl[7] = fma(p[8], hz, nl[7]);
    nl[8] = fma(p[0], px, nl[8]); nl[8] = fma(p[7], pz, nl[8]);
    nl[8] = fma(-p[2], hx, nl[8]); nl[8] = fma(-p[9], hz, nl[8]);
    nl[9] = fma(-p[1], hx, nl[9]); nl[9] = fma(-p[8], hz, nl[9]);
    nl[9] = fma(p[3], hx, nl[9]); nl[9] = fma(p[10], hz, nl[9]);
    nl[10] = fma(p[2], hx, nl[10]); nl[10] = fma(p[9], hz, nl[10]);
  }
  else if constexpr (J == 9) {  // w_2
    nl[7] = fma(p[2], hx, nl[7]); nl[7] = fma(p[9], hz, nl[7]);
    nl[8] = fma(-p[1], hx, nl[8]); nl[8] = fma(-p[8], hz, nl[8]);
    nl[8] = fma(p[3], hx, nl[8]); nl[8] = fma(p[10], hz, nl[8]);
    nl[9] = fma(p[0], px, nl[9]); nl[9] = fma(p[7], pz, nl[9]);
    nl[10] = fma(p[1], hx, nl[10]); nl[10] = fma(p[8], hz, nl[10]);
  }
  else if constexpr (J == 10) {  // w_3
    nl[7] = fma(p[3], hx, nl[7]); nl[7] = fma(p[10], hz, nl[7]);
    nl[8] = fma(p[2], hx, nl[8]); nl[8] = fma(p[9], hz, nl[8]);
    nl[9] = fma(p[1], hx, nl[9]); nl[9] = fma(p[8], hz, nl[9]);
    nl[10] = fma(p[0], px, nl[10]); nl[10] = fma(p[7], pz, nl[10]);
  }
}

// ---- K0 = 6 (KK = 17) ----
template <typename T> __device__ __forceinline__ void nl_y_6(const T (&p)[17], T (&nl)[17]) {
  nl[0] = (T(0.5 * MWF_BETA) * p[6]) * p[1];
  nl[0] = fma(T(-1.0 * MWF_BETA) * p[7], p[2], nl[0]);
  nl[0] = fma(T(1.5 * MWF_BETA) * p[8], p[3], nl[0]);
  nl[0] = fma(T(-2.0 * MWF_BETA) * p[9], p[4], nl[0]);
  nl[0] = fma(T(2.5 * MWF_BETA) * p[10], p[5], nl[0]);
  nl[1] = (T(-1.0 * MWF_BETA) * p[6]) * p[2];
  nl[1] = fma(T(0.5 * MWF_BETA) * p[7], p[1], nl[1]);
  nl[1] = fma(T(-1.5 * MWF_BETA) * p[7], p[3], nl[1]);
  nl[1] = fma(T(1.0 * MWF_BETA) * p[8], p[2], nl[1]);
  nl[1] = fma(T(-2.0 * MWF_BETA) * p[8], p[4], nl[1]);
  nl[1] = fma(T(1.5 * MWF_BETA) * p[9], p[3], nl[1]);
  nl[1] = fma(T(-2.5 * MWF_BETA) * p[9], p[5], nl[1]);
  nl[1] = fma(T(2.0 * MWF_BETA) * p[10], p[4], nl[1]);
  nl[2] = (T(0.5 * MWF_BETA) * p[6]) * p[1];
  nl[2] = fma(T(1.5 * MWF_BETA) * p[6], p[3], nl[2]);
  nl[2] = fma(T(-2.0 * MWF_BETA) * p[7], p[4], nl[2]);
  nl[2] = fma(T(0.5 * MWF_BETA) * p[8], p[1], nl[2]);
  nl[2] = fma(T(2.5 * MWF_BETA) * p[8], p[5], nl[2]);
  nl[2] = fma(T(-1.0 * MWF_BETA) * p[9], p[2], nl[2]);
  nl[2] = fma(T(1.5 * MWF_BETA) * p[10], p[3], nl[2]);
  nl[3] = (T(-1.0 * MWF_BETA) * p[6]) * p[2];
  nl[3] = fma(T(-2.0 * MWF_BETA) * p[6], p[4], nl[3]);
  nl[3] = fma(T(0.5 * MWF_BETA) * p[7], p[1], nl[3]);
  nl[3] = fma(T(-2.5 * MWF_BETA) * p[7], p[5], nl[3]);
  nl[3] = fma(T(0.5 * MWF_BETA) * p[9], p[1], nl[3]);
  nl[3] = fma(T(1.0 * MWF_BETA) * p[10], p[2], nl[3]);
  nl[4] = (T(1.5 * MWF_BETA) * p[6]) * p[3];
  nl[4] = fma(T(2.5 * MWF_BETA) * p[6], p[5], nl[4]);
  nl[4] = fma(T(1.0 * MWF_BETA) * p[7], p[2], nl[4]);
  nl[4] = fma(T(0.5 * MWF_BETA) * p[8], p[1], nl[4]);
  nl[4] = fma(T(0.5 * MWF_BETA) * p[10], p[1], nl[4]);
  nl[5] = (T(-2.0 * MWF_BETA) * p[6]) * p[4];
  nl[5] = fma(T(1.5 * MWF_BETA) * p[7], p[3], nl[5]);
  nl[5] = fma(T(-1.0 * MWF_BETA) * p[8], p[2], nl[5]);
  nl[5] = fma(T(0.5 * MWF_BETA) * p[9], p[1], nl[5]);
  nl[6] = (T(1.0 * MWF_BETA) * p[6]) * p[7];
  nl[6] = fma(T(-0.5 * MWF_BETA) * p[7], p[6], nl[6]);
  nl[6] = fma(T(-1.5 * MWF_BETA) * p[7], p[8], nl[6]);
  nl[6] = fma(T(1.0 * MWF_BETA) * p[8], p[7], nl[6]);
  nl[6] = fma(T(2.0 * MWF_BETA) * p[8], p[9], nl[6]);
  nl[6] = fma(T(-1.5 * MWF_BETA) * p[9], p[8], nl[6]);
  nl[6] = fma(T(-2.5 * MWF_BETA) * p[9], p[10], nl[6]);
  nl[6] = fma(T(2.0 * MWF_BETA) * p[10], p[9], nl[6]);
  nl[7] = (T(-0.5 * MWF_BETA) * p[6]) * p[6];
  nl[7] = fma(T(-1.5 * MWF_BETA) * p[6], p[8], nl[7]);
  nl[7] = fma(T(-2.0 * MWF_BETA) * p[7], p[9], nl[7]);
  nl[7] = fma(T(0.5 * MWF_BETA) * p[8], p[6], nl[7]);
  nl[7] = fma(T(-2.5 * MWF_BETA) * p[8], p[10], nl[7]);
  nl[7] = fma(T(1.0 * MWF_BETA) * p[9], p[7], nl[7]);
  nl[7] = fma(T(1.5 * MWF_BETA) * p[10], p[8], nl[7]);
  nl[8] = (T(1.0 * MWF_BETA) * p[6]) * p[7];
  nl[8] = fma(T(2.0 * MWF_BETA) * p[6], p[9], nl[8]);
  nl[8] = fma(T(0.5 * MWF_BETA) * p[7], p[6], nl[8]);
  nl[8] = fma(T(-2.5 * MWF_BETA) * p[7], p[10], nl[8]);
  nl[8] = fma(T(-0.5 * MWF_BETA) * p[9], p[6], nl[8]);
  nl[8] = fma(T(1.0 * MWF_BETA) * p[10], p[7], nl[8]);
  nl[9] = (T(-1.5 * MWF_BETA) * p[6]) * p[8];
  nl[9] = fma(T(-2.5 * MWF_BETA) * p[6], p[10], nl[9]);
  nl[9] = fma(T(1.0 * MWF_BETA) * p[7], p[7], nl[9]);
  nl[9] = fma(T(-0.5 * MWF_BETA) * p[8], p[6], nl[9]);
  nl[9] = fma(T(0.5 * MWF_BETA) * p[10], p[6], nl[9]);
  nl[10] = (T(2.0 * MWF_BETA) * p[6]) * p[9];
  nl[10] = fma(T(1.5 * MWF_BETA) * p[7], p[8], nl[10]);
  nl[10] = fma(T(1.0 * MWF_BETA) * p[8], p[7], nl[10]);
  nl[10] = fma(T(0.5 * MWF_BETA) * p[9], p[6], nl[10]);
  nl[11] = (T(0.5 * MWF_BETA) * p[6]) * p[12];
  nl[11] = fma(T(-1.0 * MWF_BETA) * p[7], p[13], nl[11]);
  nl[11] = fma(T(1.5 * MWF_BETA) * p[8], p[14], nl[11]);
  nl[11] = fma(T(-2.0 * MWF_BETA) * p[9], p[15], nl[11]);
  nl[11] = fma(T(2.5 * MWF_BETA) * p[10], p[16], nl[11]);
  nl[12] = (T(-1.0 * MWF_BETA) * p[6]) * p[13];
  nl[12] = fma(T(0.5 * MWF_BETA) * p[7], p[12], nl[12]);
  nl[12] = fma(T(-1.5 * MWF_BETA) * p[7], p[14], nl[12]);
  nl[12] = fma(T(1.0 * MWF_BETA) * p[8], p[13], nl[12]);
  nl[12] = fma(T(-2.0 * MWF_BETA) * p[8], p[15], nl[12]);
  nl[12] = fma(T(1.5 * MWF_BETA) * p[9], p[14], nl[12]);
  nl[12] = fma(T(-2.5 * MWF_BETA) * p[9], p[16], nl[12]);
  nl[12] = fma(T(2.0 * MWF_BETA) * p[10], p[15], nl[12]);
  nl[13] = (T(0.5 * MWF_BETA) * p[6]) * p[12];
  nl[13] = fma(T(1.5 * MWF_BETA) * p[6], p[14], nl[13]);
  nl[13] = fma(T(-2.0 * MWF_BETA) * p[7], p[15], nl[13]);
  nl[13] = fma(T(0.5 * MWF_BETA) * p[8], p[12], nl[13]);
  nl[13] = fma(T(2.5 * MWF_BETA) * p[8], p[16], nl[13]);
  nl[13] = fma(T(-1.0 * MWF_BETA) * p[9], p[13], nl[13]);
  nl[13] = fma(T(1.5 * MWF_BETA) * p[10], p[14], nl[13]);
  nl[14] = (T(-1.0 * MWF_BETA) * p[6]) * p[13];
  nl[14] = fma(T(-2.0 * MWF_BETA) * p[6], p[15], nl[14]);
  nl[14] = fma(T(0.5 * MWF_BETA) * p[7], p[12], nl[14]);
  nl[14] = fma(T(-2.5 * MWF_BETA) * p[7], p[16], nl[14]);
  nl[14] = fma(T(0.5 * MWF_BETA) * p[9], p[12], nl[14]);
  nl[14] = fma(T(1.0 * MWF_BETA) * p[10], p[13], nl[14]);
  nl[15] = (T(1.5 * MWF_BETA) * p[6]) * p[14];
  nl[15] = fma(T(2.5 * MWF_BETA) * p[6], p[16], nl[15]);
  nl[15] = fma(T(1.0 * MWF_BETA) * p[7], p[13], nl[15]);
  nl[15] = fma(T(0.5 * MWF_BETA) * p[8], p[12], nl[15]);
  nl[15] = fma(T(0.5 * MWF_BETA) * p[10], p[12], nl[15]);
  nl[16] = (T(-2.0 * MWF_BETA) * p[6]) * p[15];
  nl[16] = fma(T(1.5 * MWF_BETA) * p[7], p[14], nl[16]);
  nl[16] = fma(T(-1.0 * MWF_BETA) * p[8], p[13], nl[16]);
  nl[16] = fma(T(0.5 * MWF_BETA) * p[9], p[12], nl[16]);
}
template <int J, typename T> __device__ __forceinline__ void nl_xz_6(const T (&p)[17], T px, T pz, T (&nl)[17]) {
  const T hx = T(0.5) * px, hz = T(0.5) * pz;
  if constexpr (J == 0) {  // u_0
    nl[0] = fma(p[0], px, nl[0]); nl[0] = fma(p[11], pz, nl[0]);
    nl[1] = fma(p[1], px, nl[1]); nl[1] = fma(p[12], pz, nl[1]);
    nl[2] = fma(p[2], px, nl[2]); nl[2] = fma(p[13], pz, nl[2]);
    nl[3] = fma(p[3], px, nl[3]); nl[3] = fma(p[14], pz, nl[3]);
    nl[4] = fma(p[4], px, nl[4]); nl[4] = fma(p[15], pz, nl[4]);
    nl[5] = fma(p[5], px, nl[5]); nl[5] = fma(p[16], pz, nl[5]);
  }
  else if constexpr (J == 1) {  // u_1
    nl[0] = fma(p[1], hx, nl[0]); nl[0] = fma(p[12], hz, nl[0]);
    nl[1] = fma(p[0], px, nl[1]); nl[1] = fma(p[11], pz, nl[1]);
    nl[1] = fma(-p[2], hx, nl[1]); nl[1] = fma(-p[13], hz, nl[1]);
    nl[2] = fma(-p[1], hx, nl[2]); nl[2] = fma(-p[12], hz, nl[2]);
    nl[2] = fma(p[3], hx, nl[2]); nl[2] = fma(p[14], hz, nl[2]);
    nl[3] = fma(p[2], hx, nl[3]); nl[3] = fma(p[13], hz, nl[3]);
    nl[3] = fma(-p[4], hx, nl[3]); nl[3] = fma(-p[15], hz, nl[3]);
    nl[4] = fma(-p[3], hx, nl[4]); nl[4] = fma(-p[14], hz, nl[4]);
    nl[4] = fma(p[5], hx, nl[4]); nl[4] = fma(p[16], hz, nl[4]);
    nl[5] = fma(p[4], hx, nl[5]); nl[5] = fma(p[15], hz, nl[5]);
  }
  else if constexpr (J == 2) {  // u_2
    nl[0] = fma(p[2], hx, nl[0]); nl[0] = fma(p[13], hz, nl[0]);
    nl[1] = fma(-p[1], hx, nl[1]); nl[1] = fma(-p[12], hz, nl[1]);
    nl[1] = fma(p[3], hx, nl[1]); nl[1] = fma(p[14], hz, nl[1]);
    nl[2] = fma(p[0], px, nl[2]); nl[2] = fma(p[11], pz, nl[2]);
    nl[2] = fma(p[4], hx, nl[2]); nl[2] = fma(p[15], hz, nl[2]);
    nl[3] = fma(p[1], hx, nl[3]); nl[3] = fma(p[12], hz, nl[3]);
    nl[3] = fma(p[5], hx, nl[3]); nl[3] = fma(p[16], hz, nl[3]);
    nl[4] = fma(p[2], hx, nl[4]); nl[4] = fma(p[13], hz, nl[4]);
    nl[5] = fma(p[3], hx, nl[5]); nl[5] = fma(p[14], hz, nl[5]);
  }
  else if constexpr (J == 3) {  // u_3
    nl[0] = fma(p[3], hx, nl[0]); nl[0] = fma(p[14], hz, nl[0]);
    nl[1] = fma(p[2], hx, nl[1]); nl[1] = fma(p[13], hz, nl[1]);
    nl[1] = fma(-p[4], hx, nl[1]); nl[1] = fma(-p[15], hz, nl[1]);
    nl[2] = fma(p[1], hx, nl[2]); nl[2] = fma(p[12], hz, nl[2]);
    nl[2] = fma(p[5], hx, nl[2]); nl[2] = fma(p[16], hz, nl[2]);
    nl[3] = fma(p[0], px, nl[3]); nl[3] = fma(p[11], pz, nl[3]);
    nl[4] = fma(-p[1], hx, nl[4]); nl[4] = fma(-p[12], hz, nl[4]);
    nl[5] = fma(p[2], hx, nl[5]); nl[5] = fma(p[13], hz, nl[5]);
  }
  else if constexpr (J == 4) {  // u_4
    nl[0] = fma(p[4], hx, nl[0]); nl[0] = fma(p[15], hz, nl[0]);
    nl[1] = fma(-p[3], hx, nl[1]); nl[1] = fma(-p[14], hz, nl[1]);
    nl[1] = fma(p[5], hx, nl[1]); nl[1] = fma(p[16], hz, nl[1]);
    nl[2] = fma(p[2], hx, nl[2]); nl[2] = fma(p[13], hz, nl[2]);
    nl[3] = fma(-p[1], hx, nl[3]); nl[3] = fma(-p[12], hz, nl[3]);
    nl[4] = fma(p[0], px, nl[4]); nl[4] = fma(p[11], pz, nl[4]);
    nl[5] = fma(p[1], hx, nl[5]); nl[5] = fma(p[12], hz, nl[5]);
  }
  else if constexpr (J == 5) {  // u_5
    nl[0] = fma(p[5], hx, nl[0]); nl[0] = fma(p[16], hz, nl[0]);
    nl[1] = fma(p[4], hx, nl[1]); nl[1] = fma(p[15], hz, nl[1]);
    nl[2] = fma(p[3], hx, nl[2]); nl[2] = fma(p[14], hz, nl[2]);
    nl[3] = fma(p[2], hx, nl[3]); nl[3] = fma(p[13], hz, nl[3]);
    nl[4] = fma(p[1], hx, nl[4]); nl[4] = fma(p[12], hz, nl[4]);
    nl[5] = fma(p[0], px, nl[5]); nl[5] = fma(p[11], pz, nl[5]);
  }
  else if constexpr (J == 6) {  // v_1
    nl[6] = fma(p[0], px, nl[6]); nl[6] = fma(p[11], pz, nl[6]);
    nl[6] = fma(p[2], hx, nl[6]); nl[6] = fma(p[13], hz, nl[6]);
    nl[7] = fma(p[1], hx, nl[7]); nl[7] = fma(p[12], hz, nl[7]);
    nl[7] = fma(p[3], hx, nl[7]); nl[7] = fma(p[14], hz, nl[7]);
    nl[8] = fma(p[2], hx, nl[8]); nl[8] = fma(p[13], hz, nl[8]);
    nl[8] = fma(p[4], hx, nl[8]); nl[8] = fma(p[15], hz, nl[8]);
    nl[9] = fma(p[3], hx, nl[9]); nl[9] = fma(p[14], hz, nl[9]);
    nl[9] = fma(p[5], hx, nl[9]); nl[9] = fma(p[16], hz, nl[9]);
    nl[10] = fma(p[4], hx, nl[10]); nl[10] = fma(p[15], hz, nl[10]);
  }
  else if constexpr (J == 7) {  // v_2
    nl[6] = fma(p[1], hx, nl[6]); nl[6] = fma(p[12], hz, nl[6]);
    nl[6] = fma(p[3], hx, nl[6]); nl[6] = fma(p[14], hz, nl[6]);
    nl[7] = fma(p[0], px, nl[7]); nl[7] = fma(p[11], pz, nl[7]);
    nl[7] = fma(-p[4], hx, nl[7]); nl[7] = fma(-p[15], hz, nl[7]);
    nl[8] = fma(-p[1], hx, nl[8]); nl[8] = fma(-p[12], hz, nl[8]);
    nl[8] = fma(p[5], hx, nl[8]); nl[8] = fma(p[16], hz, nl[8]);
    nl[9] = fma(p[2], hx, nl[9]); nl[9] = fma(p[13], hz, nl[9]);
    nl[10] = fma(-p[3], hx, nl[10]); nl[10] = fma(-p[14], hz, nl[10]);
  }
  else if constexpr (J == 8) {  // v_3
    nl[6] = fma(p[2], hx, nl[6]); nl[6] = fma(p[13], hz, nl[6]);
    nl[6] = fma(p[4], hx, nl[6]); nl[6] = fma(p[15], hz, nl[6]);
    nl[7] = fma(-p[1], hx, nl[7]); nl[7] = fma(-p[12], hz, nl[7]);
    nl[7] = fma(p[5], hx, nl[7]); nl[7] = fma(p[16], hz, nl[7]);
    nl[8] = fma(p[0], px, nl[8]); nl[8] = fma(p[11], pz, nl[8]);
    nl[9] = fma(p[1], hx, nl[9]); nl[9] = fma(p[12], hz, nl[9]);
    nl[10] = fma(p[2], hx, nl[10]); nl[10] = fma(p[13], hz, nl[10]);
  }
  else if constexpr (J == 9) {  // v_4
    nl[6] = fma(p[3], hx, nl[6]); nl[6] = fma(p[14], hz, nl[6]);
    nl[6] = fma(p[5], hx, nl[6]); nl[6] = fma(p[16], hz, nl[6]);
    nl[7] = fma(p[2], hx, nl[7]); nl[7] = fma(p[13], hz, nl[7]);
    nl[8] = fma(p[1], hx, nl[8]); nl[8] = fma(p[12], hz, nl[8]);
    nl[9] = fma(p[0], px, nl[9]); nl[9] = fma(p[11], pz, nl[9]);
    nl[10] = fma(-p[1], hx, nl[10]); nl[10] = fma(-p[12], hz, nl[10]);
  }
  else if constexpr (J == 10) {  // v_5
    nl[6] = fma(p[4], hx, nl[6]); nl[6] = fma(p[15], hz, nl[6]);
    nl[7] = fma(-p[3], hx, nl[7]); nl[7] = fma(-p[14], hz, nl[7]);
    nl[8] = fma(p[2], hx, nl[8]); nl[8] = fma(p[13], hz, nl[8]);
    nl[9] = fma(-p[1], hx, nl[9]); nl[9] = fma(-p[12], hz, nl[9]);
    nl[10] = fma(p[0], px, nl[10]); nl[10] = fma(p[11], pz, nl[10]);
  }
  else if constexpr (J == 11) {  // w_0
    nl[11] = fma(p[0], px, nl[11]); nl[11] = fma(p[11], pz, nl[11]);
    nl[12] = fma(p[1], px, nl[12]); nl[12] = fma(p[12], pz, nl[12]);
    nl[13] = fma(p[2], px, nl[13]); nl[13] = fma(p[13], pz, nl[13]);
    nl[14] = fma(p[3], px, nl[14]); nl[14] = fma(p[14], pz, nl[14]);
    nl[15] = fma(p[4], px, nl[15]); nl[15] = fma(p[15], pz, nl[15]);
    nl[16] = fma(p[5], px, nl[16]); nl[16] = fma(p[16], pz, nl[16]);
  }
  else if constexpr (J == 12) {  // w_1
    nl[11] = fma(p[1], hx, nl[11]); nl[11] = fma(p[12], hz, nl[11]);
    nl[12] = fma(p[0], px, nl[12]); nl[12] = fma(p[11], pz, nl[12]);
    nl[12] = fma(-p[2], hx, nl[12]); nl[12] = fma(-p[13], hz, nl[12]);
    nl[13] = fma(-p[1], hx, nl[13]); nl[13] = fma(-p[12], hz, nl[13]);
    nl[13] = fma(p[3], hx, nl[13]); nl[13] = fma(p[14], hz, nl[13]);
    nl[14] = fma(p[2], hx, nl[14]); nl[14] = fma(p[13], hz, nl[14]);
    nl[14] = fma(-p[4], hx, nl[14]); nl[14] = fma(-p[15], hz, nl[14]);
    nl[15] = fma(-p[3], hx, nl[15]); nl[15] = fma(-p[14], hz, nl[15]);
    nl[15] = fma(p[5], hx, nl[15]); nl[15] = fma(p[16], hz, nl[15]);
    nl[16] = fma(p[4], hx, nl[16]); nl[16] = fma(p[15], hz, nl[16]);
  }
  else if constexpr (J == 13) {  // w_2
    nl[11] = fma(p[2], hx, nl[11]); nl[11] = fma(p[13], hz, nl[11]);
    nl[12] = fma(-p[1], hx, nl[12]); nl[12] = fma(-p[12], hz, nl[12]);
    nl[12] = fma(p[3], hx, nl[12]); nl[12] = fma(p[14], hz, nl[12]);
    nl[13] = fma(p[0], px, nl[13]); nl[13] = fma(p[11], pz, nl[13]);
    nl[13] = fma(p[4], hx, nl[13]); nl[13] = fma(p[15], hz, nl[13]);
    nl[14] = fma(p[1], hx, nl[14]); nl[14] = fma(p[12], hz, nl[14]);
    nl[14] = fma(p[5], hx, nl[14]); nl[14] = fma(p[16], hz, nl[14]);
    nl[15] = fma(p[2], hx, nl[15]); nl[15] = fma(p[13], hz, nl[15]);
    nl[16] = fma(p[3], hx, nl[16]); nl[16] = fma(p[14], hz, nl[16]);
  }
  else if constexpr (J == 14) {  // w_3
    nl[11] = fma(p[3], hx, nl[11]); nl[11] = fma(p[14], hz, nl[11]);
    nl[12] = fma(p[2], hx, nl[12]); nl[12] = fma(p[13], hz, nl[12]);
    nl[12] = fma(-p[4], hx, nl[12]); nl[12] = fma(-p[15], hz, nl[12]);
    nl[13] = fma(p[1], hx, nl[13]); nl[13] = fma(p[12], hz, nl[13]);
    nl[13] = fma(p[5], hx, nl[13]); nl[13] = fma(p[16], hz, nl[13]);
    nl[14] = fma(p[0], px, nl[14]); nl[14] = fma(p[11], pz, nl[14]);
    nl[15] = fma(-p[1], hx, nl[15]); nl[15] = fma(-p[12], hz, nl[15]);
    nl[16] = fma(p[2], hx, nl[16]); nl[16] = fma(p[13], hz, nl[16]);
  }
  else if constexpr (J == 15) {  // w_4
    nl[11] = fma(p[4], hx, nl[11]); nl[11] = fma(p[15], hz, nl[11]);
    nl[12] = fma(-p[3], hx, nl[12]); nl[12] = fma(-p[14], hz, nl[12]);
    nl[12] = fma(p[5], hx, nl[12]); nl[12] = fma(p[16], hz, nl[12]);
    nl[13] = fma(p[2], hx, nl[13]); nl[13] = fma(p[13], hz, nl[13]);
    nl[14] = fma(-p[1], hx, nl[14]); nl[14] = fma(-p[12], hz, nl[14]);
    nl[15] = fma(p[0], px, nl[15]); nl[15] = fma(p[11], pz, nl[15]);
    nl[16] = fma(p[1], hx, nl[16]); nl[16] = fma(p[12], hz, nl[16]);
  }
  else if constexpr (J == 16) {  // w_5
    nl[11] = fma(p[5], hx, nl[11]); nl[11] = fma(p[16], hz, nl[11]);
    nl[12] = fma(p[4], hx, nl[12]); nl[12] = fma(p[15], hz, nl[12]);
    nl[13] = fma(p[3], hx, nl[13]); nl[13] = fma(p[14], hz, nl[13]);
    nl[14] = fma(p[2], hx, nl[14]); nl[14] = fma(p[13], hz, nl[14]);
    nl[15] = fma(p[1], hx, nl[15]); nl[15] = fma(p[12], hz, nl[15]);
    nl[16] = fma(p[0], px, nl[16]); nl[16] = fma(p[11], pz, nl[16]);
  }
}

