// Generated by gen_nl.py -- do not edit.  Galerkin coupling of Model Waleffe Flow.
#pragma once
#define MWF_BETA 1.5707963267948966

// ---- K0 = 4 (KK = 11) ----
template <typename T, typename P, typename NL> __device__ __forceinline__ void nl_y_4(const P& p, NL&& nl) {
  const T p1 = p[1];
  const T p2 = p[2];
  const T p3 = p[3];
  const T p4 = p[4];
  const T p5 = p[5];
  const T p6 = p[6];
  const T p8 = p[8];
  const T p9 = p[9];
  const T p10 = p[10];
  { T a = (T(0.5 * MWF_BETA) * p4) * p1;
    a = fma(T(-1.0 * MWF_BETA) * p5, p2, a);
    a = fma(T(1.5 * MWF_BETA) * p6, p3, a);
    nl[0] = a; }
  { T a = (T(-1.0 * MWF_BETA) * p4) * p2;
    a = fma(T(0.5 * MWF_BETA) * p5, p1, a);
    a = fma(T(-1.5 * MWF_BETA) * p5, p3, a);
    a = fma(T(1.0 * MWF_BETA) * p6, p2, a);
    nl[1] = a; }
  { T a = (T(0.5 * MWF_BETA) * p4) * p1;
    a = fma(T(1.5 * MWF_BETA) * p4, p3, a);
    a = fma(T(0.5 * MWF_BETA) * p6, p1, a);
    nl[2] = a; }
  { T a = (T(-1.0 * MWF_BETA) * p4) * p2;
    a = fma(T(0.5 * MWF_BETA) * p5, p1, a);
    nl[3] = a; }
  { T a = (T(1.0 * MWF_BETA) * p4) * p5;
    a = fma(T(-0.5 * MWF_BETA) * p5, p4, a);
    a = fma(T(-1.5 * MWF_BETA) * p5, p6, a);
    a = fma(T(1.0 * MWF_BETA) * p6, p5, a);
    nl[4] = a; }
  { T a = (T(-0.5 * MWF_BETA) * p4) * p4;
    a = fma(T(-1.5 * MWF_BETA) * p4, p6, a);
    a = fma(T(0.5 * MWF_BETA) * p6, p4, a);
    nl[5] = a; }
  { T a = (T(1.0 * MWF_BETA) * p4) * p5;
    a = fma(T(0.5 * MWF_BETA) * p5, p4, a);
    nl[6] = a; }
  { T a = (T(0.5 * MWF_BETA) * p4) * p8;
    a = fma(T(-1.0 * MWF_BETA) * p5, p9, a);
    a = fma(T(1.5 * MWF_BETA) * p6, p10, a);
    nl[7] = a; }
  { T a = (T(-1.0 * MWF_BETA) * p4) * p9;
    a = fma(T(0.5 * MWF_BETA) * p5, p8, a);
    a = fma(T(-1.5 * MWF_BETA) * p5, p10, a);
    a = fma(T(1.0 * MWF_BETA) * p6, p9, a);
    nl[8] = a; }
  { T a = (T(0.5 * MWF_BETA) * p4) * p8;
    a = fma(T(1.5 * MWF_BETA) * p4, p10, a);
    a = fma(T(0.5 * MWF_BETA) * p6, p8, a);
    nl[9] = a; }
  { T a = (T(-1.0 * MWF_BETA) * p4) * p9;
    a = fma(T(0.5 * MWF_BETA) * p5, p8, a);
    nl[10] = a; }
}
template <int J, typename T, typename P, typename NL> __device__ __forceinline__ void nl_xz_4(const P& p, T px, T pz, NL&& nl) {
  const T hx = T(0.5) * px, hz = T(0.5) * pz;
  if constexpr (J == 0) {  // u_0
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p9 = p[9];
    const T p10 = p[10];
    { T a = nl[0]; a = fma(p0, px, a); a = fma(p7, pz, a); nl[0] = a; }
    { T a = nl[1]; a = fma(p1, px, a); a = fma(p8, pz, a); nl[1] = a; }
    { T a = nl[2]; a = fma(p2, px, a); a = fma(p9, pz, a); nl[2] = a; }
    { T a = nl[3]; a = fma(p3, px, a); a = fma(p10, pz, a); nl[3] = a; }
  }
  else if constexpr (J == 1) {  // u_1
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p9 = p[9];
    const T p10 = p[10];
    { T a = nl[0]; a = fma(p1, hx, a); a = fma(p8, hz, a); nl[0] = a; }
    { T a = nl[1]; a = fma(p0, px, a); a = fma(p7, pz, a); a = fma(-p2, hx, a); a = fma(-p9, hz, a); nl[1] = a; }
    { T a = nl[2]; a = fma(-p1, hx, a); a = fma(-p8, hz, a); a = fma(p3, hx, a); a = fma(p10, hz, a); nl[2] = a; }
    { T a = nl[3]; a = fma(p2, hx, a); a = fma(p9, hz, a); nl[3] = a; }
  }
  else if constexpr (J == 2) {  // u_2
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p9 = p[9];
    const T p10 = p[10];
    { T a = nl[0]; a = fma(p2, hx, a); a = fma(p9, hz, a); nl[0] = a; }
    { T a = nl[1]; a = fma(-p1, hx, a); a = fma(-p8, hz, a); a = fma(p3, hx, a); a = fma(p10, hz, a); nl[1] = a; }
    { T a = nl[2]; a = fma(p0, px, a); a = fma(p7, pz, a); nl[2] = a; }
    { T a = nl[3]; a = fma(p1, hx, a); a = fma(p8, hz, a); nl[3] = a; }
  }
  else if constexpr (J == 3) {  // u_3
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p9 = p[9];
    const T p10 = p[10];
    { T a = nl[0]; a = fma(p3, hx, a); a = fma(p10, hz, a); nl[0] = a; }
    { T a = nl[1]; a = fma(p2, hx, a); a = fma(p9, hz, a); nl[1] = a; }
    { T a = nl[2]; a = fma(p1, hx, a); a = fma(p8, hz, a); nl[2] = a; }
    { T a = nl[3]; a = fma(p0, px, a); a = fma(p7, pz, a); nl[3] = a; }
  }
  else if constexpr (J == 4) {  // v_1
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p9 = p[9];
    const T p10 = p[10];
    { T a = nl[4]; a = fma(p0, px, a); a = fma(p7, pz, a); a = fma(p2, hx, a); a = fma(p9, hz, a); nl[4] = a; }
    { T a = nl[5]; a = fma(p1, hx, a); a = fma(p8, hz, a); a = fma(p3, hx, a); a = fma(p10, hz, a); nl[5] = a; }
    { T a = nl[6]; a = fma(p2, hx, a); a = fma(p9, hz, a); nl[6] = a; }
  }
  else if constexpr (J == 5) {  // v_2
    const T p0 = p[0];
    const T p1 = p[1];
    const T p3 = p[3];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p10 = p[10];
    { T a = nl[4]; a = fma(p1, hx, a); a = fma(p8, hz, a); a = fma(p3, hx, a); a = fma(p10, hz, a); nl[4] = a; }
    { T a = nl[5]; a = fma(p0, px, a); a = fma(p7, pz, a); nl[5] = a; }
    { T a = nl[6]; a = fma(-p1, hx, a); a = fma(-p8, hz, a); nl[6] = a; }
  }
  else if constexpr (J == 6) {  // v_3
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p9 = p[9];
    { T a = nl[4]; a = fma(p2, hx, a); a = fma(p9, hz, a); nl[4] = a; }
    { T a = nl[5]; a = fma(-p1, hx, a); a = fma(-p8, hz, a); nl[5] = a; }
    { T a = nl[6]; a = fma(p0, px, a); a = fma(p7, pz, a); nl[6] = a; }
  }
  else if constexpr (J == 7) {  // w_0
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p9 = p[9];
    const T p10 = p[10];
    { T a = nl[7]; a = fma(p0, px, a); a = fma(p7, pz, a); nl[7] = a; }
    { T a = nl[8]; a = fma(p1, px, a); a = fma(p8, pz, a); nl[8] = a; }
    { T a = nl[9]; a = fma(p2, px, a); a = fma(p9, pz, a); nl[9] = a; }
    { T a = nl[10]; a = fma(p3, px, a); a = fma(p10, pz, a); nl[10] = a; }
  }
  else if constexpr (J == 8) {  // w_1
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p9 = p[9];
    const T p10 = p[10];
    { T a = nl[7]; a = fma(p1, hx, a); a = fma(p8, hz, a); nl[7] = a; }
    { T a = nl[8]; a = fma(p0, px, a); a = fma(p7, pz, a); a = fma(-p2, hx, a); a = fma(-p9, hz, a); nl[8] = a; }
    { T a = nl[9]; a = fma(-p1, hx, a); a = fma(-p8, hz, a); a = fma(p3, hx, a); a = fma(p10, hz, a); nl[9] = a; }
    { T a = nl[10]; a = fma(p2, hx, a); a = fma(p9, hz, a); nl[10] = a; }
  }
  else if constexpr (J == 9) {  // w_2
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p9 = p[9];
    const T p10 = p[10];
    { T a = nl[7]; a = fma(p2, hx, a); a = fma(p9, hz, a); nl[7] = a; }
    { T a = nl[8]; a = fma(-p1, hx, a); a = fma(-p8, hz, a); a = fma(p3, hx, a); a = fma(p10, hz, a); nl[8] = a; }
    { T a = nl[9]; a = fma(p0, px, a); a = fma(p7, pz, a); nl[9] = a; }
    { T a = nl[10]; a = fma(p1, hx, a); a = fma(p8, hz, a); nl[10] = a; }
  }
  else if constexpr (J == 10) {  // w_3
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p7 = p[7];
    const T p8 = p[8];
    const T p9 = p[9];
    const T p10 = p[10];
    { T a = nl[7]; a = fma(p3, hx, a); a = fma(p10, hz, a); nl[7] = a; }
    { T a = nl[8]; a = fma(p2, hx, a); a = fma(p9, hz, a); nl[8] = a; }
    { T a = nl[9]; a = fma(p1, hx, a); a = fma(p8, hz, a); nl[9] = a; }
    { T a = nl[10]; a = fma(p0, px, a); a = fma(p7, pz, a); nl[10] = a; }
  }
}

// ---- K0 = 6 (KK = 17) ----
template <typename T, typename P, typename NL> __device__ __forceinline__ void nl_y_6(const P& p, NL&& nl) {
  const T p1 = p[1];
  const T p2 = p[2];
  const T p3 = p[3];
  const T p4 = p[4];
  const T p5 = p[5];
  const T p6 = p[6];
  const T p7 = p[7];
  const T p8 = p[8];
  const T p9 = p[9];
  const T p10 = p[10];
  const T p12 = p[12];
  const T p13 = p[13];
  const T p14 = p[14];
  const T p15 = p[15];
  const T p16 = p[16];
  { T a = (T(0.5 * MWF_BETA) * p6) * p1;
    a = fma(T(-1.0 * MWF_BETA) * p7, p2, a);
    a = fma(T(1.5 * MWF_BETA) * p8, p3, a);
    a = fma(T(-2.0 * MWF_BETA) * p9, p4, a);
    a = fma(T(2.5 * MWF_BETA) * p10, p5, a);
    nl[0] = a; }
  { T a = (T(-1.0 * MWF_BETA) * p6) * p2;
    a = fma(T(0.5 * MWF_BETA) * p7, p1, a);
    a = fma(T(-1.5 * MWF_BETA) * p7, p3, a);
    a = fma(T(1.0 * MWF_BETA) * p8, p2, a);
    a = fma(T(-2.0 * MWF_BETA) * p8, p4, a);
    a = fma(T(1.5 * MWF_BETA) * p9, p3, a);
    a = fma(T(-2.5 * MWF_BETA) * p9, p5, a);
    a = fma(T(2.0 * MWF_BETA) * p10, p4, a);
    nl[1] = a; }
  { T a = (T(0.5 * MWF_BETA) * p6) * p1;
    a = fma(T(1.5 * MWF_BETA) * p6, p3, a);
    a = fma(T(-2.0 * MWF_BETA) * p7, p4, a);
    a = fma(T(0.5 * MWF_BETA) * p8, p1, a);
    a = fma(T(2.5 * MWF_BETA) * p8, p5, a);
    a = fma(T(-1.0 * MWF_BETA) * p9, p2, a);
    a = fma(T(1.5 * MWF_BETA) * p10, p3, a);
    nl[2] = a; }
  { T a = (T(-1.0 * MWF_BETA) * p6) * p2;
    a = fma(T(-2.0 * MWF_BETA) * p6, p4, a);
    a = fma(T(0.5 * MWF_BETA) * p7, p1, a);
    a = fma(T(-2.5 * MWF_BETA) * p7, p5, a);
    a = fma(T(0.5 * MWF_BETA) * p9, p1, a);
    a = fma(T(1.0 * MWF_BETA) * p10, p2, a);
    nl[3] = a; }
  { T a = (T(1.5 * MWF_BETA) * p6) * p3;
    a = fma(T(2.5 * MWF_BETA) * p6, p5, a);
    a = fma(T(1.0 * MWF_BETA) * p7, p2, a);
    a = fma(T(0.5 * MWF_BETA) * p8, p1, a);
    a = fma(T(0.5 * MWF_BETA) * p10, p1, a);
    nl[4] = a; }
  { T a = (T(-2.0 * MWF_BETA) * p6) * p4;
    a = fma(T(1.5 * MWF_BETA) * p7, p3, a);
    a = fma(T(-1.0 * MWF_BETA) * p8, p2, a);
    a = fma(T(0.5 * MWF_BETA) * p9, p1, a);
    nl[5] = a; }
  { T a = (T(1.0 * MWF_BETA) * p6) * p7;
    a = fma(T(-0.5 * MWF_BETA) * p7, p6, a);
    a = fma(T(-1.5 * MWF_BETA) * p7, p8, a);
    a = fma(T(1.0 * MWF_BETA) * p8, p7, a);
    a = fma(T(2.0 * MWF_BETA) * p8, p9, a);
    a = fma(T(-1.5 * MWF_BETA) * p9, p8, a);
    a = fma(T(-2.5 * MWF_BETA) * p9, p10, a);
    a = fma(T(2.0 * MWF_BETA) * p10, p9, a);
    nl[6] = a; }
  { T a = (T(-0.5 * MWF_BETA) * p6) * p6;
    a = fma(T(-1.5 * MWF_BETA) * p6, p8, a);
    a = fma(T(-2.0 * MWF_BETA) * p7, p9, a);
    a = fma(T(0.5 * MWF_BETA) * p8, p6, a);
    a = fma(T(-2.5 * MWF_BETA) * p8, p10, a);
    a = fma(T(1.0 * MWF_BETA) * p9, p7, a);
    a = fma(T(1.5 * MWF_BETA) * p10, p8, a);
    nl[7] = a; }
  { T a = (T(1.0 * MWF_BETA) * p6) * p7;
    a = fma(T(2.0 * MWF_BETA) * p6, p9, a);
    a = fma(T(0.5 * MWF_BETA) * p7, p6, a);
    a = fma(T(-2.5 * MWF_BETA) * p7, p10, a);
    a = fma(T(-0.5 * MWF_BETA) * p9, p6, a);
    a = fma(T(1.0 * MWF_BETA) * p10, p7, a);
    nl[8] = a; }
  { T a = (T(-1.5 * MWF_BETA) * p6) * p8;
    a = fma(T(-2.5 * MWF_BETA) * p6, p10, a);
    a = fma(T(1.0 * MWF_BETA) * p7, p7, a);
    a = fma(T(-0.5 * MWF_BETA) * p8, p6, a);
    a = fma(T(0.5 * MWF_BETA) * p10, p6, a);
    nl[9] = a; }
  { T a = (T(2.0 * MWF_BETA) * p6) * p9;
    a = fma(T(1.5 * MWF_BETA) * p7, p8, a);
    a = fma(T(1.0 * MWF_BETA) * p8, p7, a);
    a = fma(T(0.5 * MWF_BETA) * p9, p6, a);
    nl[10] = a; }
  { T a = (T(0.5 * MWF_BETA) * p6) * p12;
    a = fma(T(-1.0 * MWF_BETA) * p7, p13, a);
    a = fma(T(1.5 * MWF_BETA) * p8, p14, a);
    a = fma(T(-2.0 * MWF_BETA) * p9, p15, a);
    a = fma(T(2.5 * MWF_BETA) * p10, p16, a);
    nl[11] = a; }
  { T a = (T(-1.0 * MWF_BETA) * p6) * p13;
    a = fma(T(0.5 * MWF_BETA) * p7, p12, a);
    a = fma(T(-1.5 * MWF_BETA) * p7, p14, a);
    a = fma(T(1.0 * MWF_BETA) * p8, p13, a);
    a = fma(T(-2.0 * MWF_BETA) * p8, p15, a);
    a = fma(T(1.5 * MWF_BETA) * p9, p14, a);
    a = fma(T(-2.5 * MWF_BETA) * p9, p16, a);
    a = fma(T(2.0 * MWF_BETA) * p10, p15, a);
    nl[12] = a; }
  { T a = (T(0.5 * MWF_BETA) * p6) * p12;
    a = fma(T(1.5 * MWF_BETA) * p6, p14, a);
    a = fma(T(-2.0 * MWF_BETA) * p7, p15, a);
    a = fma(T(0.5 * MWF_BETA) * p8, p12, a);
    a = fma(T(2.5 * MWF_BETA) * p8, p16, a);
    a = fma(T(-1.0 * MWF_BETA) * p9, p13, a);
    a = fma(T(1.5 * MWF_BETA) * p10, p14, a);
    nl[13] = a; }
  { T a = (T(-1.0 * MWF_BETA) * p6) * p13;
    a = fma(T(-2.0 * MWF_BETA) * p6, p15, a);
    a = fma(T(0.5 * MWF_BETA) * p7, p12, a);
    a = fma(T(-2.5 * MWF_BETA) * p7, p16, a);
    a = fma(T(0.5 * MWF_BETA) * p9, p12, a);
    a = fma(T(1.0 * MWF_BETA) * p10, p13, a);
    nl[14] = a; }
  { T a = (T(1.5 * MWF_BETA) * p6) * p14;
    a = fma(T(2.5 * MWF_BETA) * p6, p16, a);
    a = fma(T(1.0 * MWF_BETA) * p7, p13, a);
    a = fma(T(0.5 * MWF_BETA) * p8, p12, a);
    a = fma(T(0.5 * MWF_BETA) * p10, p12, a);
    nl[15] = a; }
  { T a = (T(-2.0 * MWF_BETA) * p6) * p15;
    a = fma(T(1.5 * MWF_BETA) * p7, p14, a);
    a = fma(T(-1.0 * MWF_BETA) * p8, p13, a);
    a = fma(T(0.5 * MWF_BETA) * p9, p12, a);
    nl[16] = a; }
}
template <int J, typename T, typename P, typename NL> __device__ __forceinline__ void nl_xz_6(const P& p, T px, T pz, NL&& nl) {
  const T hx = T(0.5) * px, hz = T(0.5) * pz;
  if constexpr (J == 0) {  // u_0
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[0]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[0] = a; }
    { T a = nl[1]; a = fma(p1, px, a); a = fma(p12, pz, a); nl[1] = a; }
    { T a = nl[2]; a = fma(p2, px, a); a = fma(p13, pz, a); nl[2] = a; }
    { T a = nl[3]; a = fma(p3, px, a); a = fma(p14, pz, a); nl[3] = a; }
    { T a = nl[4]; a = fma(p4, px, a); a = fma(p15, pz, a); nl[4] = a; }
    { T a = nl[5]; a = fma(p5, px, a); a = fma(p16, pz, a); nl[5] = a; }
  }
  else if constexpr (J == 1) {  // u_1
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[0]; a = fma(p1, hx, a); a = fma(p12, hz, a); nl[0] = a; }
    { T a = nl[1]; a = fma(p0, px, a); a = fma(p11, pz, a); a = fma(-p2, hx, a); a = fma(-p13, hz, a); nl[1] = a; }
    { T a = nl[2]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); a = fma(p3, hx, a); a = fma(p14, hz, a); nl[2] = a; }
    { T a = nl[3]; a = fma(p2, hx, a); a = fma(p13, hz, a); a = fma(-p4, hx, a); a = fma(-p15, hz, a); nl[3] = a; }
    { T a = nl[4]; a = fma(-p3, hx, a); a = fma(-p14, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[4] = a; }
    { T a = nl[5]; a = fma(p4, hx, a); a = fma(p15, hz, a); nl[5] = a; }
  }
  else if constexpr (J == 2) {  // u_2
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[0]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[0] = a; }
    { T a = nl[1]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); a = fma(p3, hx, a); a = fma(p14, hz, a); nl[1] = a; }
    { T a = nl[2]; a = fma(p0, px, a); a = fma(p11, pz, a); a = fma(p4, hx, a); a = fma(p15, hz, a); nl[2] = a; }
    { T a = nl[3]; a = fma(p1, hx, a); a = fma(p12, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[3] = a; }
    { T a = nl[4]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[4] = a; }
    { T a = nl[5]; a = fma(p3, hx, a); a = fma(p14, hz, a); nl[5] = a; }
  }
  else if constexpr (J == 3) {  // u_3
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[0]; a = fma(p3, hx, a); a = fma(p14, hz, a); nl[0] = a; }
    { T a = nl[1]; a = fma(p2, hx, a); a = fma(p13, hz, a); a = fma(-p4, hx, a); a = fma(-p15, hz, a); nl[1] = a; }
    { T a = nl[2]; a = fma(p1, hx, a); a = fma(p12, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[2] = a; }
    { T a = nl[3]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[3] = a; }
    { T a = nl[4]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); nl[4] = a; }
    { T a = nl[5]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[5] = a; }
  }
  else if constexpr (J == 4) {  // u_4
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[0]; a = fma(p4, hx, a); a = fma(p15, hz, a); nl[0] = a; }
    { T a = nl[1]; a = fma(-p3, hx, a); a = fma(-p14, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[1] = a; }
    { T a = nl[2]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[2] = a; }
    { T a = nl[3]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); nl[3] = a; }
    { T a = nl[4]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[4] = a; }
    { T a = nl[5]; a = fma(p1, hx, a); a = fma(p12, hz, a); nl[5] = a; }
  }
  else if constexpr (J == 5) {  // u_5
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[0]; a = fma(p5, hx, a); a = fma(p16, hz, a); nl[0] = a; }
    { T a = nl[1]; a = fma(p4, hx, a); a = fma(p15, hz, a); nl[1] = a; }
    { T a = nl[2]; a = fma(p3, hx, a); a = fma(p14, hz, a); nl[2] = a; }
    { T a = nl[3]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[3] = a; }
    { T a = nl[4]; a = fma(p1, hx, a); a = fma(p12, hz, a); nl[4] = a; }
    { T a = nl[5]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[5] = a; }
  }
  else if constexpr (J == 6) {  // v_1
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[6]; a = fma(p0, px, a); a = fma(p11, pz, a); a = fma(p2, hx, a); a = fma(p13, hz, a); nl[6] = a; }
    { T a = nl[7]; a = fma(p1, hx, a); a = fma(p12, hz, a); a = fma(p3, hx, a); a = fma(p14, hz, a); nl[7] = a; }
    { T a = nl[8]; a = fma(p2, hx, a); a = fma(p13, hz, a); a = fma(p4, hx, a); a = fma(p15, hz, a); nl[8] = a; }
    { T a = nl[9]; a = fma(p3, hx, a); a = fma(p14, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[9] = a; }
    { T a = nl[10]; a = fma(p4, hx, a); a = fma(p15, hz, a); nl[10] = a; }
  }
  else if constexpr (J == 7) {  // v_2
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[6]; a = fma(p1, hx, a); a = fma(p12, hz, a); a = fma(p3, hx, a); a = fma(p14, hz, a); nl[6] = a; }
    { T a = nl[7]; a = fma(p0, px, a); a = fma(p11, pz, a); a = fma(-p4, hx, a); a = fma(-p15, hz, a); nl[7] = a; }
    { T a = nl[8]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[8] = a; }
    { T a = nl[9]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[9] = a; }
    { T a = nl[10]; a = fma(-p3, hx, a); a = fma(-p14, hz, a); nl[10] = a; }
  }
  else if constexpr (J == 8) {  // v_3
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[6]; a = fma(p2, hx, a); a = fma(p13, hz, a); a = fma(p4, hx, a); a = fma(p15, hz, a); nl[6] = a; }
    { T a = nl[7]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[7] = a; }
    { T a = nl[8]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[8] = a; }
    { T a = nl[9]; a = fma(p1, hx, a); a = fma(p12, hz, a); nl[9] = a; }
    { T a = nl[10]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[10] = a; }
  }
  else if constexpr (J == 9) {  // v_4
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p16 = p[16];
    { T a = nl[6]; a = fma(p3, hx, a); a = fma(p14, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[6] = a; }
    { T a = nl[7]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[7] = a; }
    { T a = nl[8]; a = fma(p1, hx, a); a = fma(p12, hz, a); nl[8] = a; }
    { T a = nl[9]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[9] = a; }
    { T a = nl[10]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); nl[10] = a; }
  }
  else if constexpr (J == 10) {  // v_5
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    { T a = nl[6]; a = fma(p4, hx, a); a = fma(p15, hz, a); nl[6] = a; }
    { T a = nl[7]; a = fma(-p3, hx, a); a = fma(-p14, hz, a); nl[7] = a; }
    { T a = nl[8]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[8] = a; }
    { T a = nl[9]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); nl[9] = a; }
    { T a = nl[10]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[10] = a; }
  }
  else if constexpr (J == 11) {  // w_0
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[11]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[11] = a; }
    { T a = nl[12]; a = fma(p1, px, a); a = fma(p12, pz, a); nl[12] = a; }
    { T a = nl[13]; a = fma(p2, px, a); a = fma(p13, pz, a); nl[13] = a; }
    { T a = nl[14]; a = fma(p3, px, a); a = fma(p14, pz, a); nl[14] = a; }
    { T a = nl[15]; a = fma(p4, px, a); a = fma(p15, pz, a); nl[15] = a; }
    { T a = nl[16]; a = fma(p5, px, a); a = fma(p16, pz, a); nl[16] = a; }
  }
  else if constexpr (J == 12) {  // w_1
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[11]; a = fma(p1, hx, a); a = fma(p12, hz, a); nl[11] = a; }
    { T a = nl[12]; a = fma(p0, px, a); a = fma(p11, pz, a); a = fma(-p2, hx, a); a = fma(-p13, hz, a); nl[12] = a; }
    { T a = nl[13]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); a = fma(p3, hx, a); a = fma(p14, hz, a); nl[13] = a; }
    { T a = nl[14]; a = fma(p2, hx, a); a = fma(p13, hz, a); a = fma(-p4, hx, a); a = fma(-p15, hz, a); nl[14] = a; }
    { T a = nl[15]; a = fma(-p3, hx, a); a = fma(-p14, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[15] = a; }
    { T a = nl[16]; a = fma(p4, hx, a); a = fma(p15, hz, a); nl[16] = a; }
  }
  else if constexpr (J == 13) {  // w_2
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[11]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[11] = a; }
    { T a = nl[12]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); a = fma(p3, hx, a); a = fma(p14, hz, a); nl[12] = a; }
    { T a = nl[13]; a = fma(p0, px, a); a = fma(p11, pz, a); a = fma(p4, hx, a); a = fma(p15, hz, a); nl[13] = a; }
    { T a = nl[14]; a = fma(p1, hx, a); a = fma(p12, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[14] = a; }
    { T a = nl[15]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[15] = a; }
    { T a = nl[16]; a = fma(p3, hx, a); a = fma(p14, hz, a); nl[16] = a; }
  }
  else if constexpr (J == 14) {  // w_3
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[11]; a = fma(p3, hx, a); a = fma(p14, hz, a); nl[11] = a; }
    { T a = nl[12]; a = fma(p2, hx, a); a = fma(p13, hz, a); a = fma(-p4, hx, a); a = fma(-p15, hz, a); nl[12] = a; }
    { T a = nl[13]; a = fma(p1, hx, a); a = fma(p12, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[13] = a; }
    { T a = nl[14]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[14] = a; }
    { T a = nl[15]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); nl[15] = a; }
    { T a = nl[16]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[16] = a; }
  }
  else if constexpr (J == 15) {  // w_4
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[11]; a = fma(p4, hx, a); a = fma(p15, hz, a); nl[11] = a; }
    { T a = nl[12]; a = fma(-p3, hx, a); a = fma(-p14, hz, a); a = fma(p5, hx, a); a = fma(p16, hz, a); nl[12] = a; }
    { T a = nl[13]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[13] = a; }
    { T a = nl[14]; a = fma(-p1, hx, a); a = fma(-p12, hz, a); nl[14] = a; }
    { T a = nl[15]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[15] = a; }
    { T a = nl[16]; a = fma(p1, hx, a); a = fma(p12, hz, a); nl[16] = a; }
  }
  else if constexpr (J == 16) {  // w_5
    const T p0 = p[0];
    const T p1 = p[1];
    const T p2 = p[2];
    const T p3 = p[3];
    const T p4 = p[4];
    const T p5 = p[5];
    const T p11 = p[11];
    const T p12 = p[12];
    const T p13 = p[13];
    const T p14 = p[14];
    const T p15 = p[15];
    const T p16 = p[16];
    { T a = nl[11]; a = fma(p5, hx, a); a = fma(p16, hz, a); nl[11] = a; }
    { T a = nl[12]; a = fma(p4, hx, a); a = fma(p15, hz, a); nl[12] = a; }
    { T a = nl[13]; a = fma(p3, hx, a); a = fma(p14, hz, a); nl[13] = a; }
    { T a = nl[14]; a = fma(p2, hx, a); a = fma(p13, hz, a); nl[14] = a; }
    { T a = nl[15]; a = fma(p1, hx, a); a = fma(p12, hz, a); nl[15] = a; }
    { T a = nl[16]; a = fma(p0, px, a); a = fma(p11, pz, a); nl[16] = a; }
  }
}

