// CPU restatement of the MWF timestep in C++ (FP64, OpenMP).  Test and baseline
// infrastructure, not the product: tests check it against the numpy oracle, and the bench's
// CPU legs time it as the CPU implementation of the path, because the reference's own Fortran
// (FFTW3, netCDF, MPI) cannot be built without those libraries and a Fortran compiler.
//
// One step follows vel_TS / vel_nonlinear (program/velocity.f90:21-41, 92-113):
//   var_mpt2spec + vel_addlam + var_spec_grad     (variables.f90:390-434, 600-612; velocity.f90:76-82)
//   tra_spec2phys for u, ux, uz                   (transform.fftw5.f90:64-87)
//   udotgradu at every grid point                 (modes.M4.f90:14-36 / modes.M6.f90:14-20, 22-79)
//   tra_phys2spec, var_spec2mpt                   (transform.fftw5.f90:122-145; variables.f90:440-480)
//   implicit / AB2 update                         (velocity.f90:27-39)
// with the same FFT sign conventions as FFTW (backward e^{+i}, forward e^{-i}, unnormalised,
// c2r ignoring the imaginary part of the n = 0 coefficient, 1/(3MM*3NN) applied before the
// forward transforms).  The transforms are this file's own mixed-radix Stockham FFT (radices
// 4, 2, 3); two real z lines share one complex transform.  Work is split over x lines (z
// pass) and z columns n (x passes), so each thread's lines stay in its caches.
//
// The mode coupling comes in as a list of terms out[d] += coef * P[a] * P[b] over the 3KK
// physical fields P = (u, du/dx, du/dz), built by the caller from the Galerkin tensors.
#include <cmath>
#include <algorithm>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

struct cd { double re, im; };
inline cd add(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
inline cd sub(cd a, cd b) { return {a.re - b.re, a.im - b.im}; }
inline cd mul(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline cd mulc(cd a, cd b) { return {a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im}; }   // a * conj(b)
inline cd conj(cd a) { return {a.re, -a.im}; }

// ---- FFT ----------------------------------------------------------------------------------
struct Plan {
  int N = 0;
  std::vector<int> rad, ns;
  std::vector<std::vector<cd>> tw;    // per stage: e^{-2 pi i r k / (Ns R)} at [k (R-1) + r - 1]
};

bool make_plan(int N, Plan& p) {
  p.N = N;
  int rest = N;
  while (rest % 4 == 0) { p.rad.push_back(4); rest /= 4; }
  while (rest % 2 == 0) { p.rad.push_back(2); rest /= 2; }
  while (rest % 3 == 0) { p.rad.push_back(3); rest /= 3; }
  if (rest != 1) return false;
  int Ns = 1;
  const double two_pi = 2.0 * 3.14159265358979323846;
  for (int R : p.rad) {
    p.ns.push_back(Ns);
    std::vector<cd> t((size_t)Ns * (R - 1));
    for (int k = 0; k < Ns; ++k)
      for (int r = 1; r < R; ++r) {
        const double a = -two_pi * (double)r * k / ((double)Ns * R);
        t[(size_t)k * (R - 1) + r - 1] = {std::cos(a), std::sin(a)};
      }
    p.tw.push_back(std::move(t));
    Ns *= R;
  }
  return true;
}

// Length-R DFT of a[0..R-1] in place (R = 2, 3, 4); BWD = e^{+i}.
template <int R, bool BWD>
inline void dft(cd* a) {
  if constexpr (R == 2) {
    const cd t = a[1];
    a[1] = sub(a[0], t);
    a[0] = add(a[0], t);
  } else if constexpr (R == 4) {
    const cd t0 = add(a[0], a[2]), t1 = sub(a[0], a[2]), t2 = add(a[1], a[3]), t3 = sub(a[1], a[3]);
    const cd it3 = BWD ? cd{-t3.im, t3.re} : cd{t3.im, -t3.re};          // +i t3 or -i t3
    a[0] = add(t0, t2); a[2] = sub(t0, t2);
    a[1] = add(t1, it3); a[3] = sub(t1, it3);
  } else {
    const double h3 = 0.86602540378443864676;                            // sqrt(3) / 2
    const cd s12 = add(a[1], a[2]), d12 = sub(a[1], a[2]);
    const cd t = {a[0].re - 0.5 * s12.re, a[0].im - 0.5 * s12.im};
    const cd sd = {h3 * d12.re, h3 * d12.im};
    const cd isd = BWD ? cd{-sd.im, sd.re} : cd{sd.im, -sd.re};          // +i s or -i s
    a[0] = add(a[0], s12);
    a[1] = add(t, isd); a[2] = sub(t, isd);
  }
}

// One Stockham stage: element j = q Ns + k of each of the R strided inputs, twiddled by
// w^{r k}, transformed, and stored at q Ns R + k + r Ns.
template <int R, bool BWD>
void stage(const cd* __restrict src, cd* __restrict dst, int N, int Ns, const cd* __restrict tw) {
  const int L = N / R;
  for (int q = 0; q < L / Ns; ++q) {
    const cd* s = src + q * Ns;
    cd* d = dst + q * Ns * R;
    for (int k = 0; k < Ns; ++k) {
      cd a[R];
      for (int r = 0; r < R; ++r) a[r] = s[k + r * L];
      if (Ns > 1) {
        const cd* t = tw + (size_t)k * (R - 1);
        for (int r = 1; r < R; ++r) a[r] = BWD ? mulc(a[r], t[r - 1]) : mul(a[r], t[r - 1]);
      }
      dft<R, BWD>(a);
      for (int r = 0; r < R; ++r) d[k + r * Ns] = a[r];
    }
  }
}

// In-place transform of x (length N) with scratch w (length N); bwd = e^{+i}.
void fft(const Plan& p, cd* x, cd* w, bool bwd) {
  const int N = p.N;
  cd* src = x;
  cd* dst = w;
  for (size_t s = 0; s < p.rad.size(); ++s) {
    const int R = p.rad[s], Ns = p.ns[s];
    const cd* tw = p.tw[s].data();
    if (R == 4) bwd ? stage<4, true>(src, dst, N, Ns, tw) : stage<4, false>(src, dst, N, Ns, tw);
    else if (R == 2) bwd ? stage<2, true>(src, dst, N, Ns, tw) : stage<2, false>(src, dst, N, Ns, tw);
    else bwd ? stage<3, true>(src, dst, N, Ns, tw) : stage<3, false>(src, dst, N, Ns, tw);
    cd* t = src; src = dst; dst = t;
  }
  if (src != x) std::memcpy(x, src, sizeof(cd) * N);
}

struct Term { int d, a, b; double coef; };

struct Cpu {
  int K0, MM, NN, K, KK, M, X, Z;
  double alpha, gamma, dt, cth, sth;
  std::vector<double> lhs, rhs, m1, n1, k1;
  std::vector<Term> terms;
  Plan px, pz;
  std::vector<cd> T, NLT;
};

inline int signed_m(int ms, int MM, int M) { return ms <= MM - 1 ? ms : ms - M; }

// var_mpt2spec (+ vel_addlam when lam) of one (m, n) column: s[0..KK-1].
void mpt2spec_col(const Cpu& P, const cd* cc, int ms, int n, bool lam, cd* s) {
  const int K0 = P.K0;
  const double M1 = P.m1[ms], N1 = P.n1[n], H = -(M1 * M1) - N1 * N1;
  if (ms == 0 && n == 0) {
    for (int f = 0; f < P.KK; ++f) s[f] = {0.0, 0.0};
    for (int k = 1; k < K0; ++k) {
      s[k] = cc[k];
      s[k + 2 * K0 - 1] = cc[k + K0 - 1];
    }
    if (lam) {
      s[1].re += P.cth;
      s[2 * K0].re += P.sth;
    }
    return;
  }
  for (int k = 0; k < K0; ++k) {
    const cd psi = cc[k], phi = cc[k + K0 - 1];
    const double k1 = P.k1[k];
    s[k] = {-(-psi.im * N1 + phi.im * k1 * M1), -psi.re * N1 + phi.re * k1 * M1};
    s[k + K0 - 1] = {-phi.re * H, -(phi.im * H)};
    s[k + 2 * K0 - 1] = {-(psi.im * M1 + phi.im * k1 * N1), psi.re * M1 + phi.re * k1 * N1};
  }
}

// var_spec2mpt of one column: c[0..K-1] from s[0..KK-1].
void spec2mpt_col(const Cpu& P, const cd* s, int ms, int n, cd* c) {
  const int K0 = P.K0;
  const double M1 = P.m1[ms], N1 = P.n1[n], H = -(M1 * M1) - N1 * N1;
  for (int k = 0; k < K0; ++k) {
    const cd su = s[k], sv = s[k + K0 - 1], sw = s[k + 2 * K0 - 1];
    const double k1 = P.k1[k];
    c[k + K0 - 1] = {-(su.im * M1 * k1 + sw.im * N1 * k1) + sv.re * H,
                     (su.re * M1 * k1 + sw.re * N1 * k1) + sv.im * H};
    c[k] = {sw.im * M1 - su.im * N1, -(sw.re * M1 - su.re * N1)};
  }
  if (ms == 0 && n == 0) {
    c[0] = {0.0, 0.0};
    for (int k = 1; k < K0; ++k) {
      c[k] = {-s[k].re, -s[k].im};
      c[k + K0 - 1] = {-s[k + 2 * K0 - 1].re, -s[k + 2 * K0 - 1].im};
    }
  }
}

// Columns n per x-pass work item: T and NLT are [f][x][n], so a block of kNB columns writes
// (reads) kNB * 16 contiguous bytes per (f, x) instead of single elements.
constexpr int kNB = 4;

// x forward (spec -> x lines) for the 3KK fields u, du/dx, du/dz; T[f][x][n].
void x_forward(Cpu& P, const cd* c) {
  const int NN = P.NN, M = P.M, MM = P.MM, X = P.X, KK = P.KK, K = P.K;
  const int F = 3 * KK;
  const int nblk = (NN + kNB - 1) / kNB;
#pragma omp parallel
  {
    std::vector<cd> spec((size_t)kNB * M * KK), lines((size_t)kNB * X), w(X);
#pragma omp for schedule(static)
    for (int blk = 0; blk < nblk; ++blk) {
      const int n0 = blk * kNB, nb = std::min(kNB, NN - n0);
      for (int i = 0; i < nb; ++i)
        for (int ms = 0; ms < M; ++ms)
          mpt2spec_col(P, c + ((size_t)(n0 + i) * M + ms) * K, ms, n0 + i, true,
                       spec.data() + ((size_t)i * M + ms) * KK);
      for (int f = 0; f < F; ++f) {
        const int g = f % KK, part = f / KK;          // part 0: u, 1: du/dx, 2: du/dz
        for (int i = 0; i < nb; ++i) {
          cd* l = lines.data() + (size_t)i * X;
          std::fill(l, l + X, cd{0.0, 0.0});
          const double gn = P.n1[n0 + i];
          for (int ms = 0; ms < M; ++ms) {
            const int m = signed_m(ms, MM, M);
            const cd v = spec[((size_t)i * M + ms) * KK + g];
            const double fac = part == 1 ? P.m1[ms] : gn;
            l[m < 0 ? m + X : m] = part == 0 ? v : cd{-v.im * fac, v.re * fac};
          }
          fft(P.px, l, w.data(), true);
        }
        cd* out = P.T.data() + (size_t)f * X * NN + n0;
        for (int x = 0; x < X; ++x)
          for (int i = 0; i < nb; ++i) out[(size_t)x * NN + i] = lines[(size_t)i * X + x];
      }
    }
  }
}

// z pass per x line: c2r of the 3KK fields, the coupling terms, r2c of the KK results.
constexpr int kZC = 64;

void z_pass(Cpu& P) {
  const int NN = P.NN, X = P.X, Z = P.Z, KK = P.KK;
  const int F = 3 * KK;
  const double scale = 1.0 / ((double)X * (double)Z);
#pragma omp parallel
  {
    std::vector<double> ph((size_t)F * Z), out((size_t)KK * Z);
    std::vector<cd> h(Z), w(Z);
#pragma omp for schedule(static)
    for (int x = 0; x < X; ++x) {
      for (int f = 0; f < F; f += 2) {
        const bool two = f + 1 < F;
        const cd* la = P.T.data() + ((size_t)f * X + x) * NN;
        const cd* lb = two ? P.T.data() + ((size_t)(f + 1) * X + x) * NN : nullptr;
        std::fill(h.begin(), h.end(), cd{0.0, 0.0});
        h[0] = {la[0].re, two ? lb[0].re : 0.0};
        for (int n = 1; n < NN; ++n) {
          const cd a = la[n], b = two ? lb[n] : cd{0.0, 0.0};
          h[n] = {a.re - b.im, a.im + b.re};          // a + i b
          h[Z - n] = {a.re + b.im, b.re - a.im};      // conj(a) + i conj(b)
        }
        fft(P.pz, h.data(), w.data(), true);
        double* pa = ph.data() + (size_t)f * Z;
        for (int z = 0; z < Z; ++z) pa[z] = h[z].re;
        if (two) {
          double* pb = ph.data() + (size_t)(f + 1) * Z;
          for (int z = 0; z < Z; ++z) pb[z] = h[z].im;
        }
      }
      // coupling terms over chunks of kZC points, so the chunk's fields stay in L1
      std::fill(out.begin(), out.end(), 0.0);
      for (int z0 = 0; z0 < Z; z0 += kZC) {
        const int zn = std::min(kZC, Z - z0);
        for (const Term& t : P.terms) {
          double* o = out.data() + (size_t)t.d * Z + z0;
          const double* a = ph.data() + (size_t)t.a * Z + z0;
          const double* b = ph.data() + (size_t)t.b * Z + z0;
          const double cf = t.coef;
          for (int z = 0; z < zn; ++z) o[z] += cf * a[z] * b[z];
        }
      }
      for (int d = 0; d < KK; d += 2) {
        const bool two = d + 1 < KK;
        const double* oa = out.data() + (size_t)d * Z;
        const double* ob = two ? out.data() + (size_t)(d + 1) * Z : nullptr;
        for (int z = 0; z < Z; ++z) h[z] = {scale * oa[z], two ? scale * ob[z] : 0.0};
        fft(P.pz, h.data(), w.data(), false);
        cd* na = P.NLT.data() + ((size_t)d * X + x) * NN;
        cd* nb = two ? P.NLT.data() + ((size_t)(d + 1) * X + x) * NN : nullptr;
        for (int n = 0; n < NN; ++n) {
          const cd hn = h[n], hm = conj(h[n == 0 ? 0 : Z - n]);
          na[n] = {0.5 * (hn.re + hm.re), 0.5 * (hn.im + hm.im)};
          if (two) nb[n] = {0.5 * (hn.im - hm.im), -0.5 * (hn.re - hm.re)};   // (hn - hm) / (2i)
        }
      }
    }
  }
}

// x inverse per block of columns n: forward x transforms of the KK fields, truncation,
// spec2mpt and the implicit / AB2 update.
void x_inverse(Cpu& P, cd* c, cd* onl, bool first) {
  const int NN = P.NN, M = P.M, MM = P.MM, X = P.X, KK = P.KK, K = P.K;
  const double hdt = P.dt / 2.0;
  const int nblk = (NN + kNB - 1) / kNB;
#pragma omp parallel
  {
    std::vector<cd> lines((size_t)kNB * KK * X), w(X), s(KK), nl(K);
#pragma omp for schedule(static)
    for (int blk = 0; blk < nblk; ++blk) {
      const int n0 = blk * kNB, nb = std::min(kNB, NN - n0);
      for (int d = 0; d < KK; ++d) {
        const cd* in = P.NLT.data() + (size_t)d * X * NN + n0;
        for (int x = 0; x < X; ++x)
          for (int i = 0; i < nb; ++i) lines[((size_t)i * KK + d) * X + x] = in[(size_t)x * NN + i];
        for (int i = 0; i < nb; ++i) fft(P.px, lines.data() + ((size_t)i * KK + d) * X, w.data(), false);
      }
      for (int i = 0; i < nb; ++i) {
        const int n = n0 + i;
        const cd* li = lines.data() + (size_t)i * KK * X;
        for (int ms = 0; ms < M; ++ms) {
          const int m = signed_m(ms, MM, M);
          const int x = m < 0 ? m + X : m;
          for (int d = 0; d < KK; ++d) s[d] = li[(size_t)d * X + x];
          spec2mpt_col(P, s.data(), ms, n, nl.data());
          const size_t o = ((size_t)n * M + ms) * K;
          for (int k = 0; k < K; ++k) {
            const cd on = first ? nl[k] : onl[o + k];
            const double r = P.rhs[o + k], l = P.lhs[o + k];
            cd v = {r * c[o + k].re + hdt * (3.0 * nl[k].re - on.re),
                    r * c[o + k].im + hdt * (3.0 * nl[k].im - on.im)};
            v = {v.re / l, v.im / l};
            c[o + k] = v;
            onl[o + k] = nl[k];
          }
          if (ms == 0 && n == 0) c[o].re = 0.0;
        }
      }
    }
  }
}

}  // namespace

extern "C" {

// Tables in the reference layouts: lhs, rhs (NN, M, K) real; m1[M] = alpha*m per slot,
// n1[NN] = gamma*n, k1[K0]; terms as (d, a, b) int triples + coefficients.
void* mwfcpu_create(int K0, int MM, int NN, double alpha, double gamma, double dt, double cth, double sth,
                    const double* lhs, const double* rhs, const double* m1, const double* n1, const double* k1,
                    int nterms, const int* tidx, const double* tcoef) {
  Cpu* P = new Cpu;
  P->K0 = K0; P->MM = MM; P->NN = NN;
  P->K = 2 * K0 - 1; P->KK = 3 * K0 - 1; P->M = 2 * MM - 1; P->X = 3 * MM; P->Z = 3 * NN;
  P->alpha = alpha; P->gamma = gamma; P->dt = dt; P->cth = cth; P->sth = sth;
  const size_t csz = (size_t)NN * P->M * P->K;
  P->lhs.assign(lhs, lhs + csz);
  P->rhs.assign(rhs, rhs + csz);
  P->m1.assign(m1, m1 + P->M);
  P->n1.assign(n1, n1 + NN);
  P->k1.assign(k1, k1 + K0);
  for (int i = 0; i < nterms; ++i) P->terms.push_back({tidx[3 * i], tidx[3 * i + 1], tidx[3 * i + 2], tcoef[i]});
  if (!make_plan(P->X, P->px) || !make_plan(P->Z, P->pz)) { delete P; return nullptr; }
  P->T.assign((size_t)3 * P->KK * P->X * NN, cd{0.0, 0.0});
  P->NLT.assign((size_t)P->KK * P->X * NN, cd{0.0, 0.0});
  return P;
}

void mwfcpu_destroy(void* h) { delete static_cast<Cpu*>(h); }

// c, onl: interleaved complex (NN, M, K).  *nst = 1 makes the first step the Euler start
// (the history is then ignored); it is cleared after that step.
int mwfcpu_step(void* h, double* c, double* onl, int* nst, int nsteps, int threads) {
  Cpu* P = static_cast<Cpu*>(h);
  if (!P) return -1;
  if (threads > 0) omp_set_num_threads(threads);
  cd* cc = reinterpret_cast<cd*>(c);
  cd* oo = reinterpret_cast<cd*>(onl);
  for (int s = 0; s < nsteps; ++s) {
    x_forward(*P, cc);
    z_pass(*P);
    x_inverse(*P, cc, oo, *nst != 0);
    *nst = 0;
  }
  return 0;
}

}  // extern "C"
