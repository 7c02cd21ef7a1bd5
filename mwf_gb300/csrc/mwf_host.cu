// C-ABI implementation (include/mwf_gpu.h): plans, FP64 tables, device arena, work lists,
// CUDA-graph replay of the timestep, state copies and the energy diagnostic.
#include <cmath>
#include <cstddef>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "../../include/mwf_gpu.h"
#include "mwf_common.cuh"
#include "mwf_launch.h"

using namespace mwf;

namespace {

thread_local char g_err[512];

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return fail(MWF_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

constexpr int kMaxLen = 4096;      // longest x line (3*MM) supported by the plans
constexpr int kMaxNN = 1024;       // longest z half-line (NN) supported by the z pass
constexpr size_t kSmemLimit = 200 * 1024;

bool is_23_smooth(int n) {
  if (n < 1) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  return n == 1;
}

// Radix plan for N = 2^a 3^b with radices up to maxr (8, 12 or 16): as few stages as
// possible.  Each 3 pairs with a 4 into a radix-12 stage while both are left (maxr >= 12),
// leftover 3s are radix-3 stages, and the power of two is split into the fewest stages of
// 16/8/4/2, balanced toward 8s.
bool make_plan(int N, FftPlanDev& pl, int maxr) {
  if (!is_23_smooth(N) || N < 2) return false;
  int a = 0, b = 0, rest = N;
  while (rest % 2 == 0) { rest /= 2; ++a; }
  while (rest % 3 == 0) { rest /= 3; ++b; }
  std::vector<int> rad;
  if (maxr >= 12) {
    while (b > 0 && a >= 2) { rad.push_back(12); --b; a -= 2; }
  }
  while (b > 0) { rad.push_back(3); --b; }
  static const int p16[13][3] = {{0, 0, 0}, {2, 0, 0}, {4, 0, 0}, {8, 0, 0}, {16, 0, 0}, {8, 4, 0},
                                 {8, 8, 0}, {16, 8, 0}, {16, 16, 0}, {8, 8, 8}, {16, 8, 8}, {16, 16, 8},
                                 {16, 16, 16}};
  while (a > 0) {
    if (maxr >= 16) {
      const int take = std::min(a, 12);
      for (int i = 0; i < 3 && p16[take][i]; ++i) rad.push_back(p16[take][i]);
      a -= take;
    } else {
      const int take = a >= 3 ? 3 : a;
      rad.push_back(1 << take);
      a -= take;
    }
  }
  if ((int)rad.size() > MWF_MAX_STAGES) return false;
  pl.N = N;
  pl.nst = 0;
  int ns = 1;
  for (int r : rad) {
    pl.radix[pl.nst] = r;
    pl.ns[pl.nst] = ns;
    pl.fnb[pl.nst] = make_fastdiv(N / r);
    pl.fns[pl.nst] = make_fastdiv(ns);
    ++pl.nst;
    ns *= r;
  }
  return ns == N;
}

// tw[t] = exp(-2 pi i t / N) for t in [t0, t0 + cnt), evaluated in long double and rounded
// once; out receives 2*cnt values (re, im interleaved).
template <typename T>
void twiddles_into(int N, int t0, int cnt, T* out) {
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int t = t0; t < t0 + cnt; ++t) {
    // reduce by symmetry so the argument stays in [0, pi/4]
    long double c, s;
    const int q8 = 8 * t;               // angle = 2 pi t/N = (pi/4) * (8t/N)
    if (q8 % N == 0) {
      const int oct = q8 / N;           // exact multiples of pi/4
      const long double h = 0.707106781186547524400844362104849039L;
      static const int cs[8][2] = {{2, 0}, {1, 1}, {0, 2}, {-1, 1}, {-2, 0}, {-1, -1}, {0, -2}, {1, -1}};
      auto val = [&](int v) -> long double { return v == 2 ? 1.0L : v == -2 ? -1.0L : v * h; };
      c = val(cs[oct][0]);
      s = val(cs[oct][1]);
    } else {
      const long double a = two_pi * (long double)t / (long double)N;
      c = cosl(a);
      s = sinl(a);
    }
    out[2 * (size_t)(t - t0)] = (T)c;
    out[2 * (size_t)(t - t0) + 1] = (T)(-s);
  }
}

template <typename T>
std::vector<T> twiddles(int N) {
  std::vector<T> out(2 * (size_t)N);
  twiddles_into<T>(N, 0, N, out.data());
  return out;
}

// var_precompute tables (variables.f90:516-531) and var_LHSRHS (variables.f90:565-597) in
// the reference's loop order, stored in the device layout [n][k][m].
void lhsrhs(const mwf_run_desc& d, std::vector<double>& inv_lhs, std::vector<double>& rhs) {
  const int MM = d.MM, NN = d.NN, K0 = d.K0, M = 2 * (MM - 1) + 1, K = 2 * K0 - 1;
  const double beta = 3.1415926535897931 / 2.0;
  std::vector<double> m2(M), n2(NN), k2(K0);
  for (int m = 0; m < MM; ++m) {
    if (m > 0) m2[M - m] = -d.alpha * m * d.alpha * m;
    m2[m] = -d.alpha * m * d.alpha * m;
  }
  for (int n = 0; n < NN; ++n) n2[n] = -d.gamma * n * d.gamma * n;
  for (int k = 0; k < K0; ++k) k2[k] = -k * k * beta * beta;
  std::vector<double> L((size_t)NN * K * M), R((size_t)NN * K * M);
  auto at = [&](std::vector<double>& a, int k, int m, int n) -> double& { return a[((size_t)n * K + k) * M + m]; };
  for (int n = 0; n < NN; ++n)
    for (int m = 0; m < M; ++m)
      for (int k = 0; k < K0; ++k) {
        const int a = k, b = k + K0 - 1;
        const double lap = m2[m] + k2[k] + n2[n];
        const double hlap = m2[m] + n2[n];
        const double ilap16 = d.hypo / (m2[m] + k2[k] + n2[n]);
        double tvl;
        if (d.dragall || k == 0) tvl = 1.0 - d.dt * (lap / d.Re + ilap16 - d.drag);
        else tvl = 1.0 - d.dt * (lap / d.Re + ilap16);
        if (m == 0 && n == 0) {
          at(L, a, m, n) = tvl;
          at(L, b, m, n) = tvl;
          at(R, a, m, n) = 1.0;
          at(R, b, m, n) = 1.0;
          at(L, 0, m, n) = 1.0;
          at(R, 0, m, n) = 0.0;
        } else {
          at(L, a, m, n) = tvl * hlap;
          if (d.dragall) at(L, b, m, n) = tvl * hlap * lap + d.dt * (d.vdrag - d.drag) * hlap * hlap;
          else at(L, b, m, n) = tvl * hlap * lap;
          at(R, a, m, n) = hlap;
          at(R, b, m, n) = hlap * lap;
        }
      }
  inv_lhs.resize(L.size());
  for (size_t i = 0; i < L.size(); ++i) inv_lhs[i] = 1.0 / L[i];
  rhs.swap(R);
}

struct RunHost {
  mwf_run_desc d;
  int K, KK, M, X, Z;
  size_t csz;        // complex elements of c
  size_t off_c, off_onl, off_ilhs, off_rhs, off_T, off_NLT, off_twX, off_twQ, off_twZ, off_nst;
  int n_diag_xf, n_diag_z;   // work items of the physical-space diagnostic
  int xf_nb, xi_nb, z_lx;
  int z_ppt, z_nt;
  int x_nt;          // block size of the x passes
  int x_radix, z_radix;
  int zb_lx = 0;     // x lines per item of the batched FP32 z pass (0: z_nonlinear_kernel)
  int xbf_nb = 0, xbi_nb = 0;   // columns per item of the subset-split FP32 x passes (0: not used)
  bool persist = false;         // all three passes batched: the run steps in the persistent kernel
  int active = 1;    // host copy of RunDesc::active
};

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Tiling of one run; returns false if the run does not fit the kernels' shapes.
bool plan_run(RunHost& r, const char*& why) {
  const mwf_run_desc& d = r.d;
  if (d.K0 != 4 && d.K0 != 6) { why = "K0 must be 4 (M4) or 6 (M6)"; return false; }
  if (d.MM < 2 || d.NN < 2) { why = "MM and NN must be >= 2"; return false; }
  if (!is_23_smooth(d.MM) || !is_23_smooth(d.NN)) { why = "MM and NN must be of the form 2^a 3^b"; return false; }
  r.K = 2 * d.K0 - 1;
  r.KK = 3 * d.K0 - 1;
  r.M = 2 * (d.MM - 1) + 1;
  r.X = 3 * d.MM;
  r.Z = 3 * d.NN;
  if (r.X > kMaxLen) { why = "3*MM exceeds the longest supported x line (4096)"; return false; }
  if (d.NN > kMaxNN) { why = "NN exceeds the longest supported z half-line (1024)"; return false; }
  if (d.precision != MWF_FP64 && d.precision != MWF_FP32) { why = "precision must be MWF_FP64 or MWF_FP32"; return false; }
  const size_t cb = d.precision == MWF_FP64 ? 16 : 8;
  // x forward: nb*X <= VPT*threads, smem <= limit; equal tiles
  r.x_nt = xpass_threads(d.precision, r.X);
  const int xfv = xf_vpt(d.precision);
  // the FP64 x forward also holds its wavenumber tables in static shared memory
  const size_t xf_smem = kSmemLimit - (d.precision == MWF_FP64 ? kXTabBytes : 0);
  int nbmax = std::min(xfv * r.x_nt / r.X, (int)(xf_smem / (r.X * cb * 9 / 8 + cb)));
  nbmax = std::max(1, std::min(nbmax, d.NN));
  if (nbmax * r.X > xfv * r.x_nt) { why = "x line too long for the x-forward pass"; return false; }
  r.xf_nb = d.NN / ((d.NN + nbmax - 1) / nbmax);
  while (r.xf_nb > 1 && d.NN % r.xf_nb) --r.xf_nb;
  // FP32 runs whose MM has a compile-time plan use the subset-split x passes unless an x radix
  // cap is given (which selects x_forward_kernel / x_inverse_kernel and their run-time plans);
  // the column knobs then apply to them
  const bool xb = d.precision == MWF_FP32 && d.x_radix == 0 && xb_supported(d.MM);
  r.xbf_nb = r.xbi_nb = 0;
  if (xb) {
    auto widest = [&](size_t (*smem)(int, int), size_t budget) {
      int nb = 1;
      while (nb < 8 && nb < d.NN && smem(d.MM, nb + 1) <= budget) ++nb;
      return nb;
    };
    const size_t fbudget = zb_smem_budget(kXfBlocks), ibudget = zb_smem_budget(kXiBlocks);
    const int fmax = widest(xbf_smem, fbudget), imax = widest(xbi_smem, ibudget);
    if (xbf_smem(d.MM, 1) > fbudget || xbi_smem(d.MM, 1) > ibudget) { why = "x line too long for the x passes"; return false; }
    r.xbf_nb = fmax;
    r.xbi_nb = imax;
    if (d.xf_cols) {
      if (d.xf_cols < 1 || d.xf_cols > std::min(fmax, d.NN)) { why = "xf_cols out of range for this run"; return false; }
      r.xbf_nb = d.xf_cols;
    }
    if (d.xi_cols) {
      if (d.xi_cols < 1 || d.xi_cols > std::min(imax, d.NN)) { why = "xi_cols out of range for this run"; return false; }
      r.xbi_nb = d.xi_cols;
    }
  }
  if (d.xf_cols && !xb) {
    if (d.xf_cols < 1 || d.xf_cols > nbmax) { why = "xf_cols out of range for this run"; return false; }
    r.xf_nb = d.xf_cols;
  }
  // x inverse: nb*X <= VPT*threads per field, three fields resident
  nbmax = std::min(kXiVpt * r.x_nt / r.X, (int)(kSmemLimit / (3 * r.X * cb * 9 / 8 + cb)));
  nbmax = std::max(1, std::min(nbmax, d.NN));
  if (nbmax * r.X > kXiVpt * r.x_nt) { why = "x line too long for the x-inverse pass"; return false; }
  r.xi_nb = d.NN / ((d.NN + nbmax - 1) / nbmax);
  while (r.xi_nb > 1 && d.NN % r.xi_nb) --r.xi_nb;
  if (d.xi_cols && !xb) {
    if (d.xi_cols < 1 || d.xi_cols > nbmax) { why = "xi_cols out of range for this run"; return false; }
    r.xi_nb = d.xi_cols;
  }
  // z pass: points per CTA = threads * points-per-thread >= NN
  r.z_ppt = d.NN <= kZThreads ? 1 : 2;
  r.z_nt = (d.precision == MWF_FP32 && d.NN <= kZThreadsSmall) ? kZThreadsSmall : kZThreads;
  if (d.K0 == 6 && d.precision == MWF_FP64 && r.z_ppt == 2) {
    why = "M6 in FP64 supports NN <= 512";
    return false;
  }
  r.z_lx = std::max(1, r.z_nt * r.z_ppt / d.NN);
  r.z_lx = std::min(r.z_lx, r.X);
  // FP32 runs whose z line length has a compile-time plan use the batched z pass unless a z
  // radix cap is given (which selects z_nonlinear_kernel and its run-time plans)
  r.zb_lx = 0;
  if (d.precision == MWF_FP32 && d.z_radix == 0 && zb_supported(d.K0, d.NN)) {
    const size_t budget = zb_smem_budget(zb_blocks_per_sm(d.K0, d.NN));
    int L = 1;
    while (L < r.X && zb_smem(d.K0, d.NN, L + 1) <= budget) ++L;
    if (d.z_lines) {
      if (d.z_lines < 1 || d.z_lines > L) { why = "z_lines out of range for this run"; return false; }
      L = d.z_lines;
    }
    r.zb_lx = L;
  } else if (d.z_lines) {
    if (d.z_lines < 1 || d.z_lines > r.z_lx) { why = "z_lines out of range for this run"; return false; }
    r.z_lx = d.z_lines;
  }
  // largest radix: the kernels' compile-time caps (x: 12 FP64 / 16 FP32; z: 8 / 12)
  const int xcap = d.precision == MWF_FP64 ? 12 : 16, zcap = d.precision == MWF_FP64 ? 8 : 12;
  auto radix_ok = [](int v, int cap) { return v == 0 || ((v == 8 || v == 12 || v == 16) && v <= cap); };
  if (!radix_ok(d.x_radix, xcap) || !radix_ok(d.z_radix, zcap)) { why = "x_radix/z_radix must be 8, 12 or 16 within the pass caps"; return false; }
  r.x_radix = d.x_radix ? d.x_radix : xcap;
  r.z_radix = d.z_radix ? d.z_radix : zcap;
  r.n_diag_xf = ((d.NN + r.xf_nb - 1) / r.xf_nb) * r.KK;
  r.n_diag_z = ((r.X + r.z_lx - 1) / r.z_lx) * 3;
  return true;
}

size_t run_bytes(RunHost& r, size_t base) {
  const size_t cb = r.d.precision == MWF_FP64 ? 16 : 8;
  size_t o = base;
  r.csz = (size_t)r.K * r.M * r.d.NN;
  r.off_c = o; o = align_up(o + r.csz * cb, 256);
  r.off_onl = o; o = align_up(o + r.csz * cb, 256);
  r.off_ilhs = o; o = align_up(o + r.csz * 8, 256);
  r.off_rhs = o; o = align_up(o + r.csz * 8, 256);
  r.off_T = o; o = align_up(o + (size_t)2 * r.KK * r.X * r.d.NN * cb, 256);
  r.off_NLT = o; o = align_up(o + (size_t)3 * r.KK * r.X * r.d.NN * cb, 256);   // one partial per z-subset
  r.off_twX = o; o = align_up(o + (size_t)r.X * cb, 256);
  r.off_twQ = o; o = align_up(o + (size_t)r.d.NN * cb, 256);
  r.off_twZ = o; o = align_up(o + (size_t)r.Z * cb, 256);
  r.off_nst = o; o = align_up(o + sizeof(int), 256);
  return o;
}

struct Launch {
  int kind;       // 0 x-forward, 1 z pass, 2 x-inverse
  int prec, K0, ppt, nt;
  size_t smem;
  size_t item_off; // offset into the device item array
  int nitems;
  int zbQ = 0;     // z pass: 0 = z_nonlinear_kernel, else the batched FP32 z pass for NN = zbQ
  int xbMM = 0;    // x passes: 0 = x_forward_kernel / x_inverse_kernel, else the subset-split
                   // FP32 kernels for MM = xbMM
  bool persist_group = false;   // its runs can step in the persistent kernel instead (step mode)
};

cudaError_t launch_pass(const Launch& L, const RunDesc* runs, const WorkItem* items, int* err, cudaStream_t st) {
  if (L.kind == 0 && L.xbMM) return launch_x_forward_batched(L.xbMM, runs, items, L.nitems, L.smem, err, st);
  if (L.kind == 2 && L.xbMM) return launch_x_inverse_batched(L.xbMM, runs, items, L.nitems, L.smem, err, st);
  if (L.kind == 0)
    return L.prec == 0 ? launch_x_forward_f64(L.nt, runs, items, L.nitems, L.smem, err, st)
                       : launch_x_forward_f32(L.nt, runs, items, L.nitems, L.smem, err, st);
  if (L.kind == 1) {
    if (L.zbQ) return launch_z_batched(L.K0, L.zbQ, runs, items, L.nitems, L.smem, err, st);
    return L.prec == 0 ? launch_z_nonlinear_f64(L.K0, L.ppt, L.nt, runs, items, L.nitems, L.smem, err, st)
                       : launch_z_nonlinear_f32(L.K0, L.ppt, L.nt, runs, items, L.nitems, L.smem, err, st);
  }
  return L.prec == 0 ? launch_x_inverse_f64(L.nt, runs, items, L.nitems, L.smem, err, st)
                     : launch_x_inverse_f32(L.nt, runs, items, L.nitems, L.smem, err, st);
}

}  // namespace

struct mwf_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<RunHost> runs;
  unsigned char* arena = nullptr;
  size_t arena_bytes = 0;
  RunDesc* d_runs = nullptr;
  WorkItem* d_items = nullptr;
  WorkItem* d_diag_items = nullptr;  // scratch for one run's diagnostic work items
  int* d_err = nullptr;
  int* d_flag = nullptr;
  double* d_partial = nullptr;
  double* d_eout = nullptr;
  double* d_stage = nullptr;     // 2 * max(csz) doubles for state copies
  size_t stage_elems = 0;
  std::vector<Launch> launches;
  size_t off_nst_all = 0;            // arena offset of the runs' Euler-start flags (one int each)
  // persistent FP32 step: its items, counters (cleared before every launch), shared memory, grid
  void* d_pitems = nullptr;
  int n_pitems = 0;
  int* d_counters = nullptr;
  size_t counters_bytes = 0;
  size_t persist_smem = 0;
  int persist_grid = 0;
  bool persist_mode = false;         // step with the persistent kernel (mwf_set_persistent)
  bool any_sym = false;
  cudaGraphExec_t graph1 = nullptr;   // one step
  cudaGraphExec_t graphG = nullptr;   // kGraphSteps steps
  static constexpr int kGraphSteps = 16;
  static constexpr int kEnergyParts = 256;
};

namespace {

int enqueue_step(mwf_handle* h) {
  cudaStream_t st = h->stream;
  if (h->any_sym) {
    for (size_t i = 0; i < h->runs.size(); ++i) {
      const RunHost& r = h->runs[i];
      const int modes[3] = {r.d.reflect, r.d.uvreflect, r.d.wreflect};
      for (int mode = 0; mode < 3; ++mode) {
        if (!modes[mode]) continue;
        cudaError_t e = r.d.precision == MWF_FP64
                            ? launch_imposesym_f64(h->d_runs, (int)i, mode, r.M, r.d.NN, st)
                            : launch_imposesym_f32(h->d_runs, (int)i, mode, r.M, r.d.NN, st);
        if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "imposesym launch: %s", cudaGetErrorString(e));
      }
    }
  }
  const bool persist = h->persist_mode && h->n_pitems;
  if (persist) {
    cudaError_t e = cudaMemsetAsync(h->d_counters, 0, h->counters_bytes, st);
    if (e == cudaSuccess)
      e = launch_persistent_step(h->d_runs, h->d_pitems, h->n_pitems, h->d_counters, h->persist_smem,
                                 h->persist_grid, h->d_err, st);
    if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "persistent step launch: %s", cudaGetErrorString(e));
  }
  for (const Launch& L : h->launches) {
    if (persist && L.persist_group) continue;
    cudaError_t e = launch_pass(L, h->d_runs, h->d_items + L.item_off, h->d_err, st);
    if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "pass %d launch: %s", L.kind, cudaGetErrorString(e));
  }
  // the Euler start applies to one step only (velocity.f90:24-27)
  cudaError_t e = cudaMemsetAsync(h->arena + h->off_nst_all, 0, sizeof(int) * h->runs.size(), st);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "nst reset: %s", cudaGetErrorString(e));
  return MWF_OK;
}

int build_graph(mwf_handle* h, int steps, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int rc = MWF_OK;
  for (int s = 0; s < steps && rc == MWF_OK; ++s) rc = enqueue_step(h);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (rc != MWF_OK) { if (g) cudaGraphDestroy(g); return rc; }
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  return MWF_OK;
}

int check_device_err(mwf_handle* h) {
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (herr) return fail(MWF_ERR_DEVICE, "kernel reported internal error flags 0x%x", herr);
  return MWF_OK;
}

void free_handle(mwf_handle* h) {
  if (!h) return;
  if (h->graph1) cudaGraphExecDestroy(h->graph1);
  if (h->graphG) cudaGraphExecDestroy(h->graphG);
  if (h->arena) cudaFree(h->arena);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

}  // namespace

extern "C" {

long long mwf_run_dof(const mwf_run_desc* d) {
  if (!d) return 0;
  return (long long)(2 * d->K0 - 1) * (2 * (d->MM - 1) + 1) * d->NN;
}

long long mwf_footprint_bytes(const mwf_run_desc* runs, int n_runs) {
  if (!runs || n_runs <= 0) return -1;
  size_t o = 0;
  size_t stage = 0;
  for (int i = 0; i < n_runs; ++i) {
    RunHost r;
    r.d = runs[i];
    const char* why = "";
    if (!plan_run(r, why)) return -1;
    o = run_bytes(r, o);
    stage = std::max(stage, r.csz);
  }
  return (long long)(o + 2 * stage * sizeof(double) + 4096 + (size_t)n_runs * sizeof(RunDesc));
}

int mwf_describe_run(const mwf_run_desc* d, mwf_run_plan* out) {
  if (!d || !out) return fail(MWF_ERR_ARG, "mwf_describe_run: null argument");
  RunHost r;
  r.d = *d;
  const char* why = "";
  if (!plan_run(r, why)) return fail(MWF_ERR_SIZE, "mwf_describe_run: %s", why);
  const int prec = d->precision == MWF_FP64 ? 0 : 1;
  mwf_run_plan p;
  memset(&p, 0, sizeof p);
  p.batched_x = r.xbf_nb ? 1 : 0;
  p.batched_z = r.zb_lx ? 1 : 0;
  if (p.batched_x) {
    p.xf_cols = r.xbf_nb;
    p.xi_cols = r.xbi_nb;
    p.xf_ctas_per_sm = kXfBlocks;
    p.xi_ctas_per_sm = kXiBlocks;
    p.xf_smem = (long long)xbf_smem(d->MM, r.xbf_nb);
    p.xi_smem = (long long)xbi_smem(d->MM, r.xbi_nb);
    p.xf_items = ((d->NN + r.xbf_nb - 1) / r.xbf_nb) * d->K0;
    p.xi_items = ((d->NN + r.xbi_nb - 1) / r.xbi_nb) * d->K0;
  } else {
    p.xf_cols = r.xf_nb;
    p.xi_cols = r.xi_nb;
    p.xf_smem = (long long)xpass_smem(prec, (size_t)r.xf_nb * r.X);
    p.xi_smem = (long long)xpass_smem(prec, (size_t)3 * r.xi_nb * r.X);
    p.xf_items = ((d->NN + r.xf_nb - 1) / r.xf_nb) * 2 * r.KK;
    p.xi_items = ((d->NN + r.xi_nb - 1) / r.xi_nb) * d->K0;
  }
  if (p.batched_z) {
    p.z_lines = r.zb_lx;
    p.z_ctas_per_sm = zb_blocks_per_sm(d->K0, d->NN);
    p.z_smem = (long long)zb_smem(d->K0, d->NN, r.zb_lx);
    p.z_items = (r.X + r.zb_lx - 1) / r.zb_lx;
  } else {
    p.z_lines = r.z_lx;
    p.z_smem = (long long)zpass_smem(prec, d->K0, r.z_ppt, r.z_nt);
    p.z_items = ((r.X + r.z_lx - 1) / r.z_lx) * (zpass_summed(prec) ? 1 : 3);
  }
  *out = p;
  return MWF_OK;
}

int mwf_create(const mwf_run_desc* runs, int n_runs, int device, mwf_handle** out) {
  if (!runs || n_runs <= 0 || !out) return fail(MWF_ERR_ARG, "mwf_create: null argument or n_runs <= 0");
  *out = nullptr;
  mwf_handle* h = new mwf_handle();
  h->device = device;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    free_handle(h);
    return fail(MWF_ERR_CUDA, "mwf_create: no CUDA device");
  }
  if (device < 0 || device >= ndev) { free_handle(h); return fail(MWF_ERR_ARG, "mwf_create: bad device %d", device); }
  if (cudaSetDevice(device) != cudaSuccess) { free_handle(h); return fail(MWF_ERR_CUDA, "cudaSetDevice failed"); }
  h->runs.resize(n_runs);
  size_t o = 0;
  for (int i = 0; i < n_runs; ++i) {
    RunHost& r = h->runs[i];
    r.d = runs[i];
    const char* why = "";
    if (!plan_run(r, why)) { free_handle(h); return fail(MWF_ERR_SIZE, "run %d: %s", i, why); }
    if ((r.d.reflect || r.d.uvreflect || r.d.wreflect) && r.d.K0 != 4) {
      free_handle(h);
      return fail(MWF_ERR_ARG, "run %d: the reference defines the symmetry masks for K0 = 4 only", i);
    }
    if (r.d.reflect || r.d.uvreflect || r.d.wreflect) h->any_sym = true;
    if (!(r.d.dt > 0) || !(r.d.Re > 0)) { free_handle(h); return fail(MWF_ERR_ARG, "run %d: dt and Re must be > 0", i); }
    o = run_bytes(r, o);
    h->stage_elems = std::max(h->stage_elems, r.csz);
  }
  // the Euler-start flags of all runs side by side, so one memset per step clears them
  const size_t off_nst_all = o; o = align_up(o + sizeof(int) * n_runs, 256);
  for (int i = 0; i < n_runs; ++i) h->runs[i].off_nst = off_nst_all + sizeof(int) * i;
  h->off_nst_all = off_nst_all;
  const size_t off_runs = o; o = align_up(o + sizeof(RunDesc) * n_runs, 256);
  // work items
  std::vector<WorkItem> items;
  // group launches: x-forward per precision, z pass per (precision, K0, threads), x-inverse per precision
  static const int kXbSizes[] = {32, 48, 64, 96, 128, 192, 256};
  // runs whose three passes all have batched forms step in the persistent kernel
#ifndef MWF_NO_PERSIST
  for (RunHost& r : h->runs) r.persist = r.d.precision == MWF_FP32 && r.xbf_nb && r.zb_lx && r.xbi_nb;
#endif
  // launch groups of the other runs and of the runs that can step in the persistent kernel
  auto build_groups = [&](bool pset) {
  for (int prec = 0; prec < 2; ++prec) {
    // subset-split FP32 x forward: one launch per MM; an item writes u_k, v_k, w_k of one
    // wall-normal mode k and their x derivatives for a block of columns
    for (int MM : kXbSizes) {
      Launch L{0, prec, 0, 0, kXbThreads, 0, items.size(), 0};
      L.xbMM = MM;
      for (int i = 0; i < n_runs; ++i) {
        const RunHost& r = h->runs[i];
        if (r.persist != pset || r.d.precision != prec || r.d.MM != MM || !r.xbf_nb) continue;
        for (int n0 = 0; n0 < r.d.NN; n0 += r.xbf_nb)
          for (int k = 0; k < r.d.K0; ++k) items.push_back(WorkItem{i, n0, k, 0});
        L.smem = std::max(L.smem, xbf_smem(MM, r.xbf_nb));
      }
      L.nitems = (int)(items.size() - L.item_off);
      if (L.nitems) { L.persist_group = pset; h->launches.push_back(L); }
    }
    // x forward, grouped by block size
    for (int nt : {kXThreadsSmall, kXfThreads}) {
      Launch L{0, prec, 0, 0, nt, 0, items.size(), 0};
      for (int i = 0; i < n_runs; ++i) {
        const RunHost& r = h->runs[i];
        if (r.persist != pset || r.d.precision != prec || r.x_nt != nt || r.xbf_nb) continue;
        for (int n0 = 0; n0 < r.d.NN; n0 += r.xf_nb)
          for (int f = 0; f < 2 * r.KK; ++f) items.push_back(WorkItem{i, n0, f, 0});
        L.smem = std::max(L.smem, xpass_smem(prec, (size_t)r.xf_nb * r.X));
      }
      L.nitems = (int)(items.size() - L.item_off);
      if (L.nitems) { L.persist_group = pset; h->launches.push_back(L); }
    }
    // batched FP32 z pass: one launch per (model, NN)
    for (int K0 : {4, 6})
      for (int Q : {32, 48, 64, 96, 128, 192, 256}) {
        Launch L{1, prec, K0, 0, kZbThreads, 0, items.size(), 0, Q};
        for (int i = 0; i < n_runs; ++i) {
          const RunHost& r = h->runs[i];
          if (r.persist != pset || r.d.precision != prec || r.d.K0 != K0 || r.d.NN != Q || !r.zb_lx) continue;
          for (int x0 = 0; x0 < r.X; x0 += r.zb_lx) items.push_back(WorkItem{i, x0, 0, 0});
          L.smem = std::max(L.smem, zb_smem(K0, Q, r.zb_lx));
        }
        L.nitems = (int)(items.size() - L.item_off);
        if (L.nitems) { L.persist_group = pset; h->launches.push_back(L); }
      }
    for (int K0 : {4, 6})
      for (int ppt : {1, 2})
        for (int nt : {kZThreadsSmall, kZThreads}) {
        Launch L{1, prec, K0, ppt, nt, 0, items.size(), 0};
        for (int i = 0; i < n_runs; ++i) {
          const RunHost& r = h->runs[i];
          if (r.persist != pset || r.d.precision != prec || r.d.K0 != K0 || r.z_ppt != ppt || r.z_nt != nt || r.zb_lx) continue;
          // FP32: one item per line block running the three z-subsets, summed (RunDesc::z_sum),
          // so the x-inverse pass reads one partial instead of three
          for (int x0 = 0; x0 < r.X; x0 += r.z_lx) {
            if (zpass_summed(prec)) items.push_back(WorkItem{i, x0, 3, 0});
            else
              for (int sub = 0; sub < 3; ++sub) items.push_back(WorkItem{i, x0, sub, 0});
          }
          L.smem = zpass_smem(prec, K0, ppt, nt);
        }
        L.nitems = (int)(items.size() - L.item_off);
        if (L.nitems) { L.persist_group = pset; h->launches.push_back(L); }
      }
    for (int MM : kXbSizes) {
      Launch L{2, prec, 0, 0, kXbThreads, 0, items.size(), 0};
      L.xbMM = MM;
      for (int i = 0; i < n_runs; ++i) {
        const RunHost& r = h->runs[i];
        if (r.persist != pset || r.d.precision != prec || r.d.MM != MM || !r.xbi_nb) continue;
        for (int n0 = 0; n0 < r.d.NN; n0 += r.xbi_nb)
          for (int k = 0; k < r.d.K0; ++k) items.push_back(WorkItem{i, n0, k, 0});
        L.smem = std::max(L.smem, xbi_smem(MM, r.xbi_nb));
      }
      L.nitems = (int)(items.size() - L.item_off);
      if (L.nitems) { L.persist_group = pset; h->launches.push_back(L); }
    }
    for (int nt : {kXThreadsSmall, kXiThreads}) {
      Launch L{2, prec, 0, 0, nt, 0, items.size(), 0};
      for (int i = 0; i < n_runs; ++i) {
        const RunHost& r = h->runs[i];
        if (r.persist != pset || r.d.precision != prec || r.x_nt != nt || r.xbi_nb) continue;
        for (int n0 = 0; n0 < r.d.NN; n0 += r.xi_nb)
          for (int k = 0; k < r.d.K0; ++k) items.push_back(WorkItem{i, n0, k, 0});
        L.smem = std::max(L.smem, xpass_smem(prec, (size_t)3 * r.xi_nb * r.X));
      }
      L.nitems = (int)(items.size() - L.item_off);
      if (L.nitems) { L.persist_group = pset; h->launches.push_back(L); }
    }
  }
  };
  build_groups(false);
  build_groups(true);
  // the persistent step's items: a three-stage pipeline over groups of runs whose x-transformed
  // fields total at most kGroupBytes (the x forward of group p beside the z pass of group p-1 and
  // the x inverse of group p-2, each stage's lists merged in proportion), so every item's
  // prerequisites hold lower tickets
  std::vector<PersistItem> pitems;
  {
    auto size_index = [](int v) {
      for (int k = 0; k < 7; ++k)
        if (kXbSizes[k] == v) return k;
      return 255;
    };
    const size_t kGroupBytes = (size_t)40 << 20;
    std::vector<std::vector<int>> groups;
    size_t acc = 0;
    for (int i = 0; i < n_runs; ++i) {
      const RunHost& r = h->runs[i];
      if (!r.persist) continue;
      const size_t tb = (size_t)2 * r.KK * r.X * r.d.NN * 8;
      if (groups.empty() || acc + tb > kGroupBytes) {
        groups.emplace_back();
        acc = 0;
      }
      groups.back().push_back(i);
      acc += tb;
    }
    auto stage_items = [&](int g, int pass) {
      std::vector<PersistItem> v;
      for (int i : groups[g]) {
        const RunHost& r = h->runs[i];
        if (pass == 0) {
          for (int n0 = 0; n0 < r.d.NN; n0 += r.xbf_nb)
            for (int k = 0; k < r.d.K0; ++k) v.push_back(PersistItem{i, n0, k, size_index(r.d.MM)});
        } else if (pass == 1) {
          const int kind = r.d.K0 == 4 ? 1 : 2;
          for (int x0 = 0; x0 < r.X; x0 += r.zb_lx) v.push_back(PersistItem{i, x0, 0, kind << 8 | size_index(r.d.NN)});
        } else {
          for (int n0 = 0; n0 < r.d.NN; n0 += r.xbi_nb)
            for (int k = 0; k < r.d.K0; ++k) v.push_back(PersistItem{i, n0, k, 3 << 8 | size_index(r.d.MM)});
        }
      }
      return v;
    };
    const int G = (int)groups.size();
    for (int p = 0; p < G + 2; ++p) {
      std::vector<std::vector<PersistItem>> lists;
      if (p < G) lists.push_back(stage_items(p, 0));
      if (p >= 1 && p - 1 < G) lists.push_back(stage_items(p - 1, 1));
      if (p >= 2 && p - 2 < G) lists.push_back(stage_items(p - 2, 2));
      struct Key { double key; int li, j; };
      std::vector<Key> keys;
      for (int li = 0; li < (int)lists.size(); ++li)
        for (int j = 0; j < (int)lists[li].size(); ++j) keys.push_back(Key{(j + 0.5) / lists[li].size(), li, j});
      std::stable_sort(keys.begin(), keys.end(), [](const Key& x, const Key& y) { return x.key < y.key; });
      for (const Key& k : keys) pitems.push_back(lists[k.li][k.j]);
    }
    for (const PersistItem& it : pitems)
      if ((it.code & 0xff) > 6) {
        free_handle(h);
        return fail(MWF_ERR_SIZE, "persistent step: no batched kernel for run %d", it.run);
      }
    for (const RunHost& r : h->runs)
      if (r.persist)
        h->persist_smem = std::max({h->persist_smem, zb_smem(r.d.K0, r.d.NN, r.zb_lx), xbf_smem(r.d.MM, r.xbf_nb),
                                    xbi_smem(r.d.MM, r.xbi_nb)});
  }
  // launch order: all x-forward, then z, then x-inverse (independent precisions interleave)
  std::stable_sort(h->launches.begin(), h->launches.end(),
                   [](const Launch& a, const Launch& b) { return a.kind < b.kind; });
  const size_t off_items = o; o = align_up(o + sizeof(WorkItem) * items.size(), 256);
  const size_t off_pitems = o; o = align_up(o + sizeof(PersistItem) * pitems.size(), 256);
  const size_t off_counters = o; o = align_up(o + sizeof(int) * (1 + 2 * (size_t)n_runs), 256);
  size_t max_diag = 0;
  for (const RunHost& r : h->runs) max_diag = std::max(max_diag, (size_t)(r.n_diag_xf + r.n_diag_z));
  const size_t off_diag = o; o = align_up(o + sizeof(WorkItem) * max_diag, 256);
  const size_t off_err = o; o = align_up(o + 2 * sizeof(int), 256);
  const size_t off_part = o; o = align_up(o + sizeof(double) * (mwf_handle::kEnergyParts + 1), 256);
  const size_t off_stage = o; o = align_up(o + sizeof(double) * 2 * h->stage_elems, 256);
  h->arena_bytes = o;
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    free_handle(h);
    return fail(MWF_ERR_CUDA, "stream creation failed");
  }
  if (cudaMalloc(&h->arena, o) != cudaSuccess) {
    cudaGetLastError();
    h->arena = nullptr;
    free_handle(h);
    return fail(MWF_ERR_NOMEM, "cudaMalloc of %zu bytes failed", o);
  }
  h->d_runs = reinterpret_cast<RunDesc*>(h->arena + off_runs);
  h->d_items = reinterpret_cast<WorkItem*>(h->arena + off_items);
  h->d_diag_items = reinterpret_cast<WorkItem*>(h->arena + off_diag);
  h->d_err = reinterpret_cast<int*>(h->arena + off_err);
  h->d_flag = h->d_err + 1;
  h->d_partial = reinterpret_cast<double*>(h->arena + off_part);
  h->d_eout = h->d_partial + mwf_handle::kEnergyParts;
  h->d_stage = reinterpret_cast<double*>(h->arena + off_stage);
  h->d_pitems = h->arena + off_pitems;
  h->n_pitems = (int)pitems.size();
  h->d_counters = reinterpret_cast<int*>(h->arena + off_counters);
  h->counters_bytes = sizeof(int) * (1 + 2 * (size_t)n_runs);
  if (h->n_pitems) {
    h->persist_grid = persistent_grid(h->persist_smem);
    if (h->persist_grid <= 0) {
      free_handle(h);
      return fail(MWF_ERR_CUDA, "persistent step: the device holds no CTA with %zu bytes of shared memory",
                  h->persist_smem);
    }
  }
  int rc = MWF_OK;
  auto ck = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && rc == MWF_OK) rc = fail(MWF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  };
  ck(cudaMemsetAsync(h->arena, 0, o, h->stream), "arena clear");
  // The uploads below are cudaMemcpy calls on the legacy default stream, which does not wait
  // for the handle's non-blocking stream: finish the clear first, or it can land after them
  // and zero the tables of the first runs.
  ck(cudaStreamSynchronize(h->stream), "arena clear");
  std::vector<RunDesc> rds(n_runs);
  for (int i = 0; i < n_runs && rc == MWF_OK; ++i) {
    RunHost& r = h->runs[i];
    RunDesc& D = rds[i];
    memset(&D, 0, sizeof D);
    D.K0 = r.d.K0; D.MM = r.d.MM; D.NN = r.d.NN; D.M = r.M; D.X = r.X; D.Z = r.Z; D.K = r.K; D.KK = r.KK;
    D.prec = r.d.precision;
    D.xf_nb = r.xf_nb; D.xi_nb = r.xi_nb; D.z_lx = r.z_lx;
    D.z_sum = zpass_summed(r.d.precision == MWF_FP64 ? 0 : 1) ? 1 : 0;
    D.zb_lx = r.zb_lx;
    D.xbf_nb = r.xbf_nb;
    D.xbi_nb = r.xbi_nb;
    D.xbf_items = r.xbf_nb ? ((r.d.NN + r.xbf_nb - 1) / r.xbf_nb) * r.d.K0 : 0;
    D.zb_items = r.zb_lx ? (r.X + r.zb_lx - 1) / r.zb_lx : 0;
    D.alpha = r.d.alpha; D.gamma = r.d.gamma; D.dt = r.d.dt;
    D.alpha_f = (float)r.d.alpha; D.gamma_f = (float)r.d.gamma;
    D.cth = cos(r.d.theta); D.sth = sin(r.d.theta);
    D.scale = 1.0 / ((double)r.X * (double)r.Z);
    D.c = h->arena + r.off_c;
    D.onl = h->arena + r.off_onl;
    D.inv_lhs = reinterpret_cast<const double*>(h->arena + r.off_ilhs);
    D.rhs = reinterpret_cast<const double*>(h->arena + r.off_rhs);
    D.T = h->arena + r.off_T;
    D.NLT = h->arena + r.off_NLT;
    D.twX = h->arena + r.off_twX;
    D.twQ = h->arena + r.off_twQ;
    D.twZ = h->arena + r.off_twZ;
    D.nst = reinterpret_cast<int*>(h->arena + r.off_nst);
    D.active = 1;
    if (!make_plan(r.X, D.planX, r.x_radix) || !make_plan(r.d.NN, D.planQ, r.z_radix)) {
      rc = fail(MWF_ERR_SIZE, "run %d: no FFT plan", i);
      break;
    }
    std::vector<double> il, rh;
    lhsrhs(r.d, il, rh);
    if (r.d.precision == MWF_FP64) {
      ck(cudaMemcpy(h->arena + r.off_ilhs, il.data(), il.size() * 8, cudaMemcpyHostToDevice), "lhs upload");
      ck(cudaMemcpy(h->arena + r.off_rhs, rh.data(), rh.size() * 8, cudaMemcpyHostToDevice), "rhs upload");
    } else {
      // FP32 runs: c' = A c + B (3 nl - onl) with A = rhs/lhs as a float pair (hi, lo) in the
      // 1/lhs slot and B = (dt/2)/lhs in the rhs slot, all formed in FP64
      const size_t n = il.size();
      std::vector<float> a(2 * n), b(n);
      for (size_t j = 0; j < n; ++j) {
        const double A = rh[j] * il[j];
        a[j] = (float)A;
        a[n + j] = (float)(A - (double)a[j]);
        b[j] = (float)(r.d.dt / 2.0 * il[j]);
      }
      ck(cudaMemcpy(h->arena + r.off_ilhs, a.data(), a.size() * 4, cudaMemcpyHostToDevice), "table upload");
      ck(cudaMemcpy(h->arena + r.off_rhs, b.data(), b.size() * 4, cudaMemcpyHostToDevice), "table upload");
    }
    auto up = [&](size_t off, int N) {
      if (r.d.precision == MWF_FP64) {
        std::vector<double> t = twiddles<double>(N);
        ck(cudaMemcpy(h->arena + off, t.data(), t.size() * 8, cudaMemcpyHostToDevice), "twiddle upload");
      } else {
        std::vector<float> t = twiddles<float>(N);
        ck(cudaMemcpy(h->arena + off, t.data(), t.size() * 4, cudaMemcpyHostToDevice), "twiddle upload");
      }
    };
    up(r.off_twX, r.X);
    up(r.off_twQ, r.d.NN);
    up(r.off_twZ, r.Z);
    const int one = 1;
    ck(cudaMemcpy(h->arena + r.off_nst, &one, sizeof(int), cudaMemcpyHostToDevice), "nst init");
  }
  if (rc == MWF_OK) {
    ck(cudaMemcpy(h->d_runs, rds.data(), sizeof(RunDesc) * n_runs, cudaMemcpyHostToDevice), "desc upload");
    ck(cudaMemcpy(h->d_items, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice), "item upload");
    if (!pitems.empty())
      ck(cudaMemcpy(h->d_pitems, pitems.data(), sizeof(PersistItem) * pitems.size(), cudaMemcpyHostToDevice),
         "persistent item upload");
    ck(cudaDeviceSynchronize(), "create sync");
  }
  if (rc == MWF_OK) rc = build_graph(h, 1, &h->graph1);
  if (rc == MWF_OK) rc = build_graph(h, mwf_handle::kGraphSteps, &h->graphG);
  if (rc != MWF_OK) { free_handle(h); return rc; }
  *out = h;
  return MWF_OK;
}

int mwf_destroy(mwf_handle* h) {
  if (!h) return fail(MWF_ERR_ARG, "mwf_destroy: null handle");
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  free_handle(h);
  return MWF_OK;
}

static int check_run(mwf_handle* h, int run) {
  if (!h) return fail(MWF_ERR_ARG, "null handle");
  if (run < 0 || run >= (int)h->runs.size()) return fail(MWF_ERR_ARG, "run index %d out of range", run);
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(MWF_ERR_CUDA, "cudaSetDevice failed");
  return MWF_OK;
}

int mwf_set_state(mwf_handle* h, int run, const double* re, const double* im) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!re || !im) return fail(MWF_ERR_ARG, "mwf_set_state: null state array");
  const RunHost& r = h->runs[run];
  double* sre = h->d_stage;
  double* sim = h->d_stage + h->stage_elems;
  CK(cudaMemcpyAsync(sre, re, r.csz * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(sim, im, r.csz * 8, cudaMemcpyHostToDevice, h->stream));
  cudaError_t e = r.d.precision == MWF_FP64
                      ? launch_ref_to_dev_f64(sre, sim, h->arena + r.off_c, r.K, r.M, r.d.NN, h->stream)
                      : launch_ref_to_dev_f32(sre, sim, h->arena + r.off_c, r.K, r.M, r.d.NN, h->stream);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "state conversion: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(h->stream));
  return MWF_OK;
}

int mwf_get_state(mwf_handle* h, int run, double* re, double* im) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!re || !im) return fail(MWF_ERR_ARG, "mwf_get_state: null state array");
  const RunHost& r = h->runs[run];
  double* sre = h->d_stage;
  double* sim = h->d_stage + h->stage_elems;
  cudaError_t e = r.d.precision == MWF_FP64
                      ? launch_dev_to_ref_f64(h->arena + r.off_c, sre, sim, r.K, r.M, r.d.NN, h->stream)
                      : launch_dev_to_ref_f32(h->arena + r.off_c, sre, sim, r.K, r.M, r.d.NN, h->stream);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "state conversion: %s", cudaGetErrorString(e));
  CK(cudaMemcpyAsync(re, sre, r.csz * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(im, sim, r.csz * 8, cudaMemcpyDeviceToHost, h->stream));
  return check_device_err(h);
}

int mwf_get_history(mwf_handle* h, int run, double* re, double* im, int* euler_next) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!re || !im || !euler_next) return fail(MWF_ERR_ARG, "mwf_get_history: null argument");
  const RunHost& r = h->runs[run];
  double* sre = h->d_stage;
  double* sim = h->d_stage + h->stage_elems;
  cudaError_t e = r.d.precision == MWF_FP64
                      ? launch_dev_to_ref_f64(h->arena + r.off_onl, sre, sim, r.K, r.M, r.d.NN, h->stream)
                      : launch_dev_to_ref_f32(h->arena + r.off_onl, sre, sim, r.K, r.M, r.d.NN, h->stream);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "history conversion: %s", cudaGetErrorString(e));
  CK(cudaMemcpyAsync(re, sre, r.csz * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(im, sim, r.csz * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(euler_next, h->arena + r.off_nst, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  return check_device_err(h);
}

int mwf_set_history(mwf_handle* h, int run, const double* re, const double* im, int euler_next) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!re || !im) return fail(MWF_ERR_ARG, "mwf_set_history: null argument");
  const RunHost& r = h->runs[run];
  double* sre = h->d_stage;
  double* sim = h->d_stage + h->stage_elems;
  CK(cudaMemcpyAsync(sre, re, r.csz * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(sim, im, r.csz * 8, cudaMemcpyHostToDevice, h->stream));
  cudaError_t e = r.d.precision == MWF_FP64
                      ? launch_ref_to_dev_f64(sre, sim, h->arena + r.off_onl, r.K, r.M, r.d.NN, h->stream)
                      : launch_ref_to_dev_f32(sre, sim, h->arena + r.off_onl, r.K, r.M, r.d.NN, h->stream);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "history conversion: %s", cudaGetErrorString(e));
  const int v = euler_next ? 1 : 0;
  CK(cudaMemcpyAsync(h->arena + r.off_nst, &v, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return MWF_OK;
}

int mwf_query(mwf_handle* h, int* idle) {
  if (!h || !idle) return fail(MWF_ERR_ARG, "mwf_query: null argument");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(MWF_ERR_CUDA, "cudaSetDevice failed");
  const cudaError_t e = cudaStreamQuery(h->stream);
  if (e == cudaErrorNotReady) {
    *idle = 0;
    return MWF_OK;
  }
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "mwf_query: %s", cudaGetErrorString(e));
  *idle = 1;
  return MWF_OK;
}

int mwf_step_async(mwf_handle* h, int nsteps) {
  if (!h) return fail(MWF_ERR_ARG, "null handle");
  if (nsteps < 0) return fail(MWF_ERR_ARG, "nsteps < 0");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(MWF_ERR_CUDA, "cudaSetDevice failed");
  int s = nsteps;
  while (s >= mwf_handle::kGraphSteps) {
    CK(cudaGraphLaunch(h->graphG, h->stream));
    s -= mwf_handle::kGraphSteps;
  }
  while (s-- > 0) CK(cudaGraphLaunch(h->graph1, h->stream));
  return MWF_OK;
}

int mwf_synchronize(mwf_handle* h) {
  if (!h) return fail(MWF_ERR_ARG, "null handle");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(MWF_ERR_CUDA, "cudaSetDevice failed");
  return check_device_err(h);
}

int mwf_step(mwf_handle* h, int nsteps) {
  int rc = mwf_step_async(h, nsteps);
  if (rc) return rc;
  return mwf_synchronize(h);
}

int mwf_reset_history(mwf_handle* h, int run) {
  int rc = check_run(h, run);
  if (rc) return rc;
  const int one = 1;
  CK(cudaMemcpyAsync(h->arena + h->runs[run].off_nst, &one, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return MWF_OK;
}

int mwf_phys_diagnostics(mwf_handle* h, int run, double threshold, double* count_above, double* energy) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!count_above || !energy) return fail(MWF_ERR_ARG, "mwf_phys_diagnostics: null output");
  const RunHost& r = h->runs[run];
  if (!r.active) return fail(MWF_ERR_ARG, "run %d is not active", run);
  const int prec = r.d.precision;
  std::vector<WorkItem> items;
  items.reserve(r.n_diag_xf + r.n_diag_z);
  for (int n0 = 0; n0 < r.d.NN; n0 += r.xf_nb)
    for (int f = 0; f < r.KK; ++f) items.push_back(WorkItem{run, n0, f, 1});
  for (int x0 = 0; x0 < r.X; x0 += r.z_lx)
    for (int sub = 0; sub < 3; ++sub) items.push_back(WorkItem{run, x0, sub, 0});
  if ((int)items.size() != r.n_diag_xf + r.n_diag_z) return fail(MWF_ERR_DEVICE, "diagnostic item count mismatch");
  cudaStream_t st = h->stream;
  CK(cudaMemcpyAsync(h->d_diag_items, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice, st));
  RunDesc* d = h->d_runs + run;
  CK(cudaMemcpyAsync(reinterpret_cast<unsigned char*>(d) + offsetof(RunDesc, diag_ct), &threshold, sizeof(double),
                     cudaMemcpyHostToDevice, st));
  const size_t xfs = xpass_smem(prec, (size_t)r.xf_nb * r.X);
  const size_t zsm = zpass_smem(prec, r.d.K0, r.z_ppt, r.z_nt);
  cudaError_t e = prec == MWF_FP64 ? launch_x_forward_f64(r.x_nt, h->d_runs, h->d_diag_items, r.n_diag_xf, xfs, h->d_err, st)
                                   : launch_x_forward_f32(r.x_nt, h->d_runs, h->d_diag_items, r.n_diag_xf, xfs, h->d_err, st);
  if (e == cudaSuccess)
    e = prec == MWF_FP64
            ? launch_z_diag_f64(r.d.K0, r.z_ppt, r.z_nt, h->d_runs, h->d_diag_items + r.n_diag_xf, r.n_diag_z, zsm, h->d_err, st)
            : launch_z_diag_f32(r.d.K0, r.z_ppt, r.z_nt, h->d_runs, h->d_diag_items + r.n_diag_xf, r.n_diag_z, zsm, h->d_err, st);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "diagnostic launch: %s", cudaGetErrorString(e));
  std::vector<double> part(2 * (size_t)r.n_diag_z);
  CK(cudaMemcpyAsync(part.data(), h->arena + r.off_NLT, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, st));
  rc = check_device_err(h);
  if (rc) return rc;
  double cnt = 0.0, sum = 0.0, comp = 0.0;
  for (int i = 0; i < r.n_diag_z; ++i) {
    cnt += part[2 * i];
    const double t = part[2 * i + 1];
    const double y = sum + t;
    comp += (fabs(sum) >= fabs(t)) ? (sum - y) + t : (t - y) + sum;
    sum = y;
  }
  *count_above = cnt;
  *energy = (sum + comp) / ((double)r.X * (double)r.Z);
  return MWF_OK;
}

int mwf_set_active(mwf_handle* h, int run, int active) {
  int rc = check_run(h, run);
  if (rc) return rc;
  const int v = active ? 1 : 0;
  h->runs[run].active = v;
  RunDesc* d = h->d_runs + run;
  CK(cudaMemcpyAsync(reinterpret_cast<unsigned char*>(d) + offsetof(RunDesc, active), &v, sizeof(int),
                     cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return MWF_OK;
}

int mwf_test_copy_timeout(mwf_handle* h, int run, unsigned extra_bytes, double wait_ms) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!(wait_ms >= 0.0) || wait_ms > 1000.0 || extra_bytes % 16 || extra_bytes > (1u << 20))
    return fail(MWF_ERR_ARG, "mwf_test_copy_timeout: wait_ms must be in [0, 1000] and extra_bytes a multiple "
                             "of 16 up to 1 MiB");
  const unsigned long long ns = (unsigned long long)(wait_ms * 1e6);
  RunDesc* d = h->d_runs + run;
  CK(cudaMemcpyAsync(reinterpret_cast<unsigned char*>(d) + offsetof(RunDesc, test_tx_extra), &extra_bytes,
                     sizeof(unsigned), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(reinterpret_cast<unsigned char*>(d) + offsetof(RunDesc, test_wait_ns), &ns,
                     sizeof(unsigned long long), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return MWF_OK;
}

int mwf_energy(mwf_handle* h, int run, double* e) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!e) return fail(MWF_ERR_ARG, "mwf_energy: null output");
  const RunHost& r = h->runs[run];
  CK(cudaMemsetAsync(h->d_flag, 0, sizeof(int), h->stream));
  cudaError_t ce = r.d.precision == MWF_FP64 ? launch_nonfinite_f64(h->d_runs, run, h->d_flag, h->stream)
                                             : launch_nonfinite_f32(h->d_runs, run, h->d_flag, h->stream);
  if (ce != cudaSuccess) return fail(MWF_ERR_CUDA, "non-finite check: %s", cudaGetErrorString(ce));
  ce = r.d.precision == MWF_FP64
           ? launch_energy_f64(h->d_runs, run, h->d_partial, mwf_handle::kEnergyParts, h->d_eout, h->stream)
           : launch_energy_f32(h->d_runs, run, h->d_partial, mwf_handle::kEnergyParts, h->d_eout, h->stream);
  if (ce != cudaSuccess) return fail(MWF_ERR_CUDA, "energy launch: %s", cudaGetErrorString(ce));
  int flag = 0;
  CK(cudaMemcpyAsync(e, h->d_eout, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(&flag, h->d_flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  rc = check_device_err(h);
  if (rc) return rc;
  if (flag) return fail(MWF_ERR_NONFINITE, "run %d: state contains NaN/Inf", run);
  return MWF_OK;
}

// ---- state operations and diagnostics outside the timestep ----

int mwf_get_phys(mwf_handle* h, int run, double* p) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!p) return fail(MWF_ERR_ARG, "mwf_get_phys: null output");
  const RunHost& r = h->runs[run];
  if (!r.active) return fail(MWF_ERR_ARG, "run %d is not active", run);
  const int prec = r.d.precision;
  FftPlanDev pz{};
  if (!make_plan(r.Z, pz, prec == MWF_FP64 ? 12 : 16) || r.Z > kPhysVpt * kPhysThreads)
    return fail(MWF_ERR_SIZE, "no z plan for Z = %d", r.Z);
  std::vector<WorkItem> items;
  items.reserve(r.n_diag_xf);
  for (int n0 = 0; n0 < r.d.NN; n0 += r.xf_nb)
    for (int f = 0; f < r.KK; ++f) items.push_back(WorkItem{run, n0, f, 1});
  cudaStream_t st = h->stream;
  CK(cudaMemcpyAsync(h->d_diag_items, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice, st));
  const size_t xfs = xpass_smem(prec, (size_t)r.xf_nb * r.X);
  const size_t zs = xpass_smem(prec, (size_t)r.Z);
  double* out = reinterpret_cast<double*>(h->arena + r.off_NLT);   // KK*X*Z doubles fit the NLT scratch
  cudaError_t e = prec == MWF_FP64 ? launch_x_forward_f64(r.x_nt, h->d_runs, h->d_diag_items, (int)items.size(), xfs, h->d_err, st)
                                   : launch_x_forward_f32(r.x_nt, h->d_runs, h->d_diag_items, (int)items.size(), xfs, h->d_err, st);
  if (e == cudaSuccess)
    e = prec == MWF_FP64 ? launch_phys_z_f64(h->d_runs, run, r.X, r.KK, pz, zs, out, h->d_err, st)
                         : launch_phys_z_f32(h->d_runs, run, r.X, r.KK, pz, zs, out, h->d_err, st);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "physical-field launch: %s", cudaGetErrorString(e));
  CK(cudaMemcpyAsync(p, out, sizeof(double) * (size_t)r.KK * r.X * r.Z, cudaMemcpyDeviceToHost, st));
  return check_device_err(h);
}

int mwf_spectrum_maxima(mwf_handle* h, int run, double* m_max, double* n_max) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!m_max || !n_max) return fail(MWF_ERR_ARG, "mwf_spectrum_maxima: null output");
  const RunHost& r = h->runs[run];
  const int MM = r.d.MM, NN = r.d.NN;
  unsigned long long* mx = reinterpret_cast<unsigned long long*>(h->arena + r.off_NLT);
  cudaStream_t st = h->stream;
  CK(cudaMemsetAsync(mx, 0, sizeof(unsigned long long) * (MM + NN), st));
  cudaError_t e = r.d.precision == MWF_FP64 ? launch_spectrum_f64(h->d_runs, run, r.M, NN, mx, st)
                                            : launch_spectrum_f32(h->d_runs, run, r.M, NN, mx, st);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "spectrum launch: %s", cudaGetErrorString(e));
  std::vector<double> v(MM + NN);
  CK(cudaMemcpyAsync(v.data(), mx, sizeof(double) * v.size(), cudaMemcpyDeviceToHost, st));
  rc = check_device_err(h);
  if (rc) return rc;
  std::copy(v.begin(), v.begin() + MM, m_max);
  std::copy(v.begin() + MM, v.end(), n_max);
  return MWF_OK;
}

int mwf_history(mwf_handle* h, int run, double y, int n_probes, double* H) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!H) return fail(MWF_ERR_ARG, "mwf_history: null output");
  const RunHost& r = h->runs[run];
  if (n_probes < 1 || n_probes >= r.Z) return fail(MWF_ERR_ARG, "n_probes must be in [1, Z-1]");
  const int KK = r.KK, NN = r.d.NN, K0 = r.d.K0;
  std::vector<int> zs(n_probes);
  for (int j = 0; j < n_probes; ++j) zs[j] = (int)((long long)j * r.Z / n_probes) + 1;
  unsigned char* base = h->arena + r.off_NLT;
  double2* g = reinterpret_cast<double2*>(base);
  int* dz = reinterpret_cast<int*>(base + align_up(sizeof(double2) * (size_t)KK * NN, 256));
  double* dout = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(dz) + align_up(sizeof(int) * (size_t)n_probes, 256));
  cudaStream_t st = h->stream;
  CK(cudaMemcpyAsync(dz, zs.data(), sizeof(int) * zs.size(), cudaMemcpyHostToDevice, st));
  cudaError_t e = r.d.precision == MWF_FP64 ? launch_probes_f64(h->d_runs, run, K0, NN, g, dz, n_probes, dout, st)
                                            : launch_probes_f32(h->d_runs, run, K0, NN, g, dz, n_probes, dout, st);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "probe launch: %s", cudaGetErrorString(e));
  std::vector<double> V((size_t)n_probes * KK);
  CK(cudaMemcpyAsync(V.data(), dout, sizeof(double) * V.size(), cudaMemcpyDeviceToHost, st));
  rc = check_device_err(h);
  if (rc) return rc;
  // velU / velV / velW (modes.M4.f90:83-107, modes.M6.f90:81-111): u_k and w_k on 1,
  // sin(k beta y) (k odd), cos(k beta y) (k even); v_k on cos (k odd), sin (k even).
  const double beta = 0.5 * M_PI;
  std::vector<double> bu(K0), bv(K0);
  bu[0] = 1.0;
  for (int k = 1; k < K0; ++k) {
    bu[k] = (k & 1) ? std::sin(k * beta * y) : std::cos(k * beta * y);
    bv[k] = (k & 1) ? std::cos(k * beta * y) : std::sin(k * beta * y);
  }
  const double Lz = 2.0 * M_PI / r.d.gamma;
  for (int j = 0; j < n_probes; ++j) {
    const double* v = V.data() + (size_t)j * KK;
    double U = 0.0, Vv = 0.0, W = 0.0;
    for (int k = 0; k < K0; ++k) U += bu[k] * v[k];
    for (int k = 1; k < K0; ++k) Vv += bv[k] * v[K0 + k - 1];
    for (int k = 0; k < K0; ++k) W += bu[k] * v[2 * K0 - 1 + k];
    H[4 * j + 0] = zs[j] * Lz / r.Z;
    H[4 * j + 1] = U;
    H[4 * j + 2] = Vv;
    H[4 * j + 3] = W;
  }
  return MWF_OK;
}

static int set_nst(mwf_handle* h, const RunHost& r) {
  const int one = 1;
  CK(cudaMemcpyAsync(h->arena + r.off_nst, &one, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  return MWF_OK;
}

int mwf_remap_x(mwf_handle* h, int run, int factor) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (factor < 1) return fail(MWF_ERR_ARG, "mwf_remap_x: factor must be >= 1");
  const RunHost& r = h->runs[run];
  const size_t cb = r.d.precision == MWF_FP64 ? 16 : 8;
  void* src = h->arena + r.off_T;          // the old state, in the transform scratch
  CK(cudaMemcpyAsync(src, h->arena + r.off_c, r.csz * cb, cudaMemcpyDeviceToDevice, h->stream));
  cudaError_t e = r.d.precision == MWF_FP64 ? launch_remap_x_f64(h->d_runs, run, src, r.csz, factor, h->stream)
                                            : launch_remap_x_f32(h->d_runs, run, src, r.csz, factor, h->stream);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "remap launch: %s", cudaGetErrorString(e));
  rc = set_nst(h, r);
  if (rc) return rc;
  return check_device_err(h);
}

int mwf_blend_state(mwf_handle* h, int run, int other, double d) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (other < 0 || other >= (int)h->runs.size()) return fail(MWF_ERR_ARG, "run index %d out of range", other);
  const RunHost& r = h->runs[run];
  const RunHost& o = h->runs[other];
  if (r.d.K0 != o.d.K0 || r.d.MM != o.d.MM || r.d.NN != o.d.NN || r.d.precision != o.d.precision)
    return fail(MWF_ERR_ARG, "mwf_blend_state: runs %d and %d differ in model, size or precision", run, other);
  if (!std::isfinite(d)) return fail(MWF_ERR_ARG, "mwf_blend_state: weight is not finite");
  cudaError_t e = r.d.precision == MWF_FP64 ? launch_blend_f64(h->d_runs, run, other, r.csz, d, h->stream)
                                            : launch_blend_f32(h->d_runs, run, other, r.csz, d, h->stream);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "blend launch: %s", cudaGetErrorString(e));
  rc = set_nst(h, r);
  if (rc) return rc;
  return check_device_err(h);
}

int mwf_add_noise(mwf_handle* h, int run, double scale, unsigned long long seed) {
  int rc = check_run(h, run);
  if (rc) return rc;
  if (!std::isfinite(scale)) return fail(MWF_ERR_ARG, "mwf_add_noise: scale is not finite");
  const RunHost& r = h->runs[run];
  cudaError_t e = r.d.precision == MWF_FP64 ? launch_noise_f64(h->d_runs, run, r.csz, scale, seed, h->stream)
                                            : launch_noise_f32(h->d_runs, run, r.csz, scale, seed, h->stream);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "noise launch: %s", cudaGetErrorString(e));
  return check_device_err(h);
}

// CUDA events (and a device buffer) released when the scope ends, on every return path of
// the timing helpers below, whose CK checks return early.
struct EventSet {
  std::vector<cudaEvent_t> ev;
  explicit EventSet(size_t n) : ev(n, nullptr) {}
  ~EventSet() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
  cudaError_t create() {
    for (cudaEvent_t& e : ev) {
      const cudaError_t r = cudaEventCreate(&e);
      if (r != cudaSuccess) return r;
    }
    return cudaSuccess;
  }
  cudaEvent_t operator[](size_t i) const { return ev[i]; }
};
struct DeviceBuffer {
  void* p = nullptr;
  ~DeviceBuffer() {
    if (p) cudaFree(p);
  }
};

int mwf_step_timed(mwf_handle* h, int nsteps, double* ms) {
  if (!h || !ms) return fail(MWF_ERR_ARG, "mwf_step_timed: null argument");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(MWF_ERR_CUDA, "cudaSetDevice failed");
  EventSet ev(2);
  CK(ev.create());
  CK(cudaEventRecord(ev[0], h->stream));
  int rc = mwf_step_async(h, nsteps);
  if (rc == MWF_OK) {
    CK(cudaEventRecord(ev[1], h->stream));
    CK(cudaEventSynchronize(ev[1]));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, ev[0], ev[1]));
    *ms = f;
    rc = check_device_err(h);
  }
  return rc;
}

int mwf_profile_passes(mwf_handle* h, int nreps, double* ms_per_pass) {
  if (!h || !ms_per_pass || nreps <= 0) return fail(MWF_ERR_ARG, "mwf_profile_passes: bad argument");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(MWF_ERR_CUDA, "cudaSetDevice failed");
  const size_t nl = h->launches.size();
  EventSet ev(2 * nl * nreps);
  CK(ev.create());
  // the passes of one step, launched individually (the same launches the graph holds)
  int rc = MWF_OK;
  for (int rep = 0; rep < nreps && rc == MWF_OK; ++rep) {
    for (size_t i = 0; i < nl && rc == MWF_OK; ++i) {
      const Launch& L = h->launches[i];
      cudaStream_t st = h->stream;
      CK(cudaEventRecord(ev[2 * (rep * nl + i)], st));
      cudaError_t e = launch_pass(L, h->d_runs, h->d_items + L.item_off, h->d_err, st);
      if (e != cudaSuccess) rc = fail(MWF_ERR_CUDA, "profile launch: %s", cudaGetErrorString(e));
      CK(cudaEventRecord(ev[2 * (rep * nl + i) + 1], st));
    }
    CK(cudaMemsetAsync(h->arena + h->off_nst_all, 0, sizeof(int) * h->runs.size(), h->stream));
  }
  if (rc == MWF_OK) {
    CK(cudaStreamSynchronize(h->stream));
    double acc[3] = {0, 0, 0};
    for (int rep = 0; rep < nreps; ++rep)
      for (size_t i = 0; i < nl; ++i) {
        float f = 0.f;
        CK(cudaEventElapsedTime(&f, ev[2 * (rep * nl + i)], ev[2 * (rep * nl + i) + 1]));
        acc[h->launches[i].kind] += f;
      }
    for (int k = 0; k < 3; ++k) ms_per_pass[k] = acc[k] / nreps;
    rc = check_device_err(h);
  }
  return rc;
}

}  // extern "C"

namespace {

// Device memory of one stand-alone transform call (mwf_spec2phys / mwf_phys2spec), released on
// every return path: descriptor, error word, twiddles of X and Z, the spectral fields in the
// device layout, the x-transformed fields, the physical fields and the staging of the split
// Re/Im arrays, in one allocation.
struct TransformCall {
  unsigned char* mem = nullptr;
  RunHost r;
  RunDesc* d = nullptr;
  int* err = nullptr;
  double2* sp = nullptr;
  double* ph = nullptr;
  double* s_re = nullptr;
  double* s_im = nullptr;
  FftPlanDev pz{};
  size_t nspec = 0, nphys = 0;
  ~TransformCall() {
    if (mem) cudaFree(mem);
  }
};

int transform_setup(const mwf_run_desc* desc, const char* who, TransformCall& tc) {
  if (!desc) return fail(MWF_ERR_ARG, "%s: null argument", who);
  tc.r.d = *desc;
  tc.r.d.precision = MWF_FP64;
  tc.r.d.xf_cols = tc.r.d.xi_cols = tc.r.d.z_lines = tc.r.d.x_radix = tc.r.d.z_radix = 0;
  const char* why = "";
  if (!plan_run(tc.r, why)) return fail(MWF_ERR_SIZE, "%s: %s", who, why);
  RunHost& r = tc.r;
  if (r.Z > kPhysVpt * kPhysThreads) return fail(MWF_ERR_SIZE, "%s: 3NN = %d exceeds %d", who, r.Z, kPhysVpt * kPhysThreads);
  RunDesc D;
  memset(&D, 0, sizeof D);
  if (!make_plan(r.Z, tc.pz, 12) || !make_plan(r.X, D.planX, 12)) return fail(MWF_ERR_SIZE, "%s: no FFT plan", who);
  tc.nspec = (size_t)r.KK * r.M * r.d.NN;
  tc.nphys = (size_t)r.KK * r.Z * r.X;
  size_t o = 0;
  const size_t off_d = o; o = align_up(o + sizeof(RunDesc), 256);
  const size_t off_err = o; o = align_up(o + sizeof(int), 256);
  const size_t off_twX = o; o = align_up(o + 16 * (size_t)r.X, 256);
  const size_t off_twZ = o; o = align_up(o + 16 * (size_t)r.Z, 256);
  const size_t off_sp = o; o = align_up(o + 16 * tc.nspec, 256);
  const size_t off_W = o; o = align_up(o + 16 * (size_t)r.KK * r.X * r.d.NN, 256);
  const size_t off_ph = o; o = align_up(o + 8 * tc.nphys, 256);
  const size_t off_re = o; o = align_up(o + 8 * tc.nspec, 256);
  const size_t off_im = o; o = align_up(o + 8 * tc.nspec, 256);
  if (cudaMalloc(&tc.mem, o) != cudaSuccess) {
    cudaGetLastError();
    tc.mem = nullptr;
    return fail(MWF_ERR_NOMEM, "%s: cudaMalloc of %zu bytes failed", who, o);
  }
  tc.d = reinterpret_cast<RunDesc*>(tc.mem + off_d);
  tc.err = reinterpret_cast<int*>(tc.mem + off_err);
  tc.sp = reinterpret_cast<double2*>(tc.mem + off_sp);
  tc.ph = reinterpret_cast<double*>(tc.mem + off_ph);
  tc.s_re = reinterpret_cast<double*>(tc.mem + off_re);
  tc.s_im = reinterpret_cast<double*>(tc.mem + off_im);
  D.K0 = r.d.K0; D.MM = r.d.MM; D.NN = r.d.NN; D.M = r.M; D.X = r.X; D.Z = r.Z; D.K = r.K; D.KK = r.KK;
  D.prec = 0;
  D.alpha = r.d.alpha; D.gamma = r.d.gamma; D.dt = r.d.dt;
  D.scale = 1.0 / ((double)r.X * (double)r.Z);
  D.T = tc.mem + off_W;
  D.twX = tc.mem + off_twX;
  D.twZ = tc.mem + off_twZ;
  D.active = 1;
  const std::vector<double> twx = twiddles<double>(r.X), twz = twiddles<double>(r.Z);
  CK(cudaMemcpy(tc.d, &D, sizeof D, cudaMemcpyHostToDevice));
  CK(cudaMemset(tc.err, 0, sizeof(int)));
  CK(cudaMemcpy(tc.mem + off_twX, twx.data(), twx.size() * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(tc.mem + off_twZ, twz.data(), twz.size() * 8, cudaMemcpyHostToDevice));
  return MWF_OK;
}

int transform_finish(TransformCall& tc, const char* who) {
  int herr = 0;
  CK(cudaMemcpy(&herr, tc.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) return fail(MWF_ERR_DEVICE, "%s: kernel reported internal error flags 0x%x", who, herr);
  return MWF_OK;
}

}  // namespace

extern "C" {

int mwf_spec2phys(const mwf_run_desc* d, const double* s_re, const double* s_im, double* p) {
  if (!s_re || !s_im || !p) return fail(MWF_ERR_ARG, "mwf_spec2phys: null argument");
  TransformCall tc;
  int rc = transform_setup(d, "mwf_spec2phys", tc);
  if (rc) return rc;
  const RunHost& r = tc.r;
  CK(cudaMemcpy(tc.s_re, s_re, 8 * tc.nspec, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(tc.s_im, s_im, 8 * tc.nspec, cudaMemcpyHostToDevice));
  cudaError_t e = launch_ref_to_dev_f64(tc.s_re, tc.s_im, tc.sp, r.KK, r.M, r.d.NN, 0);
  if (e == cudaSuccess) e = launch_spec_x_backward_f64(tc.d, 0, r.X, r.KK, r.d.NN, tc.sp, tc.err, 0);
  if (e == cudaSuccess) e = launch_phys_z_f64(tc.d, 0, r.X, r.KK, tc.pz, xpass_smem(0, (size_t)r.Z), tc.ph, tc.err, 0);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "mwf_spec2phys: launch: %s", cudaGetErrorString(e));
  rc = transform_finish(tc, "mwf_spec2phys");
  if (rc) return rc;
  CK(cudaMemcpy(p, tc.ph, 8 * tc.nphys, cudaMemcpyDeviceToHost));
  return MWF_OK;
}

int mwf_phys2spec(const mwf_run_desc* d, const double* p, double* s_re, double* s_im) {
  if (!s_re || !s_im || !p) return fail(MWF_ERR_ARG, "mwf_phys2spec: null argument");
  TransformCall tc;
  int rc = transform_setup(d, "mwf_phys2spec", tc);
  if (rc) return rc;
  const RunHost& r = tc.r;
  CK(cudaMemcpy(tc.ph, p, 8 * tc.nphys, cudaMemcpyHostToDevice));
  cudaError_t e = launch_phys_z_forward_f64(tc.d, 0, r.X, r.KK, r.Z, tc.pz, tc.ph, tc.err, 0);
  if (e == cudaSuccess) e = launch_spec_x_forward_f64(tc.d, 0, r.X, r.KK, r.d.NN, tc.sp, tc.err, 0);
  if (e == cudaSuccess) e = launch_dev_to_ref_f64(tc.sp, tc.s_re, tc.s_im, r.KK, r.M, r.d.NN, 0);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "mwf_phys2spec: launch: %s", cudaGetErrorString(e));
  rc = transform_finish(tc, "mwf_phys2spec");
  if (rc) return rc;
  CK(cudaMemcpy(s_re, tc.s_re, 8 * tc.nspec, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(s_im, tc.s_im, 8 * tc.nspec, cudaMemcpyDeviceToHost));
  return MWF_OK;
}

int mwf_set_persistent(mwf_handle* h, int on) {
  if (!h) return fail(MWF_ERR_ARG, "mwf_set_persistent: null handle");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(MWF_ERR_CUDA, "cudaSetDevice failed");
  const bool want = on != 0;
  if (want == h->persist_mode) return MWF_OK;
  CK(cudaStreamSynchronize(h->stream));
  h->persist_mode = want;
  cudaGraphExec_t g1 = nullptr, gG = nullptr;
  int rc = build_graph(h, 1, &g1);
  if (rc == MWF_OK) rc = build_graph(h, mwf_handle::kGraphSteps, &gG);
  if (rc != MWF_OK) {
    if (g1) cudaGraphExecDestroy(g1);
    h->persist_mode = !want;
    return rc;
  }
  cudaGraphExecDestroy(h->graph1);
  cudaGraphExecDestroy(h->graphG);
  h->graph1 = g1;
  h->graphG = gG;
  return MWF_OK;
}

int mwf_kernels_per_step(mwf_handle* h, int* n) {
  if (!h || !n) return fail(MWF_ERR_ARG, "mwf_kernels_per_step: null argument");
  const bool persist = h->persist_mode && h->n_pitems;
  int k = persist ? 1 : 0;
  for (const Launch& L : h->launches) k += (persist && L.persist_group) ? 0 : 1;
  for (const RunHost& r : h->runs) k += (r.d.reflect ? 1 : 0) + (r.d.uvreflect ? 1 : 0) + (r.d.wreflect ? 1 : 0);
  *n = k;
  return MWF_OK;
}

int mwf_measure_fma_peak(int device, int which, double* tflops) {
  if (!tflops || (which != 0 && which != 1)) return fail(MWF_ERR_ARG, "mwf_measure_fma_peak: bad argument");
  CK(cudaSetDevice(device));
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  DeviceBuffer out;
  const int blocks = sms * 8, threads = 256;
  CK(cudaMalloc(&out.p, (size_t)blocks * threads * 8));
  EventSet ev(2);
  CK(ev.create());
  const int iters = which == 0 ? 4096 : 65536;
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    CK(cudaEventRecord(ev[0], 0));
    cudaError_t e = launch_fma_probe(which, blocks, threads, iters, out.p, 0);
    if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "fma probe: %s", cudaGetErrorString(e));
    CK(cudaEventRecord(ev[1], 0));
    CK(cudaEventSynchronize(ev[1]));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, ev[0], ev[1]));
    const double flops = 2.0 * kFmaChains * (double)iters * blocks * threads;
    if (rep > 0) best = std::max(best, flops / (f * 1e-3) / 1e12);
  }
  *tflops = best;
  return MWF_OK;
}

int mwf_host_alloc(size_t bytes, void** p) {
  if (!p) return fail(MWF_ERR_ARG, "mwf_host_alloc: null output");
  CK(cudaHostAlloc(p, bytes, cudaHostAllocDefault));
  return MWF_OK;
}

int mwf_host_free(void* p) {
  if (p) CK(cudaFreeHost(p));
  return MWF_OK;
}

int mwf_last_error(char* buf, size_t len) {
  if (buf && len) {
    strncpy(buf, g_err, len - 1);
    buf[len - 1] = 0;
  }
  return (int)strlen(g_err);
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Time step for callers that cannot allocate device memory.
//
// Some callers of this library run where cudaMalloc is not theirs to call: a Fortran or
// C host code that owns every device buffer itself (CUDA Fortran or OpenACC device
// arrays, a memory pool it manages), or one that is not allowed to grow its device
// footprint after start-up.  mwf_step_noalloc advances a state that such a caller keeps
// in its own device arrays, with every intermediate array (device-layout state, FP64
// tables, twiddles, transposes) in the fixed file-scope array below instead of in memory
// the library allocates.  Every GPU that loads this module holds the array until the
// process exits; runs whose intermediates do not fit it are rejected.
// ---------------------------------------------------------------------------------------
#define MWF_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[MWF_NOALLOC_SCRATCH_BYTES];

namespace {

// var_LHSRHS (variables.f90:565-597) for one run, in the device layout [n][slot][m], with
// the reference's loop-order result per slot (slot < K0: psi_slot, else phi_{slot-K0+1})
// and the same FP64 operation order as the host tables (no contraction).  The stored form
// is the one the run's x-inverse pass reads, as mwf_create builds it: FP64 runs get 1/lhs
// and rhs as doubles; FP32 runs get A = rhs/lhs as a float pair (hi at ilhs[0..n), lo at
// ilhs[n..2n) as floats) and B = (dt/2)/lhs as floats in the rhs slot, formed in FP64.
__global__ void noalloc_tables_kernel(const RunDesc* rd, double Re, double drag, double vdrag, double hypo,
                                      int dragall, double* ilhs, double* rhs) {
  const int K0 = rd->K0, K = rd->K, M = rd->M, MM = rd->MM, NN = rd->NN;
  const double alpha = rd->alpha, gamma = rd->gamma, dt = rd->dt;
  const double beta = 3.1415926535897931 / 2.0;
  const size_t tot = (size_t)K * M * NN;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int ms = (int)(e % M);
    const int slot = (int)((e / M) % K);
    const int n = (int)(e / ((size_t)M * K));
    const int ma = ms < MM ? ms : M - ms;
    const double m2 = __dmul_rn(__dmul_rn(__dmul_rn(-alpha, (double)ma), alpha), (double)ma);
    const double n2 = __dmul_rn(__dmul_rn(__dmul_rn(-gamma, (double)n), gamma), (double)n);
    const bool psi = slot < K0;
    const int k = psi ? slot : slot - K0 + 1;
    const double k2 = __dmul_rn(__dmul_rn((double)(-k * k), beta), beta);
    const double lap = __dadd_rn(__dadd_rn(m2, k2), n2);
    const double hlap = __dadd_rn(m2, n2);
    const double ilap16 = hypo / lap;
    double inner = __dadd_rn(lap / Re, ilap16);
    if (dragall || k == 0) inner = __dsub_rn(inner, drag);
    const double tvl = __dsub_rn(1.0, __dmul_rn(dt, inner));
    double l, r;
    if (ms == 0 && n == 0) {
      if (slot == 0) { l = 1.0; r = 0.0; }
      else { l = tvl; r = 1.0; }
    } else if (psi) {
      l = __dmul_rn(tvl, hlap);
      r = hlap;
    } else {
      l = __dmul_rn(__dmul_rn(tvl, hlap), lap);
      if (dragall) l = __dadd_rn(l, __dmul_rn(__dmul_rn(__dmul_rn(dt, __dsub_rn(vdrag, drag)), hlap), hlap));
      r = __dmul_rn(hlap, lap);
    }
    const double il = 1.0 / l;
    if (rd->prec == MWF_FP64) {
      ilhs[e] = il;
      rhs[e] = r;
    } else {
      const double A = __dmul_rn(r, il);
      const float hi = __double2float_rn(A);
      float* a = reinterpret_cast<float*>(ilhs);
      a[e] = hi;
      a[tot + e] = __double2float_rn(__dsub_rn(A, (double)hi));
      reinterpret_cast<float*>(rhs)[e] = __double2float_rn(__dmul_rn(dt / 2.0, il));
    }
  }
}

}  // namespace

extern "C" int mwf_step_noalloc(const mwf_run_desc* d, double* c_re, double* c_im, double* onl_re,
                                double* onl_im, int first_step, int nsteps) {
  if (!d || !c_re || !c_im || !onl_re || !onl_im) return fail(MWF_ERR_ARG, "mwf_step_noalloc: null argument");
  if (nsteps < 0) return fail(MWF_ERR_ARG, "mwf_step_noalloc: nsteps < 0");
  if (d->reflect || d->uvreflect || d->wreflect)
    return fail(MWF_ERR_ARG, "mwf_step_noalloc: symmetry masks are not supported by this entry point");
  if (!(d->dt > 0) || !(d->Re > 0)) return fail(MWF_ERR_ARG, "mwf_step_noalloc: dt and Re must be > 0");
  RunHost r;
  r.d = *d;
  const char* why = "";
  if (!plan_run(r, why)) return fail(MWF_ERR_SIZE, "mwf_step_noalloc: %s", why);
  const int prec = d->precision;
  const size_t cb = prec == MWF_FP64 ? 16 : 8;
  // work items of the three passes
  const int n_xf = ((d->NN + r.xf_nb - 1) / r.xf_nb) * 2 * r.KK;
  const int n_z = ((r.X + r.z_lx - 1) / r.z_lx) * 3;
  const int n_xi = ((d->NN + r.xi_nb - 1) / r.xi_nb) * d->K0;
  const int n_items = n_xf + n_z + n_xi;
  // scratch layout: descriptor | error word | items | run arrays
  const size_t off_desc = 0;
  const size_t off_err = align_up(sizeof(RunDesc), 256);
  const size_t off_items = off_err + 256;
  const size_t base = align_up(off_items + sizeof(WorkItem) * (size_t)n_items, 256);
  const size_t need = run_bytes(r, base);
  if (need > MWF_NOALLOC_SCRATCH_BYTES)
    return fail(MWF_ERR_SIZE,
                "mwf_step_noalloc: this run needs %zu bytes of intermediates; the entry point's fixed "
                "scratch holds %zu bytes (use mwf_create/mwf_step for larger runs)",
                need, (size_t)MWF_NOALLOC_SCRATCH_BYTES);
  // The array's name in host code is a host-side stand-in, not a device address: look up its
  // address on the current device at every call (cheap next to the uploads below, and never
  // stale after a device reset or a new primary context).
  unsigned char* sc = nullptr;
  {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(MWF_ERR_CUDA, "mwf_step_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    sc = static_cast<unsigned char*>(ptr);
  }
  cudaStream_t st = 0;
  // descriptor
  RunDesc D;
  memset(&D, 0, sizeof D);
  D.K0 = d->K0; D.MM = d->MM; D.NN = d->NN; D.M = r.M; D.X = r.X; D.Z = r.Z; D.K = r.K; D.KK = r.KK;
  D.prec = prec;
  D.xf_nb = r.xf_nb; D.xi_nb = r.xi_nb; D.z_lx = r.z_lx;
  D.alpha = d->alpha; D.gamma = d->gamma; D.dt = d->dt;
  D.alpha_f = (float)d->alpha; D.gamma_f = (float)d->gamma;
  D.cth = cos(d->theta); D.sth = sin(d->theta);
  D.scale = 1.0 / ((double)r.X * (double)r.Z);
  D.c = sc + r.off_c;
  D.onl = sc + r.off_onl;
  D.inv_lhs = reinterpret_cast<const double*>(sc + r.off_ilhs);
  D.rhs = reinterpret_cast<const double*>(sc + r.off_rhs);
  D.T = sc + r.off_T;
  D.NLT = sc + r.off_NLT;
  D.twX = sc + r.off_twX;
  D.twQ = sc + r.off_twQ;
  D.twZ = sc + r.off_twZ;
  D.nst = reinterpret_cast<int*>(sc + r.off_nst);
  D.active = 1;
  if (!make_plan(r.X, D.planX, r.x_radix) || !make_plan(d->NN, D.planQ, r.z_radix))
    return fail(MWF_ERR_SIZE, "mwf_step_noalloc: no FFT plan");
  CK(cudaMemcpy(sc + off_desc, &D, sizeof D, cudaMemcpyHostToDevice));
  CK(cudaMemset(sc + off_err, 0, sizeof(int)));
  // work items, staged through a small stack buffer
  {
    WorkItem chunk[256];
    int nc = 0, done = 0;
    auto push = [&](WorkItem w) -> cudaError_t {
      chunk[nc++] = w;
      if (nc == 256) {
        cudaError_t e = cudaMemcpy(sc + off_items + sizeof(WorkItem) * done, chunk, sizeof chunk, cudaMemcpyHostToDevice);
        done += nc;
        nc = 0;
        return e;
      }
      return cudaSuccess;
    };
    for (int n0 = 0; n0 < d->NN; n0 += r.xf_nb)
      for (int f = 0; f < 2 * r.KK; ++f) CK(push(WorkItem{0, n0, f, 0}));
    for (int x0 = 0; x0 < r.X; x0 += r.z_lx)
      for (int sub = 0; sub < 3; ++sub) CK(push(WorkItem{0, x0, sub, 0}));
    for (int n0 = 0; n0 < d->NN; n0 += r.xi_nb)
      for (int k = 0; k < d->K0; ++k) CK(push(WorkItem{0, n0, k, 0}));
    if (nc) CK(cudaMemcpy(sc + off_items + sizeof(WorkItem) * done, chunk, sizeof(WorkItem) * nc, cudaMemcpyHostToDevice));
  }
  // twiddles, staged through a small stack buffer
  {
    double tw[2 * 256];
    float twf[2 * 256];
    const size_t offs[3] = {r.off_twX, r.off_twQ, r.off_twZ};
    const int lens[3] = {r.X, d->NN, r.Z};
    for (int q = 0; q < 3; ++q)
      for (int t0 = 0; t0 < lens[q]; t0 += 256) {
        const int cnt = std::min(256, lens[q] - t0);
        if (prec == MWF_FP64) {
          twiddles_into<double>(lens[q], t0, cnt, tw);
          CK(cudaMemcpy(sc + offs[q] + (size_t)t0 * cb, tw, (size_t)cnt * cb, cudaMemcpyHostToDevice));
        } else {
          twiddles_into<float>(lens[q], t0, cnt, twf);
          CK(cudaMemcpy(sc + offs[q] + (size_t)t0 * cb, twf, (size_t)cnt * cb, cudaMemcpyHostToDevice));
        }
      }
  }
  const RunDesc* d_desc = reinterpret_cast<const RunDesc*>(sc + off_desc);
  int* d_err = reinterpret_cast<int*>(sc + off_err);
  const WorkItem* d_items = reinterpret_cast<const WorkItem*>(sc + off_items);
  double* ilhs = reinterpret_cast<double*>(sc + r.off_ilhs);
  double* rhs = reinterpret_cast<double*>(sc + r.off_rhs);
  noalloc_tables_kernel<<<152 * 4, 256, 0, st>>>(d_desc, d->Re, d->drag, d->vdrag, d->hypo, d->dragall, ilhs, rhs);
  CK(cudaGetLastError());
  // caller state (reference layout, FP64) -> device layout in the scratch
  cudaError_t e;
  e = prec == MWF_FP64 ? launch_ref_to_dev_f64(c_re, c_im, sc + r.off_c, r.K, r.M, d->NN, st)
                       : launch_ref_to_dev_f32(c_re, c_im, sc + r.off_c, r.K, r.M, d->NN, st);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "mwf_step_noalloc: state conversion: %s", cudaGetErrorString(e));
  if (!first_step) {
    e = prec == MWF_FP64 ? launch_ref_to_dev_f64(onl_re, onl_im, sc + r.off_onl, r.K, r.M, d->NN, st)
                         : launch_ref_to_dev_f32(onl_re, onl_im, sc + r.off_onl, r.K, r.M, d->NN, st);
    if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "mwf_step_noalloc: history conversion: %s", cudaGetErrorString(e));
  }
  const int nst = first_step ? 1 : 0;
  CK(cudaMemcpy(sc + r.off_nst, &nst, sizeof(int), cudaMemcpyHostToDevice));
  const size_t zsm = zpass_smem(prec, d->K0, r.z_ppt, r.z_nt);
  const size_t xfs = xpass_smem(prec, (size_t)r.xf_nb * r.X);
  const size_t xis = xpass_smem(prec, (size_t)3 * r.xi_nb * r.X);
  for (int s = 0; s < nsteps; ++s) {
    e = prec == MWF_FP64 ? launch_x_forward_f64(r.x_nt, d_desc, d_items, n_xf, xfs, d_err, st)
                         : launch_x_forward_f32(r.x_nt, d_desc, d_items, n_xf, xfs, d_err, st);
    if (e == cudaSuccess)
      e = prec == MWF_FP64 ? launch_z_nonlinear_f64(d->K0, r.z_ppt, r.z_nt, d_desc, d_items + n_xf, n_z, zsm, d_err, st)
                           : launch_z_nonlinear_f32(d->K0, r.z_ppt, r.z_nt, d_desc, d_items + n_xf, n_z, zsm, d_err, st);
    if (e == cudaSuccess)
      e = prec == MWF_FP64 ? launch_x_inverse_f64(r.x_nt, d_desc, d_items + n_xf + n_z, n_xi, xis, d_err, st)
                           : launch_x_inverse_f32(r.x_nt, d_desc, d_items + n_xf + n_z, n_xi, xis, d_err, st);
    if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "mwf_step_noalloc: pass launch: %s", cudaGetErrorString(e));
    CK(cudaMemsetAsync(sc + r.off_nst, 0, sizeof(int), st));
  }
  // a pass that recorded an error skipped work: leave the caller's arrays as they were
  int herr = 0;
  CK(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) return fail(MWF_ERR_DEVICE, "mwf_step_noalloc: kernel reported internal error flags 0x%x", herr);
  // device layout -> caller arrays
  e = prec == MWF_FP64 ? launch_dev_to_ref_f64(sc + r.off_c, c_re, c_im, r.K, r.M, d->NN, st)
                       : launch_dev_to_ref_f32(sc + r.off_c, c_re, c_im, r.K, r.M, d->NN, st);
  if (e == cudaSuccess && nsteps > 0)
    e = prec == MWF_FP64 ? launch_dev_to_ref_f64(sc + r.off_onl, onl_re, onl_im, r.K, r.M, d->NN, st)
                         : launch_dev_to_ref_f32(sc + r.off_onl, onl_re, onl_im, r.K, r.M, d->NN, st);
  if (e != cudaSuccess) return fail(MWF_ERR_CUDA, "mwf_step_noalloc: state conversion: %s", cudaGetErrorString(e));
  CK(cudaStreamSynchronize(st));
  return MWF_OK;
}
