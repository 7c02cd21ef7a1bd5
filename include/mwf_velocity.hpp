// mwf_velocity.hpp -- C++17 host interface over the C ABI (mwf_gpu.h) that mirrors the
// reference's `velocity` module (program/velocity.f90) for one run, with the module's names:
//
//   reference (Fortran, velocity.f90 / io.f90)        here
//   vel_precompute (43-50), var_precompute, ...        mwf::velocity v(desc, device)
//   vel_c%Re, vel_c%Im  (module state, 15-17)          v.get_vel_c(re, im) / v.set_vel_c(re, im)
//   vel_TS with vel_imposesym (main.f90:22-24)         v.vel_TS(nsteps)
//   tim_t, tim_step (main.f90:25-26)                   v.tim_t, v.tim_step
//   nst = .true. after a restart (48)                  v.vel_reset_history()
//   vel_energy(vel_mpt2phys(vel_c)) (84-90, 144-162)   v.vel_energy()
//   vel_mpt2phys(vel_c, p) (84-90)                     v.vel_mpt2phys(p)   p = phys%Re(KK, Z, X)
//   vel_history(p, y, H) (164-180)                     v.vel_history(y, n, H)
//   io_save_Uspec maxima (io.f90:345-372)              v.vel_spec(m_max, n_max)
//   var_doubleX / var_quadX (variables.f90:147-185)    v.var_doubleX() / v.var_quadX()
//   var_randadd (variables.f90:253-269)                v.var_randadd(scl, seed)
//
// and the three text writers of io.f90 (vel_energy.dat rows, vel_history rows, vel_spec files)
// in the reference's Fortran formats.  The reference stops the program on an error
// (io.f90:135,177,195); here every failing call throws mwf::error with the library's message.
// The state lives on the GPU; the host arrays are only read or written by the calls that name
// them.  Link with -lmwfgpu.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "mwf_gpu.h"

namespace mwf {

// A failed call of the C ABI: the MWF_ERR_* code and mwf_last_error()'s message.
class error : public std::runtime_error {
 public:
  error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc) {
  if (rc == MWF_OK) return;
  char buf[512];
  mwf_last_error(buf, sizeof buf);
  throw error(rc, std::string("mwf: ") + buf);
}

// The run descriptor with the defaults of program/parameters.f90 (M4, drag 1e-2 on every
// mode, no hypo-viscosity, theta = 0, no symmetry masks, FP64).
inline mwf_run_desc run_desc(int K0, int MM, int NN, double alpha, double gamma, double Re, double dt,
                             int precision = MWF_FP64) {
  mwf_run_desc d{};
  d.K0 = K0; d.MM = MM; d.NN = NN; d.precision = precision;
  d.alpha = alpha; d.gamma = gamma; d.Re = Re; d.dt = dt;
  d.drag = 1e-2; d.vdrag = 0.0; d.hypo = 0.0; d.dragall = 1;
  d.theta = 0.0;
  return d;
}

// One run on one GPU: the module state of velocity.f90 (vel_c, vel_onl, nst) on the device.
class velocity {
 public:
  explicit velocity(const mwf_run_desc& d, int device = 0) : d_(d) {
    check(mwf_create(&d_, 1, device, &h_));
    K = 2 * d.K0 - 1;
    KK = 3 * d.K0 - 1;
    M = 2 * d.MM - 1;
    X = 3 * d.MM;
    Z = 3 * d.NN;
  }
  ~velocity() {
    if (h_) mwf_destroy(h_);
  }
  velocity(const velocity&) = delete;
  velocity& operator=(const velocity&) = delete;

  // sizes: K MPT components, KK spectral fields, M x slots, X x Z physical grid
  int K = 0, KK = 0, M = 0, X = 0, Z = 0;
  double tim_t = 0.0;
  long tim_step = 0;

  const mwf_run_desc& desc() const { return d_; }
  size_t mpt_size() const { return (size_t)K * M * d_.NN; }
  size_t phys_size() const { return (size_t)KK * Z * X; }

  // vel_c in the layout of type(mpt): Re(K, 0:M-1, 0:NN-1) and Im, K*M*NN doubles each
  void set_vel_c(const double* re, const double* im) { check(mwf_set_state(h_, 0, re, im)); }
  void get_vel_c(double* re, double* im) const { check(mwf_get_state(h_, 0, re, im)); }

  // vel_imposesym + vel_TS, nsteps times, advancing tim_t and tim_step as main.f90 does
  void vel_TS(int nsteps = 1) {
    check(mwf_step(h_, nsteps));
    tim_t += nsteps * d_.dt;
    tim_step += nsteps;
  }
  void vel_reset_history() { check(mwf_reset_history(h_, 0)); }

  double vel_energy() const {
    double e = 0.0;
    check(mwf_energy(h_, 0, &e));
    return e;
  }
  // type(phys)%Re(KK, 0:Z-1, 0:X-1), field index fastest
  void vel_mpt2phys(std::vector<double>& p) const {
    p.resize(phys_size());
    check(mwf_get_phys(h_, 0, p.data()));
  }
  // H(4, n): (z position, u, v, w) at x = 0 and height y for each probe
  void vel_history(double y, int n, std::vector<double>& H) const {
    H.resize((size_t)4 * n);
    check(mwf_history(h_, 0, y, n, H.data()));
  }
  // the two columns of vel_spec%04d.dat: max over |m| (MM values) and over n (NN values)
  void vel_spec(std::vector<double>& m_max, std::vector<double>& n_max) const {
    m_max.resize(d_.MM);
    n_max.resize(d_.NN);
    check(mwf_spectrum_maxima(h_, 0, m_max.data(), n_max.data()));
  }
  // physical-space diagnostics: points with epos > ct and the energy of vel_energy
  void phys_diagnostics(double ct, double* count, double* energy) const {
    check(mwf_phys_diagnostics(h_, 0, ct, count, energy));
  }

  void var_doubleX() { check(mwf_remap_x(h_, 0, 2)); }
  void var_quadX() { check(mwf_remap_x(h_, 0, 4)); }
  void var_randadd(double scl, unsigned long long seed = 0) { check(mwf_add_noise(h_, 0, scl, seed)); }

  mwf_handle* handle() const { return h_; }

 private:
  mwf_run_desc d_;
  mwf_handle* h_ = nullptr;
};

// ---- text output in the reference's formats ----------------------------------------------

// Fortran's Ew.d edit descriptor for w = 20, d = 12 (the reference's '(2e20.12)' and
// '(6e20.12)'): optional minus sign, "0.", twelve digits, exponent "E+dd" (or "+ddd" without
// the E from 100 on), right-justified in 20 columns.
inline std::string fortran_e20_12(double v) {
  char out[64];
  if (v == 0.0 || !std::isfinite(v)) {
    if (v == 0.0) std::snprintf(out, sizeof out, "%20s", std::signbit(v) ? "-0.000000000000E+00" : "0.000000000000E+00");
    else std::snprintf(out, sizeof out, "%20s", std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity"));
    return out;
  }
  char sci[64];
  std::snprintf(sci, sizeof sci, "%.11e", std::fabs(v));    // d.ddddddddddde+XX, 12 significant
  const char* epos = std::strchr(sci, 'e');
  const int ex = std::atoi(epos + 1) + 1;                    // 0.dddddddddddd x 10^ex
  std::string digits;
  for (const char* q = sci; q < epos; ++q)
    if (*q != '.') digits += *q;
  char mant[40];
  if (ex >= -99 && ex <= 99) std::snprintf(mant, sizeof mant, "%s0.%sE%c%02d", v < 0 ? "-" : "", digits.c_str(),
                                           ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
  else std::snprintf(mant, sizeof mant, "%s0.%s%c%03d", v < 0 ? "-" : "", digits.c_str(), ex < 0 ? '-' : '+',
                     ex < 0 ? -ex : ex);
  std::snprintf(out, sizeof out, "%20s", mant);
  return out;
}

// One row of vel_energy.dat: write(io_KE,'(2e20.12)') tim_t, E (io.f90:453-467)
inline void write_energy_row(std::FILE* f, double t, double E) {
  std::fprintf(f, "%s%s\n", fortran_e20_12(t).c_str(), fortran_e20_12(E).c_str());
}

// The rows of io_write_history (io.f90:473-483): '(6e20.12)' tim_t, 0, H(1..4, i)
inline void write_history_rows(std::FILE* f, double t, const std::vector<double>& H) {
  for (size_t i = 0; i + 3 < H.size(); i += 4)
    std::fprintf(f, "%s%s%s%s%s%s\n", fortran_e20_12(t).c_str(), fortran_e20_12(0.0).c_str(),
                 fortran_e20_12(H[i]).c_str(), fortran_e20_12(H[i + 1]).c_str(), fortran_e20_12(H[i + 2]).c_str(),
                 fortran_e20_12(H[i + 3]).c_str());
}

// vel_spec%04d.dat of io_save_Uspec (io.f90:380-393): header lines, then '(i4,1e20.12)' rows
// of |m| and of n.  The reference writes its header lines list-directed, whose number format
// depends on the Fortran compiler; they carry the same text here, with t in e20.12.
inline void write_vel_spec(const std::string& path, double t, const std::vector<double>& m_max,
                           const std::vector<double>& n_max) {
  std::FILE* f = std::fopen(path.c_str(), "w");
  if (!f) throw error(MWF_ERR_ARG, "mwf: cannot open " + path);
  std::fprintf(f, " # t = %s\n", fortran_e20_12(t).c_str());
  std::fprintf(f, " # m\n");
  for (size_t i = 0; i < m_max.size(); ++i) std::fprintf(f, "%4zu%s\n", i, fortran_e20_12(m_max[i]).c_str());
  std::fprintf(f, "\n # n\n");
  for (size_t i = 0; i < n_max.size(); ++i) std::fprintf(f, "%4zu%s\n", i, fortran_e20_12(n_max[i]).c_str());
  std::fclose(f);
}

}  // namespace mwf
