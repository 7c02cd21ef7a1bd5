// Host program for tests/test_cpp_host.py: drives one run through the C++ interface
// (include/mwf_velocity.hpp) the way the reference's main loop drives its velocity module.
//
//   velocity_parity format              write fortran_e20_12 of a few values (no GPU needed)
//   velocity_parity errors              the error path: a grid the library rejects
//   velocity_parity run <in> <out> <dir>
//       in : int32 K0, MM, NN, precision, nsteps; float64 alpha, gamma, Re, dt;
//            float64 re[K*M*NN], im[K*M*NN] (type(mpt) layout)
//       out: float64 re, im after nsteps; E (vel_energy); m_max[MM], n_max[NN];
//            H[4*32] (vel_history at y = 0); phys[KK*Z*X] (vel_mpt2phys); t
//       dir: vel_energy.dat, vel_history.dat and vel_spec0001.dat written as io.f90 does
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mwf_velocity.hpp"

static bool read_all(std::FILE* f, void* p, size_t n) { return std::fread(p, 1, n, f) == n; }

int main(int argc, char** argv) {
  if (argc >= 2 && std::strcmp(argv[1], "format") == 0) {
    const double vals[] = {0.0, 1.0, -2.5, 123456.789, 1e-7, -9.99999999999999e-3, 6.02214076e23, 1e-120};
    for (double v : vals) std::printf("[%s]\n", mwf::fortran_e20_12(v).c_str());
    return 0;
  }
  if (argc >= 2 && std::strcmp(argv[1], "errors") == 0) {
    try {
      mwf::velocity v(mwf::run_desc(4, 7, 8, 0.5, 0.5, 200.0, 0.02));   // 7 is not 2^a 3^b
      std::printf("no error\n");
      return 1;
    } catch (const mwf::error& e) {
      std::printf("code %d: %s\n", e.code(), e.what());
      return 0;
    }
  }
  if (argc != 5 || std::strcmp(argv[1], "run") != 0) {
    std::fprintf(stderr, "usage: velocity_parity format | errors | run <in> <out> <dir>\n");
    return 2;
  }
  std::FILE* fi = std::fopen(argv[2], "rb");
  if (!fi) return 3;
  int32_t hdr[5];
  double par[4];
  if (!read_all(fi, hdr, sizeof hdr) || !read_all(fi, par, sizeof par)) return 3;
  const mwf_run_desc d = mwf::run_desc(hdr[0], hdr[1], hdr[2], par[0], par[1], par[2], par[3], hdr[3]);
  const int nsteps = hdr[4];
  try {
    mwf::velocity v(d);                                   // vel_precompute
    std::vector<double> re(v.mpt_size()), im(v.mpt_size());
    if (!read_all(fi, re.data(), re.size() * 8) || !read_all(fi, im.data(), im.size() * 8)) return 3;
    std::fclose(fi);
    v.set_vel_c(re.data(), im.data());                    // io_load_state

    const std::string dir = argv[4];
    std::FILE* fe = std::fopen((dir + "/vel_energy.dat").c_str(), "w");
    std::FILE* fh = std::fopen((dir + "/vel_history.dat").c_str(), "w");
    if (!fe || !fh) return 4;
    std::vector<double> H;
    // the main loop of main.f90:18-28 with io_write2files every 5 steps
    for (int s = 0; s < nsteps; ++s) {
      if (v.tim_step % 5 == 0) {
        mwf::write_energy_row(fe, v.tim_t, v.vel_energy());
        v.vel_history(0.0, 32, H);
        mwf::write_history_rows(fh, v.tim_t, H);
      }
      v.vel_TS(1);
    }
    std::fclose(fe);
    std::fclose(fh);

    v.get_vel_c(re.data(), im.data());                    // io_save_state
    const double E = v.vel_energy();
    std::vector<double> mm, nn, phys;
    v.vel_spec(mm, nn);
    mwf::write_vel_spec(dir + "/vel_spec0001.dat", v.tim_t, mm, nn);
    v.vel_history(0.0, 32, H);
    v.vel_mpt2phys(phys);

    std::FILE* fo = std::fopen(argv[3], "wb");
    if (!fo) return 4;
    std::fwrite(re.data(), 8, re.size(), fo);
    std::fwrite(im.data(), 8, im.size(), fo);
    std::fwrite(&E, 8, 1, fo);
    std::fwrite(mm.data(), 8, mm.size(), fo);
    std::fwrite(nn.data(), 8, nn.size(), fo);
    std::fwrite(H.data(), 8, H.size(), fo);
    std::fwrite(phys.data(), 8, phys.size(), fo);
    std::fwrite(&v.tim_t, 8, 1, fo);
    std::fclose(fo);
  } catch (const mwf::error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 5;
  }
  return 0;
}
