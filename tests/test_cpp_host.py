"""The C++ host interface (include/mwf_velocity.hpp), compiled and driven like the reference's
main loop drives its velocity module (tests/cpp/velocity_parity.cpp), against the oracle."""
import os
import struct
import subprocess

import numpy as np
import pytest

from oracle import mwf_oracle as O
import mwf_gb300 as mwf

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def cpp_bin(tmp_path_factory):
    from mwf_gb300 import build
    build.build()
    lib = os.path.join(ROOT, "mwf_gb300", "lib")
    exe = str(tmp_path_factory.mktemp("cpp") / "velocity_parity")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "velocity_parity.cpp"), "-o", exe, f"-L{lib}", "-lmwfgpu",
                    f"-Wl,-rpath,{lib}"], check=True)
    return exe


def test_fortran_e_format(cpp_bin):
    """Fortran's E20.12 edit descriptor, as the reference's energy and history files use."""
    out = subprocess.run([cpp_bin, "format"], check=True, capture_output=True, text=True).stdout.split("\n")
    got = [ln[1:-1] for ln in out if ln]
    assert got == ["  0.000000000000E+00", "  0.100000000000E+01", " -0.250000000000E+01",
                   "  0.123456789000E+06", "  0.100000000000E-06", " -0.100000000000E-01",
                   "  0.602214076000E+24", "  0.100000000000-119"]
    for s, v in zip(got[:7], [0.0, 1.0, -2.5, 123456.789, 1e-7, -1e-2, 6.02214076e23]):
        assert len(s) == 20 and float(s) == pytest.approx(v, rel=1e-12)


def test_errors_raise(cpp_bin):
    """A rejected configuration reaches the caller as mwf::error (with a GPU present: the size
    check's MWF_ERR_SIZE; without a GPU, the missing device)."""
    r = subprocess.run([cpp_bin, "errors"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("code -")


@pytest.mark.gpu
def test_errors_size_code(cpp_bin):
    r = subprocess.run([cpp_bin, "errors"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith(f"code {-2}:"), r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("K0,MM,NN", [(4, 16, 16), (6, 16, 24)])
def test_cpp_velocity_matches_oracle(cpp_bin, tmp_path, K0, MM, NN):
    p = mwf.RunParams(K0=K0, MM=MM, NN=NN, alpha=2 * np.pi / 12, gamma=2 * np.pi / 6, Re=200.0, dt=0.02)
    op = O.Params(K0=K0, MM=MM, NN=NN, alpha=p.alpha, gamma=p.gamma, Re=p.Re, dt=p.dt)
    c0 = 0.01 * mwf.ic.gaussian_ic(p, seed=4, kmax=6)     # small amplitude: stays bounded over the steps
    nsteps = 7
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        f.write(struct.pack("<5i4d", K0, MM, NN, 0, nsteps, p.alpha, p.gamma, p.Re, p.dt))
        f.write(np.ascontiguousarray(c0.real).tobytes())
        f.write(np.ascontiguousarray(c0.imag).tobytes())
    subprocess.run([cpp_bin, "run", str(fin), str(fout), str(tmp_path)], check=True)

    n = p.dof
    raw = np.fromfile(fout, dtype=np.float64)
    re, im = raw[:n].reshape(p.shape), raw[n:2 * n].reshape(p.shape)
    o = 2 * n
    E = raw[o]; o += 1
    mm = raw[o:o + MM]; o += MM
    nn = raw[o:o + NN]; o += NN
    H = raw[o:o + 128].reshape(32, 4); o += 128
    phys = raw[o:o + p.KK * p.Z * p.X].reshape(p.X, p.Z, p.KK); o += p.KK * p.Z * p.X
    t = raw[o]

    s = O.Solver(op, c0)
    s.step(nsteps)
    c = re + 1j * im
    rel = lambda a, b: np.abs(a - b).max() / np.abs(b).max()
    assert rel(c, s.c) < 1e-12
    assert abs(E - O.energy(op, s.c)) < 1e-12 * abs(E)
    mo, no = O.spectrum_maxima(op, s.c)
    assert rel(mm, mo) < 1e-12 and rel(nn, no) < 1e-12
    assert np.abs(c).max() < 10 * np.abs(c0).max()
    ph = O.phys_field(op, s.c)
    assert rel(phys, ph) < 1e-12
    Ho = O.history(op, s.c, 0.0, 32)
    assert np.array_equal(H[:, 0], Ho[:, 0])
    assert np.abs(H[:, 1:] - Ho[:, 1:]).max() < 1e-12 * np.abs(ph).max()
    assert t == pytest.approx(nsteps * p.dt, rel=1e-15)

    # the text files, in io.f90's formats: energy rows at steps 0 and 5, 32 history rows each
    rows = [ln.split() for ln in open(tmp_path / "vel_energy.dat")]
    assert len(rows) == 2 and all(len(r) == 2 for r in rows)
    assert float(rows[0][1]) == pytest.approx(O.energy(op, c0), rel=1e-11)
    assert float(rows[1][0]) == pytest.approx(5 * p.dt, rel=1e-11)
    hist = [ln for ln in open(tmp_path / "vel_history.dat")]
    assert len(hist) == 64 and all(len(ln.rstrip("\n")) == 120 for ln in hist)
    spec = open(tmp_path / "vel_spec0001.dat").read().split("\n")
    assert spec[0].startswith(" # t =") and spec[1] == " # m" and spec[2 + MM] == "" and spec[3 + MM] == " # n"
    assert float(spec[2][4:]) == pytest.approx(mo[0], rel=1e-11)
