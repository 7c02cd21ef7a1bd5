"""Host-side helpers: initial conditions, state files, size rounding (CPU)."""
import numpy as np
import pytest

import mwf_gb300 as mwf
from mwf_gb300 import ic, state_io
from oracle import mwf_oracle as O


def test_gaussian_ic_properties():
    p = mwf.RunParams(K0=4, MM=48, NN=48)
    c = ic.gaussian_ic(p, seed=0)
    assert c.shape == p.shape
    for m in range(1, p.MM):
        assert np.array_equal(c[0, (-m) % p.M, :], np.conj(c[0, m, :]))
    assert np.all(c[0, 0, :].imag == 0) and c[0, 0, 0] == 0
    n, m = np.nonzero(np.abs(c).sum(axis=2))
    ms = np.where(m >= p.MM, m - p.M, m)
    assert np.all(ms ** 2 + n ** 2 <= 64)
    assert np.array_equal(c, ic.gaussian_ic(p, seed=0))
    assert not np.array_equal(c, ic.gaussian_ic(p, seed=1))
    # the same low modes on a different grid
    q = mwf.RunParams(K0=4, MM=32, NN=24)
    c2 = ic.gaussian_ic(q, seed=0)
    assert np.array_equal(c2[:9, :9, :], c[:9, :9, :])


def test_spot_ic_is_localised_and_hermitian():
    p = mwf.RunParams.square(4, 64, 200.0)
    c = ic.spot_ic(p, seed=2, width=20.0)
    for m in range(1, p.MM):
        assert np.allclose(c[0, (-m) % p.M, :], np.conj(c[0, m, :]), atol=1e-15)
    op = O.Params(K0=4, MM=p.MM, NN=p.NN, alpha=p.alpha, gamma=p.gamma)
    e = O.epos(4, O.spec2phys(op, O.mpt2spec(op, c)))
    X, Z = e.shape
    centre = e[X // 2 - 5:X // 2 + 5, Z // 2 - 5:Z // 2 + 5].mean()
    corner = e[:10, :10].mean()
    assert centre > 20 * corner


@pytest.mark.parametrize("K0,MM,NN", [(4, 16, 12), (6, 24, 16), (4, 9, 8)])
def test_uvw_map_inverts_mpt2spec(K0, MM, NN):
    """ic.mpt_to_uvw is the oracle's var_mpt2spec (variables.f90:390-434) without the base flow,
    and ic.uvw_to_mpt inverts it on every MPT state with psi_0(0,0) = 0 (the coefficient
    var_mpt2spec does not carry)."""
    p = mwf.RunParams(K0=K0, MM=MM, NN=NN, alpha=0.3, gamma=0.45)
    rng = np.random.default_rng(K0 * 100 + MM)
    c = rng.standard_normal(p.shape) + 1j * rng.standard_normal(p.shape)
    c[0, 0, :] = c[0, 0, :].real
    c[0, 0, 0] = 0.0
    op = O.Params(K0=K0, MM=MM, NN=NN, alpha=p.alpha, gamma=p.gamma)
    s = ic.mpt_to_uvw(p, c)
    ref = O.mpt2spec(op, c)
    assert np.abs(s - ref).max() <= 1e-14 * np.abs(ref).max()
    assert np.abs(ic.uvw_to_mpt(p, s) - c).max() <= 1e-14 * np.abs(c).max()


def test_spot_ic_is_the_projected_envelope_field():
    """The spot IC is the projection onto MPT of (Gaussian field x envelope): its own velocity
    field, projected again, is itself (the projection is idempotent), and it differs from the
    envelope field only by a divergent part, i.e. v and the vertical vorticity agree exactly
    away from the mean mode (m, n) = (0, 0), whose plane-mean v no divergence-free field has."""
    p = mwf.RunParams.square(4, 64, 120.0)
    c = ic.spot_ic(p, seed=5, width=20.0)
    s = ic.mpt_to_uvw(p, c)
    assert np.abs(ic.uvw_to_mpt(p, s) - c).max() <= 1e-14 * np.abs(c).max()
    X, Z = 3 * p.MM, 3 * p.NN
    Lx, Lz = 2 * np.pi / p.alpha, 2 * np.pi / p.gamma
    x = np.arange(X) * Lx / X
    z = np.arange(Z) * Lz / Z
    env = np.exp(-((x[:, None] - Lx / 2) ** 2 + (z[None, :] - Lz / 2) ** 2) / (2 * 20.0 ** 2))
    g = ic.gaussian_ic(p, seed=5)
    f = ic._to_spec(p, ic._to_phys(p, ic.mpt_to_uvw(p, g)) * env[:, :, None])
    K0 = p.K0
    dv = np.abs(s[:, :, K0:2 * K0 - 1] - f[:, :, K0:2 * K0 - 1])
    dv[0, 0] = 0.0
    assert dv.max() <= 1e-13 * np.abs(f).max()
    m1, n1, _ = ic._wavenumbers(p)
    vort = lambda a: n1[:, None, None] * a[:, :, :K0] - m1[None, :, None] * a[:, :, 2 * K0 - 1:]
    dw = np.abs(vort(s) - vort(f))
    dw[0, 0] = 0.0
    assert dw.max() <= 1e-13 * np.abs(vort(f)).max()


def test_state_file_roundtrip(tmp_path):
    p = mwf.RunParams(K0=6, MM=8, NN=6)
    c = ic.gaussian_ic(p, seed=4, kmax=5)
    f = tmp_path / "state0001.cdf.dat"
    state_io.save_state(str(f), c, 6, 8, 6, t=1.5, Re=300.0, alpha=p.alpha, gamma=p.gamma, onl=2 * c)
    got, attrs = state_io.load_state(str(f), 6, 8, 6)
    assert np.array_equal(got, c)
    assert attrs["t"] == 1.5 and attrs["Re"] == 300.0
    assert np.array_equal(attrs["onl"], 2 * c)
    with pytest.raises(state_io.StateFileError):
        state_io.load_state(str(f), 4, 8, 6)
    with pytest.raises(state_io.StateFileError):
        state_io.load_state(str(tmp_path / "missing.cdf"))


def test_grid_size_rounds_to_2a3b():
    assert mwf.round_23(100) == 96
    assert mwf.round_23(64) == 64
    assert all(mwf.is_23_smooth(mwf.round_23(n)) for n in range(2, 600))


def test_fortran_e20_12_rows():
    """The '(2e20.12)' rows of vel_energy.dat (io.f90:453-467): 0.d12 mantissa, E+dd exponent,
    20 columns each."""
    f = state_io.fortran_e20_12
    assert f(0.0) == "  0.000000000000E+00"
    assert f(1.0) == "  0.100000000000E+01"
    assert f(-3.25e-7) == " -0.325000000000E-06"
    assert f(123456.789) == "  0.123456789000E+06"
    assert f(2.5e150) == "  0.250000000000+151"
    row = state_io.energy_row(0.02 * 50, 4778.66853315512)
    assert len(row) == 40
    assert state_io.parse_energy_rows(row + "\n") == [(1.0, 4778.66853316)]
