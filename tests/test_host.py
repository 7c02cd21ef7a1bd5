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
