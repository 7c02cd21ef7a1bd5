"""The FP64 oracle against the reference's own expressions and physics known answers (CPU)."""
import os

import numpy as np
import pytest

from oracle import mwf_oracle as O
from oracle import galerkin

HERE = os.path.dirname(os.path.abspath(__file__))


def golden(K0):
    return np.load(os.path.join(HERE, "golden", f"udotgradu_M{K0}.npz"))


@pytest.mark.parametrize("K0", [4, 6])
def test_udotgradu_matches_reference_expressions(K0):
    d = golden(K0)
    got = O.udotgradu(K0, d["v"], d["vx"], d["vz"])
    ref = d["udotgradu"]
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_m4_explicit_and_helper_forms_agree():
    d = golden(4)
    assert np.abs(d["udotgradu"] - d["udotgradu2"]).max() <= 1e-13 * np.abs(d["udotgradu"]).max()


@pytest.mark.parametrize("K0", [4, 6])
def test_epos_matches_reference(K0):
    d = golden(K0)
    assert np.abs(O.epos(K0, d["v"]) - d["epos"]).max() <= 1e-13 * np.abs(d["epos"]).max()


def small(K0=4, MM=8, NN=6, **kw):
    return O.Params(K0=K0, MM=MM, NN=NN, alpha=2 * np.pi / 9, gamma=2 * np.pi / 7, Re=150, dt=0.02, **kw)


def rand_state(p, seed=0, scale=0.2):
    rng = np.random.default_rng(seed)
    c = (rng.standard_normal(p.shape if hasattr(p, "shape") else (p.NN, p.M, p.K))
         + 1j * rng.standard_normal((p.NN, p.M, p.K))) * scale
    for m in range(1, p.MM):
        c[0, (-m) % p.M, :] = np.conj(c[0, m, :])
    c[0, 0, :] = c[0, 0, :].real
    c[0, 0, 0] = 0
    return c


def test_zero_perturbation_stays_zero():
    p = small()
    s = O.Solver(p, np.zeros((p.NN, p.M, p.K), complex))
    s.step(3)
    assert np.abs(s.c).max() == 0.0


def test_linear_update_closed_form(monkeypatch):
    p = small()
    c0 = rand_state(p)
    monkeypatch.setattr(O, "nonlinear", lambda p_, c: np.zeros_like(c))
    s = O.Solver(p, c0)
    s.step(4)
    L, R = O.lhsrhs(p)
    expect = c0 * (R / L) ** 4
    expect[0, 0, 0] = 1j * expect[0, 0, 0].imag
    assert np.allclose(s.c, expect, rtol=1e-13, atol=1e-15)


def test_lhsrhs_mean_and_shared_slot():
    p = small(K0=4)
    L, R = O.lhsrhs(p)
    assert L[0, 0, 0] == 1.0 and R[0, 0, 0] == 0.0            # psi_0 mean pinned
    # slot K0-1 holds psi_{K0-1}: l = tvl * hlap with lap of k = K0-1
    m1, m2, n1, n2, k1, k2 = O.tables(p)
    lap = m2[2] + k2[3] + n2[1]
    tvl = 1 - p.dt * (lap / p.Re - p.drag)
    assert np.isclose(L[1, 2, 3], tvl * (m2[2] + n2[1]), rtol=1e-15)
    assert np.all(np.isfinite(L)) and np.all(np.isfinite(R))


def test_transform_roundtrip_on_retained_modes():
    p = small(K0=4, MM=10, NN=8)
    rng = np.random.default_rng(3)
    s = rng.standard_normal((p.NN, p.M, 5)) + 1j * rng.standard_normal((p.NN, p.M, 5))
    for m in range(1, p.MM):
        s[0, (-m) % p.M, :] = np.conj(s[0, m, :])
    s[0, 0, :] = s[0, 0, :].real
    back = O.phys2spec(p, O.spec2phys(p, s))
    assert np.abs(back - s).max() < 1e-13


def test_c2r_ignores_imaginary_dc():
    p = small()
    s = np.zeros((p.NN, p.M, 1), complex)
    s[0, 0, 0] = 1.0 + 5.0j
    ph = O.spec2phys(p, s)
    assert np.allclose(ph, 1.0)


def test_velocity_is_divergence_free():
    p = small(K0=6, MM=7, NN=5)
    c = rand_state(p, 4)
    s = O.mpt2spec(p, c)
    m1, _, n1, _, k1, _ = O.tables(p)
    K0 = p.K0
    for k in range(K0):
        su, sw = s[:, :, k], s[:, :, 2 * K0 - 1 + k]
        div = 1j * m1[None, :] * su + 1j * n1[:, None] * sw
        if k >= 1:
            div = div + k1[k] * s[:, :, K0 + k - 1]
        div[0, 0] = 0.0          # mean modes are x,z-independent
        assert np.abs(div).max() < 1e-12 * max(1.0, np.abs(s).max())


def test_hermitian_column_preserved():
    p = small()
    s = O.Solver(p, rand_state(p, 5))
    s.step(2)
    c = s.c
    for m in range(1, p.MM):
        assert np.allclose(c[0, (-m) % p.M, :], np.conj(c[0, m, :]), atol=1e-14)


def test_energy_single_mode_analytic():
    p = small()
    c = np.zeros((p.NN, p.M, p.K), complex)
    psi = 0.3 - 0.1j
    c[0, 1, 1] = psi                  # psi_1 at m = +-1, n = 0  ->  w_1 = i alpha m psi_1
    c[0, p.M - 1, 1] = np.conj(psi)
    # E = weight(w_1) * sum_m |w_1(m)|^2 = 0.5 * 2 * alpha^2 |psi|^2
    expect = p.alpha ** 2 * abs(psi) ** 2
    assert np.isclose(O.energy(p, c), expect, rtol=1e-13)


def test_galerkin_tensors_are_exact_fractions():
    Gp, Gv, Hp, Hv, Ev = galerkin.tensors(4)
    for t, unit in ((Gp, 1.0), (Gv, 1.0), (Ev, 1.0), (Hp, np.pi / 2), (Hv, np.pi / 2)):
        q = t / unit * 4
        assert np.abs(q - np.round(q)).max() < 1e-10
