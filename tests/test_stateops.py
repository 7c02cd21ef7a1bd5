"""State operations and diagnostics outside the timestep: physical field (vel_mpt2phys),
spectrum maxima (io_save_Uspec), velocity probes (vel_history), x remap (var_doubleX /
var_quadX), state blend (utils/interpstate) and additive noise (var_randadd).

CPU tests pin the oracle's restatements against direct evaluations of the reference's loops;
GPU tests compare the C ABI with the oracle."""
import numpy as np
import pytest

from oracle import mwf_oracle as O
import mwf_gb300 as mwf


def oracle_params(p):
    return O.Params(K0=p.K0, MM=p.MM, NN=p.NN, alpha=p.alpha, gamma=p.gamma, Re=p.Re, dt=p.dt,
                    drag=p.drag, vdrag=p.vdrag, hypo=p.hypo, dragall=p.dragall, theta=p.theta,
                    reflect=p.reflect, uvreflect=p.uvreflect, wreflect=p.wreflect)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def rand_state(p, seed):
    g = np.random.default_rng(seed)
    return g.standard_normal(p.shape) + 1j * g.standard_normal(p.shape)


# ---------------------------------------------------------------------------------------
# Oracle restatements against literal loops (CPU)
# ---------------------------------------------------------------------------------------
def quadx_loop(c, MM, factor):
    """var_quadX (variables.f90:168-185) as a literal loop over (n, m), Fortran slot
    arithmetic, with the mirror index generalised from 4 to factor."""
    NN, M, K = c.shape
    tmp = np.zeros_like(c)
    for n in range(NN):
        for m in range(M):
            mm = factor * m
            if m > MM - 1:
                mm = M - (factor * (M - m))
                if mm < MM - 1:
                    continue
            else:
                if mm > MM - 1:
                    continue
            tmp[n, mm, :] = c[n, m, :]
    return tmp


@pytest.mark.parametrize("MM,factor", [(8, 1), (8, 2), (8, 4), (9, 3), (12, 4), (16, 2), (6, 5)])
def test_remap_oracle_matches_loop(MM, factor):
    p = O.Params(K0=4, MM=MM, NN=6)
    c = rand_state(mwf.RunParams(K0=4, MM=MM, NN=6), 1)
    assert np.array_equal(O.remap_x(p, c, factor), quadx_loop(c, MM, factor))


def test_remap_wavenumbers():
    """Wavenumber m of the old state is wavenumber factor*m of the new one."""
    MM, f = 16, 2
    p = O.Params(K0=4, MM=MM, NN=4)
    c = rand_state(mwf.RunParams(K0=4, MM=MM, NN=4), 2)
    out = O.remap_x(p, c, f)
    M = 2 * MM - 1
    for m in range(-(MM - 1), MM):
        t = f * m
        if abs(t) <= MM - 1 and t != -MM:
            assert np.array_equal(out[:, t % M], c[:, m % M])
    # the reference's quirk: wavenumber -MM (from -MM/f) lands in slot MM-1
    assert np.array_equal(out[:, MM - 1], c[:, (-MM // f) % M])


def test_remap_identity():
    p = O.Params(K0=6, MM=12, NN=5)
    c = rand_state(mwf.RunParams(K0=6, MM=12, NN=5), 3)
    assert np.array_equal(O.remap_x(p, c, 1), c)


def test_splitmix64_known_answers():
    """SplitMix64 from state 0: the published first outputs of the generator."""
    g = np.uint64(0x9E3779B97F4A7C15)
    with np.errstate(over="ignore"):
        got = [int(O._splitmix64(np.array([g * np.uint64(i)], np.uint64))[0]) for i in range(3)]
    assert got == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_noise_oracle_properties():
    p = O.Params(K0=4, MM=8, NN=6)
    c = rand_state(mwf.RunParams(K0=4, MM=8, NN=6), 4)
    a = O.add_noise(p, c, 1e-3, seed=7)
    b = O.add_noise(p, c, 1e-3, seed=7)
    assert np.array_equal(a, b)
    assert np.array_equal(a[0], c[0]) and np.array_equal(a[:, 0], c[:, 0])
    d = (a - c)[1:, 1:]
    assert (d.real >= 0).all() and (d.real < 1e-3 * (1 + 1e-12)).all()
    assert (d.imag >= 0).all() and (d.imag < 1e-3 * (1 + 1e-12)).all()
    assert not np.array_equal(O.add_noise(p, c, 1e-3, seed=8), a)


def test_spectrum_oracle_matches_loop():
    """io_save_Uspec (io.f90:345-372) as a literal loop over (n, m, k)."""
    p = O.Params(K0=4, MM=6, NN=5, alpha=0.7, gamma=0.9)
    c = rand_state(mwf.RunParams(K0=4, MM=6, NN=5), 5)
    s = O.mpt2spec(p, c)
    n_ = np.zeros(p.NN)
    m_ = np.zeros(p.MM)
    for n in range(p.NN):
        for m in range(p.M):
            mm = p.M - m if m > p.MM - 1 else m
            for k in range(p.KK):
                d = np.sqrt(s[n, m, k].real ** 2 + s[n, m, k].imag ** 2)
                n_[n] = max(d, n_[n])
                m_[mm] = max(d, m_[mm])
    mo, no = O.spectrum_maxima(p, c)
    assert np.array_equal(mo, m_) and np.array_equal(no, n_)


def test_history_oracle_direct_sum():
    """vel_history from the transforms against a direct sum of the Fourier series at x = 0."""
    p = O.Params(K0=6, MM=6, NN=8, alpha=0.5, gamma=0.8)
    c = rand_state(mwf.RunParams(K0=6, MM=6, NN=8), 6)
    y = 0.3
    H = O.history(p, c, y, n_probes=7)
    s = O.mpt2spec(p, c)                        # (NN, M, KK)
    g = s.sum(axis=1)                           # x = 0: sum over m
    beta = np.pi / 2
    for j in range(7):
        z = j * p.Z // 7 + 1
        ph = np.exp(2j * np.pi * np.arange(p.NN) * z / p.Z)
        f = g[0].real + 2 * (g[1:] * ph[1:, None]).real.sum(axis=0)
        u = f[0] + sum((np.sin(k * beta * y) if k % 2 else np.cos(k * beta * y)) * f[k] for k in range(1, 6))
        v = sum((np.cos(k * beta * y) if k % 2 else np.sin(k * beta * y)) * f[5 + k] for k in range(1, 6))
        w = f[11] + sum((np.sin(k * beta * y) if k % 2 else np.cos(k * beta * y)) * f[11 + k] for k in range(1, 6))
        assert abs(H[j, 0] - z * (2 * np.pi / p.gamma) / p.Z) < 1e-14
        np.testing.assert_allclose(H[j, 1:], [u, v, w], rtol=0, atol=1e-12 * np.abs(f).max())


def test_blend_oracle():
    c1 = rand_state(mwf.RunParams(K0=4, MM=4, NN=4), 8)
    c2 = rand_state(mwf.RunParams(K0=4, MM=4, NN=4), 9)
    assert np.array_equal(O.blend(c1, c2, 0.0), c1)
    assert np.array_equal(O.blend(c1, c2, 1.0), c2)


# ---------------------------------------------------------------------------------------
# CUDA path vs the oracle (GPU)
# ---------------------------------------------------------------------------------------
CASES = [
    (4, 16, 16, 2 * np.pi / 12, 2 * np.pi / 6, "fp64"),
    (6, 16, 24, 2 * np.pi / 12, 2 * np.pi / 8, "fp64"),
    (4, 24, 18, 0.3, 0.45, "fp64"),
    (4, 16, 16, 2 * np.pi / 12, 2 * np.pi / 6, "fp32"),
    (6, 24, 16, 0.4, 0.5, "fp32"),
]


def _case(K0, MM, NN, alpha, gamma, prec, seed=1):
    p = mwf.RunParams(K0=K0, MM=MM, NN=NN, alpha=alpha, gamma=gamma, Re=200, dt=0.02, precision=prec)
    c0 = mwf.ic.gaussian_ic(p, seed=seed, kmax=6)
    if prec == "fp32":
        c0 = c0.astype(np.complex64).astype(np.complex128)
    return p, c0


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_get_phys(built_lib, case):
    p, c0 = _case(*case)
    ref = O.phys_field(oracle_params(p), c0)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        g = ens.get_phys(0)
    tol = 1e-12 if p.precision == "fp64" else 2e-6
    assert g.shape == ref.shape
    assert rel(g, ref) < tol, rel(g, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_spectrum_maxima(built_lib, case):
    p, c0 = _case(*case)
    mo, no = O.spectrum_maxima(oracle_params(p), c0)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        m, n = ens.spectrum_maxima(0)
    tol = 1e-14 if p.precision == "fp64" else 1e-6
    assert rel(m, mo) < tol and rel(n, no) < tol, (rel(m, mo), rel(n, no))


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("y,nprobe", [(0.0, 32), (0.37, 5)])
def test_history(built_lib, case, y, nprobe):
    p, c0 = _case(*case)
    ref = O.history(oracle_params(p), c0, y, nprobe)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        H = ens.history(0, y, nprobe)
    assert np.array_equal(H[:, 0], ref[:, 0])
    tol = 1e-12 if p.precision == "fp64" else 2e-6
    scale = np.abs(O.phys_field(oracle_params(p), c0)).max()
    assert np.abs(H[:, 1:] - ref[:, 1:]).max() < tol * scale


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("factor", [1, 2, 3, 4])
def test_remap_x(built_lib, prec, factor):
    p, c0 = _case(4, 24, 16, 0.3, 0.45, prec)
    ref = O.remap_x(oracle_params(p), c0, factor)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(2)                       # leaves AB2 history that the remap must discard
        ens.set_state(0, c0)
        ens.remap_x(0, factor)
        g = ens.get_state(0)
        assert np.array_equal(g, ref)
        ens.step(1)                       # Euler start after the remap
        g1 = ens.get_state(0)
    if prec == "fp64":
        s = O.Solver(oracle_params(p), ref)
        s.step(1)
        assert rel(g1, s.c) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_blend_and_noise(built_lib, prec):
    p, c1 = _case(6, 16, 24, 0.4, 0.3, prec, seed=3)
    _, c2 = _case(6, 16, 24, 0.4, 0.3, prec, seed=4)
    d = 0.3
    # FP32 runs compute each operation in FP64 and round the result to FP32
    to_run = (lambda a: a) if prec == "fp64" else (lambda a: a.astype(np.complex64).astype(np.complex128))
    ref = to_run(O.blend(c1, c2, d))
    ref_n = to_run(O.add_noise(oracle_params(p), ref, 1e-4, 12345))
    with mwf.Ensemble([p, p]) as ens:
        ens.set_state(0, c1)
        ens.set_state(1, c2)
        ens.blend_state(0, 1, d)
        g = ens.get_state(0)
        assert np.array_equal(ens.get_state(1), c2)
        ens.add_noise(0, 1e-4, 12345)
        gn = ens.get_state(0)
    assert np.array_equal(g, ref)
    assert np.array_equal(gn, ref_n)


@pytest.mark.gpu
def test_phys_energy_parseval_large(built_lib):
    """M6, 512 x 512 modes (1536^2 grid), FP64: the physical field returned by the device
    gives the spectral (Parseval) energy of mwf_energy, and its x = 0 column the probes."""
    p = mwf.RunParams.square(6, 512, 128 * np.pi, Re=300, dt=0.01)
    c0 = mwf.ic.spot_ic(p, seed=0)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(5)
        ph = ens.get_phys(0)
        e = ens.energy(0)
        H = ens.history(0, 0.0, 32)
        _, e_dev = ens.phys_diagnostics(0, 0.1)
    e_phys = O.epos(6, ph).sum() / (p.X * p.Z)
    assert abs(e_phys - e) < 1e-10 * abs(e), (e_phys, e)
    assert abs(e_dev - e) < 1e-10 * abs(e)
    K0 = 6
    for j in range(32):
        z = j * p.Z // 32 + 1
        V = ph[0, z]
        np.testing.assert_allclose(H[j, 1], V[0] + V[2] + V[4], rtol=0, atol=1e-12 * np.abs(ph).max())
        np.testing.assert_allclose(H[j, 2], V[K0] + V[K0 + 2] + V[K0 + 4], rtol=0, atol=1e-12 * np.abs(ph).max())


@pytest.mark.gpu
def test_stateops_errors(built_lib):
    p, c0 = _case(4, 16, 16, 0.5, 0.5, "fp64")
    q = mwf.RunParams(K0=4, MM=24, NN=16)
    with mwf.Ensemble([p, q]) as ens:
        with pytest.raises(mwf.MwfError):
            ens.remap_x(0, 0)
        with pytest.raises(mwf.MwfError):
            ens.blend_state(0, 1, 0.5)
        with pytest.raises(mwf.MwfError):
            ens.history(0, 0.0, 0)
        with pytest.raises(mwf.MwfError):
            ens.history(0, 0.0, p.Z)
        ens.set_active(0, False)
        with pytest.raises(mwf.MwfError):
            ens.get_phys(0)
        ens.set_active(0, True)
        ens.set_state(0, c0)
        assert np.isfinite(ens.get_phys(0)).all()
