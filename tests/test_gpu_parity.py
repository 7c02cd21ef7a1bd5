"""CUDA path vs the FP64 oracle, through the C ABI (include/mwf_gpu.h)."""
import numpy as np
import pytest

from oracle import mwf_oracle as O
import mwf_gb300 as mwf

pytestmark = pytest.mark.gpu


def oracle_params(p):
    return O.Params(K0=p.K0, MM=p.MM, NN=p.NN, alpha=p.alpha, gamma=p.gamma, Re=p.Re, dt=p.dt,
                    drag=p.drag, vdrag=p.vdrag, hypo=p.hypo, dragall=p.dragall, theta=p.theta,
                    reflect=p.reflect, uvreflect=p.uvreflect, wreflect=p.wreflect)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


SMALL = [
    (4, 16, 16, 2 * np.pi / 12, 2 * np.pi / 6),
    (4, 48, 48, 1 / 16, 1 / 16),
    (6, 16, 24, 2 * np.pi / 12, 2 * np.pi / 8),
    (4, 24, 16, 2 * np.pi / 10, 2 * np.pi / 7),
]


@pytest.mark.parametrize("K0,MM,NN,alpha,gamma", SMALL)
def test_one_step_fp64(built_lib, K0, MM, NN, alpha, gamma):
    p = mwf.RunParams(K0=K0, MM=MM, NN=NN, alpha=alpha, gamma=gamma, Re=200, dt=0.02)
    c0 = mwf.ic.gaussian_ic(p, seed=1, kmax=6)
    s = O.Solver(oracle_params(p), c0)
    s.step(1)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(1)
        g = ens.get_state(0)
    assert rel(g, s.c) < 1e-12, rel(g, s.c)


def test_state_roundtrip(built_lib):
    p = mwf.RunParams(K0=6, MM=16, NN=16)
    c0 = mwf.ic.gaussian_ic(p, seed=3)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        assert np.array_equal(ens.get_state(0), c0)


@pytest.mark.parametrize("K0", [4, 6])
def test_energy_fp64(built_lib, K0):
    p = mwf.RunParams(K0=K0, MM=24, NN=16)
    c0 = mwf.ic.gaussian_ic(p, seed=5)
    e_ref = O.energy(oracle_params(p), c0)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        e = ens.energy(0)
    assert abs(e - e_ref) <= 1e-13 * abs(e_ref), (e, e_ref)


def test_cfg0_500_steps_energy_series(built_lib):
    """The CPU-runnable case (M4, 96x96 modes on a 144^2 grid, Lx = Lz = 32 pi, Re = 200,
    dt = 0.02, Gaussian IC seed 0) for all of its 500 steps.  The vel_energy.dat rows are written
    every 50 steps before the step (io_write2files, io.f90:87-116; io_write_energy, io.f90:453-467),
    i.e. at steps 0, 50, ..., 450, in the reference's '(2e20.12)' format: the GPU's rows match the
    oracle's to 1e-10 relative, and the coefficients after 100 steps match to 1e-11."""
    from mwf_gb300 import state_io
    p = mwf.RunParams.square(4, 96, 32 * np.pi, Re=200, dt=0.02)
    c0 = mwf.ic.gaussian_ic(p, seed=0)
    s = O.Solver(oracle_params(p), c0)
    gpu_rows, ref_rows = [], []
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        for step in range(0, 500, 50):
            t = step * p.dt
            gpu_rows.append(state_io.energy_row(t, ens.energy(0)))
            ref_rows.append(state_io.energy_row(t, s.energy()))
            ens.step(50)
            s.step(50)
            if step + 50 == 100:
                g = ens.get_state(0)
                assert rel(g, s.c) < 1e-11, rel(g, s.c)
    gpu = state_io.parse_energy_rows("\n".join(gpu_rows))
    ref = state_io.parse_energy_rows("\n".join(ref_rows))
    assert len(gpu) == len(ref) == 10 and all(len(r) == 40 for r in gpu_rows)
    for (tg, eg), (tr, er) in zip(gpu, ref):
        assert tg == tr
        assert abs(eg - er) <= 1e-10 * abs(er), (tg, eg, er)


def test_100_steps_fp64_m6(built_lib):
    p = mwf.RunParams.square(6, 64, 24 * np.pi, Re=300, dt=0.01)
    c0 = mwf.ic.spot_ic(p, seed=2, width=10.0)
    s = O.Solver(oracle_params(p), c0)
    s.step(100)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(100)
        g = ens.get_state(0)
    assert rel(g, s.c) < 1e-11, rel(g, s.c)


def test_parameters_and_odd_sizes_fp64(built_lib):
    """theta, hypo, vdrag, dragall off; NN odd (odd z grid), MM != NN."""
    p = mwf.RunParams(K0=4, MM=36, NN=27, alpha=0.3, gamma=0.4, Re=180, dt=0.015, drag=0.02,
                      vdrag=0.005, hypo=1e-4, dragall=False, theta=0.3)
    c0 = mwf.ic.gaussian_ic(p, seed=9, kmax=5, amp=0.03)
    s = O.Solver(oracle_params(p), c0)
    s.step(20)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(20)
        g = ens.get_state(0)
    assert rel(g, s.c) < 1e-12, rel(g, s.c)


def test_fp32_error_bar_after_100_steps(built_lib):
    """FP32 path vs the FP64 oracle: <= 1e-4 relative coefficient error after 100 steps and
    <= 1% mean-energy error over the run."""
    p64 = mwf.RunParams.square(4, 96, 32 * np.pi, Re=200, dt=0.02)
    p32 = p64.with_(precision="fp32")
    c0 = mwf.ic.gaussian_ic(p64, seed=0)
    s = O.Solver(oracle_params(p64), c0)
    e_ref, e_got = [], []
    with mwf.Ensemble([p32]) as ens:
        ens.set_state(0, c0)
        for _ in range(4):
            e_ref.append(s.energy())
            e_got.append(ens.energy(0))
            s.step(25)
            ens.step(25)
        g = ens.get_state(0)
    assert rel(g, s.c) <= 1e-4, rel(g, s.c)
    assert abs(np.mean(e_got) - np.mean(e_ref)) <= 1e-2 * abs(np.mean(e_ref))


def test_ensemble_mix_equals_alone(built_lib):
    a = 2 * np.pi / 40
    runs = [mwf.RunParams(K0=4, MM=32, NN=32, alpha=a, gamma=a, Re=250, dt=0.02),
            mwf.RunParams(K0=6, MM=16, NN=24, alpha=a, gamma=a, Re=300, dt=0.01),
            mwf.RunParams(K0=4, MM=48, NN=16, alpha=a, gamma=a, Re=150, dt=0.02, precision="fp32"),
            mwf.RunParams(K0=6, MM=24, NN=24, alpha=a, gamma=a, Re=350, dt=0.01, precision="fp32")]
    ics = [mwf.ic.gaussian_ic(p, seed=10 + i, kmax=6) for i, p in enumerate(runs)]
    with mwf.Ensemble(runs) as ens:
        for i, c in enumerate(ics):
            ens.set_state(i, c)
        ens.step(7)
        mixed = [ens.get_state(i) for i in range(len(runs))]
    for i, p in enumerate(runs):
        with mwf.Ensemble([p]) as one:
            one.set_state(0, ics[i])
            one.step(7)
            alone = one.get_state(0)
        assert np.all(np.isfinite(alone)), i
        assert np.array_equal(alone, mixed[i]), i


def test_restart_is_euler_step(built_lib):
    """After mwf_reset_history the next step is the Euler start (velocity.f90:24-27)."""
    p = mwf.RunParams(K0=4, MM=16, NN=16, Re=200, dt=0.02)
    c0 = mwf.ic.gaussian_ic(p, seed=11, kmax=6)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(3)
        c3 = ens.get_state(0)
        ens.reset_history(0)
        ens.step(2)
        g = ens.get_state(0)
    s = O.Solver(oracle_params(p), c3)      # fresh solver: nst = .true.
    s.step(2)
    assert rel(g, s.c) < 1e-12


def test_symmetry_masks_m4(built_lib):
    p = mwf.RunParams(K0=4, MM=16, NN=12, Re=200, dt=0.02, reflect=True, uvreflect=True, wreflect=True)
    c0 = mwf.ic.gaussian_ic(p, seed=12, kmax=6)
    s = O.Solver(oracle_params(p), c0)
    s.step(5)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(5)
        g = ens.get_state(0)
    assert rel(g, s.c) < 1e-12


def test_energy_series_cadence(built_lib):
    """vel_energy.dat rows (t, E) every 50 steps, written before the step (io.f90:87-116)."""
    p = mwf.RunParams.square(4, 64, 24 * np.pi, Re=250, dt=0.02)
    c0 = mwf.ic.gaussian_ic(p, seed=13)
    s = O.Solver(oracle_params(p), c0)
    ref, got = [], []
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        for _ in range(4):
            ref.append(s.energy())
            got.append(ens.energy(0))
            s.step(50)
            ens.step(50)
    ref, got = np.array(ref), np.array(got)
    assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()


def test_unsupported_size_is_rejected(built_lib):
    with pytest.raises(mwf.MwfError) as e:
        mwf.Ensemble([mwf.RunParams(K0=4, MM=10, NN=16)])
    assert e.value.code == -2
    with pytest.raises(mwf.MwfError) as e:
        mwf.Ensemble([mwf.RunParams(K0=5, MM=16, NN=16)])
    assert e.value.code == -2


def test_fp64_medium_grid_10_steps(built_lib):
    p = mwf.RunParams.square(6, 256, 96 * np.pi, Re=300, dt=0.01)
    c0 = mwf.ic.gaussian_ic(p, seed=14)
    s = O.Solver(oracle_params(p), c0)
    s.step(10)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(10)
        g = ens.get_state(0)
    assert rel(g, s.c) < 1e-12


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_physical_diagnostics(built_lib, prec):
    p = mwf.RunParams.square(6, 96, 30 * np.pi, Re=300, dt=0.01, precision=prec)
    c0 = mwf.ic.spot_ic(p, seed=21, width=12.0)
    op = oracle_params(p)
    e_ref = O.energy(op, c0)
    P = O.spec2phys(op, O.mpt2spec(op, c0))
    ep = O.epos(p.K0, P)
    srt = np.sort(ep.ravel())
    k = int(0.7 * srt.size)
    ct = float(0.5 * (srt[k] + srt[k + 1]))           # between two grid values: no ties
    cnt_ref, e_phys_ref = O.turbulent_count(op, c0, ct)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        cnt, e_phys = ens.phys_diagnostics(0, ct)
        e_spec = ens.energy(0)
        frac = ens.turbulent_fraction(0, ct)
    tol = 1e-12 if prec == "fp64" else 2e-6
    assert abs(e_phys - e_phys_ref) <= tol * abs(e_phys_ref)
    assert abs(e_spec - e_ref) <= tol * abs(e_ref)
    assert abs(e_phys_ref - e_ref) <= 1e-13 * e_ref          # Parseval: spectral == physical
    assert abs(cnt - cnt_ref) <= (0 if prec == "fp64" else 0.001 * p.X * p.Z)
    assert frac == cnt / ((p.X + 1) * (p.Z + 1))


@pytest.mark.parametrize("K0,MM,NN", [(4, 16, 12), (6, 24, 16), (4, 48, 27)])
def test_standalone_transforms(built_lib, K0, MM, NN):
    """mwf_spec2phys / mwf_phys2spec (the transform module's tra_spec2phys / tra_phys2spec on
    caller fields) against the oracle's FFTW-convention restatements, and their round trip."""
    from mwf_gb300 import solver
    p = mwf.RunParams(K0=K0, MM=MM, NN=NN, alpha=0.3, gamma=0.45)
    op = oracle_params(p)
    rng = np.random.default_rng(K0 * 1000 + MM + NN)
    s = rng.standard_normal((NN, p.M, p.KK)) + 1j * rng.standard_normal((NN, p.M, p.KK))
    ph = solver.spec2phys(p, s)
    ref = O.spec2phys(op, s)
    assert np.abs(ph - ref).max() <= 1e-13 * np.abs(ref).max()
    back = solver.phys2spec(p, ph)
    ref_back = O.phys2spec(op, ph)
    assert np.abs(back - ref_back).max() <= 1e-13 * np.abs(ref_back).max()
    # the round trip keeps the retained modes, except what c2r drops (Im of the n = 0, m = 0 term
    # and the non-Hermitian part of the n = 0 column)
    assert np.abs(back[1:] - s[1:]).max() <= 1e-12 * np.abs(s).max()


def test_restart_from_state_file(built_lib, tmp_path):
    """A run saved to the reference's netCDF state format (io_save_state, io.f90:257-340) and
    reloaded into a new handle continues with the Euler start the reference uses after a restart
    (the AB2 history is not in the file; nst = .true., velocity.f90:24-27,48): after 30 + 20 steps
    it matches the oracle restarted from the same state to 1e-11, and it differs from the
    uninterrupted run."""
    from mwf_gb300 import state_io
    p = mwf.RunParams.square(4, 96, 32 * np.pi, Re=200, dt=0.02)
    c0 = mwf.ic.gaussian_ic(p, seed=4)
    f = tmp_path / "state0001.cdf.dat"
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(30)
        state_io.save_state(str(f), ens.get_state(0), p.K0, p.MM, p.NN, t=30 * p.dt, Re=p.Re, alpha=p.alpha,
                            gamma=p.gamma)
        ens.step(20)
        uninterrupted = ens.get_state(0)
    c30, attrs = state_io.load_state(str(f), p.K0, p.MM, p.NN)
    assert attrs["t"] == 30 * p.dt
    vel = mwf.Velocity(p)
    vel.vel_c = c30
    vel.reset_history()
    vel.vel_TS(20)
    got = vel.vel_c
    vel.close()
    s = O.Solver(oracle_params(p), c0)
    s.step(30)
    restarted = O.Solver(oracle_params(p), s.c.copy())
    restarted.step(20)
    assert rel(got, restarted.c) < 1e-11, rel(got, restarted.c)
    assert rel(got, uninterrupted) > 1e-9


def test_persistent_step_mode_is_bitwise_the_same(built_lib):
    """One persistent launch per step (mwf_set_persistent) against the default launches per pass:
    a mixed ensemble -- FP32 M4 and M6 runs with batched passes (in the persistent launch), an
    FP32 run whose z line has no batched kernel and an FP64 run (in their own launches) -- gives
    bitwise the same states after 12 steps, and stays on the FP64 oracle."""
    a = 2 * np.pi / 40
    runs = [mwf.RunParams(K0=4, MM=32, NN=32, alpha=a, gamma=a, Re=250, dt=0.02, precision="fp32"),
            mwf.RunParams(K0=4, MM=64, NN=48, alpha=a, gamma=a, Re=200, dt=0.02, precision="fp32"),
            mwf.RunParams(K0=6, MM=48, NN=64, alpha=a, gamma=a, Re=300, dt=0.01, precision="fp32"),
            mwf.RunParams(K0=4, MM=32, NN=27, alpha=a, gamma=a, Re=180, dt=0.02, precision="fp32"),
            mwf.RunParams(K0=4, MM=32, NN=32, alpha=a, gamma=a, Re=220, dt=0.02)]
    ics = [mwf.ic.gaussian_ic(p, seed=40 + i, kmax=6) for i, p in enumerate(runs)]
    out = {}
    for persistent in (False, True):
        with mwf.Ensemble(runs) as ens:
            ens.set_persistent(persistent)
            assert (ens.kernels_per_step() < 10) == persistent
            for i, c in enumerate(ics):
                ens.set_state(i, c)
            ens.step(12)
            out[persistent] = [ens.get_state(i) for i in range(len(runs))]
    for i in range(len(runs)):
        assert np.array_equal(out[True][i], out[False][i]), i
    s = O.Solver(oracle_params(runs[1].with_(precision="fp64")), ics[1])
    s.step(12)
    assert rel(out[True][1], s.c) < 1e-4
