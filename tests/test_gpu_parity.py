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


def test_100_steps_fp64_cfg0(built_lib):
    """M4, 96x96 modes (144^2 grid), Re=200, dt=0.02: coefficients after 100 steps."""
    p = mwf.RunParams.square(4, 96, 32 * np.pi, Re=200, dt=0.02)
    c0 = mwf.ic.gaussian_ic(p, seed=0)
    s = O.Solver(oracle_params(p), c0)
    s.step(100)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(100)
        g = ens.get_state(0)
    assert rel(g, s.c) < 1e-11, rel(g, s.c)
