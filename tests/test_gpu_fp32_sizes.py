"""FP32 runs against the FP64 oracle at the grid sizes with compile-time transform plans.

The ensemble sizes (M4, N x N modes with N in {64, 96, 128, 192, 256}, i.e. MM = NN = 32..128,
domain L = N pi/3, dt = 0.02): 100 steps, coefficients within 1e-4 of the oracle and mean energy
over the run (every 25 steps) within 1 %.  Larger lines (MM = NN up to 512, M4 and M6): 20 steps
within 1e-4.  The oracle at these sizes is the C++ FP64 restatement of the step
(oracle/cpu_step.cpp), itself checked against the numpy oracle to 1e-12 (tests/test_cpu_port.py).
"""
import os

import numpy as np
import pytest

import mwf_gb300 as mwf
from oracle import cpu_port
from oracle import mwf_oracle as O

pytestmark = pytest.mark.gpu

THREADS = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def oracle(p, c0):
    op = O.Params(K0=p.K0, MM=p.MM, NN=p.NN, alpha=p.alpha, gamma=p.gamma, Re=p.Re, dt=p.dt, drag=p.drag,
                  vdrag=p.vdrag, hypo=p.hypo, dragall=p.dragall, theta=p.theta)
    return op, cpu_port.CpuSolver(op, c0, threads=THREADS)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


ENSEMBLE_SIZES = [32, 48, 64, 96, 128]        # MM = NN


def test_fp32_ensemble_sizes_100_steps(built_lib):
    runs = [mwf.RunParams.square(4, 2 * n, 2 * n * np.pi / 3, Re=150.0 + 40 * i, dt=0.02, precision="fp32")
            for i, n in enumerate(ENSEMBLE_SIZES)]
    ics = [mwf.ic.gaussian_ic(p, seed=i) for i, p in enumerate(runs)]
    refs = [oracle(p.with_(precision="fp64"), c) for p, c in zip(runs, ics)]
    e_got = [[] for _ in runs]
    e_ref = [[] for _ in runs]
    with mwf.Ensemble(runs) as ens:
        for i, c in enumerate(ics):
            ens.set_state(i, c)
        for _ in range(4):
            for i, (op, s) in enumerate(refs):
                e_got[i].append(ens.energy(i))
                e_ref[i].append(O.energy(op, s.c))
                s.step(25)
            ens.step(25)
        got = [ens.get_state(i) for i in range(len(runs))]
    for i, n in enumerate(ENSEMBLE_SIZES):
        op, s = refs[i]
        err = rel(got[i], s.c)
        assert err <= 1e-4, f"MM = NN = {n}: FP32 coefficient error {err:.3e} after 100 steps"
        me_got, me_ref = np.mean(e_got[i]), np.mean(e_ref[i])
        assert abs(me_got - me_ref) <= 1e-2 * abs(me_ref), f"MM = NN = {n}: mean energy {me_got} vs {me_ref}"
        s.close()


LARGE_SIZES = [192, 256, 384, 512]


@pytest.mark.parametrize("K0", [4, 6])
def test_fp32_large_lines_20_steps(built_lib, K0):
    runs = [mwf.RunParams.square(K0, 2 * n, 2 * n * np.pi / 3, Re=200.0, dt=0.01, precision="fp32")
            for n in LARGE_SIZES]
    ics = [0.3 * mwf.ic.gaussian_ic(p, seed=i) for i, p in enumerate(runs)]
    with mwf.Ensemble(runs) as ens:
        for i, c in enumerate(ics):
            ens.set_state(i, c)
        ens.step(20)
        got = [ens.get_state(i) for i in range(len(runs))]
    for i, n in enumerate(LARGE_SIZES):
        _, s = oracle(runs[i].with_(precision="fp64"), ics[i])
        s.step(20)
        assert np.isfinite(got[i]).all(), f"MM = NN = {n}: state not finite"
        err = rel(got[i], s.c)
        s.close()
        assert err < 1e-4, f"MM = NN = {n}: FP32 vs oracle relative error {err:.3e} after 20 steps"


@pytest.mark.parametrize("K0,MM,NN", [(4, 16, 27), (6, 12, 9), (4, 18, 81)])
def test_odd_z_lines(built_lib, K0, MM, NN):
    """Odd NN: the rows of a z task do not all start on 16-byte boundaries, so the FP32 z pass
    stages them element by element (cp.async) instead of by bulk copies; the transforms are the
    generic engine's radix-3 plans.  FP64 against the oracle, FP32 against FP64."""
    p64 = mwf.RunParams(K0=K0, MM=MM, NN=NN, alpha=2 * np.pi / 10, gamma=2 * np.pi / 9, Re=200.0, dt=0.01)
    p32 = p64.with_(precision="fp32")
    c0 = 0.3 * mwf.ic.gaussian_ic(p64, seed=21, kmax=6)
    with mwf.Ensemble([p64, p32]) as ens:
        ens.set_state(0, c0)
        ens.set_state(1, c0)
        ens.step(5)
        a, b = ens.get_state(0), ens.get_state(1)
    s = O.Solver(O.Params(K0=K0, MM=MM, NN=NN, alpha=p64.alpha, gamma=p64.gamma, Re=p64.Re, dt=p64.dt), c0)
    s.step(5)
    assert np.abs(a - s.c).max() / np.abs(s.c).max() < 1e-12
    assert np.isfinite(b).all()
    assert np.abs(b - a).max() / np.abs(a).max() < 1e-4


@pytest.mark.parametrize("kind", ["previous_x", "previous_z"])
def test_fp32_previous_kernels_still_match(built_lib, kind):
    """A radix cap selects the previous FP32 kernels (run-time plans over the whole x line, or the
    staged z pass); they stay on the oracle too (M4, 96^2 modes, 20 steps, 1e-4)."""
    kw = {"x_radix": 16} if kind == "previous_x" else {"z_radix": 12}
    p = mwf.RunParams.square(4, 96, 32 * np.pi, Re=200.0, dt=0.02, precision="fp32", **kw)
    c0 = mwf.ic.gaussian_ic(p, seed=0)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(20)
        g = ens.get_state(0)
    _, s = oracle(p.with_(precision="fp64", x_radix=0, z_radix=0), c0)
    s.step(20)
    assert rel(g, s.c) < 1e-4
    s.close()
