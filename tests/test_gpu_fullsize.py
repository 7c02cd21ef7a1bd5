"""Parity at the full sizes of the benchmark configurations, with the C++ FP64 restatement
(oracle/cpu_step.cpp, itself checked against the numpy oracle in tests/test_cpu_port.py) as the
oracle: it runs a 1536^2 or 3072^2 step in well under a second on the host's cores."""
import os

import numpy as np
import pytest

from oracle import mwf_oracle as O
from oracle import cpu_port
import mwf_gb300 as mwf

pytestmark = pytest.mark.gpu

PI = 3.1415926535897931
THREADS = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def oracle_params(p):
    return O.Params(K0=p.K0, MM=p.MM, NN=p.NN, alpha=p.alpha, gamma=p.gamma, Re=p.Re, dt=p.dt,
                    drag=p.drag, vdrag=p.vdrag, hypo=p.hypo, dragall=p.dragall, theta=p.theta)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_m6_1536_grid_100_steps(built_lib):
    """M6, 1024 x 1024 modes on the 1536^2 grid, Re 300, dt 0.01, spot IC: coefficients after
    50 and 100 steps within 1e-11 relative of the FP64 CPU restatement."""
    p = mwf.RunParams.square(6, 1024, 256 * PI, Re=300.0, dt=0.01)
    c0 = mwf.ic.spot_ic(p, seed=0)
    cpu = cpu_port.CpuSolver(oracle_params(p), c0, threads=THREADS)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        for chunk in (50, 50):
            ens.step(chunk)
            cpu.step(chunk)
            g = ens.get_state(0)
            assert rel(g, cpu.c) < 1e-11, rel(g, cpu.c)
    cpu.close()


def test_m4_3072_grid_fp64_and_fp32(built_lib):
    """M4, 2048 x 2048 modes on the 3072^2 grid, Re 250, dt 0.01, Gaussian IC |k| <= 16:
    FP64 within 1e-11 of the CPU restatement after 20 steps; FP32 within 1e-4 (coefficients)
    and 1 % (energy) of it after 100 steps."""
    p64 = mwf.RunParams.square(4, 2048, 512 * PI, Re=250.0, dt=0.01)
    p32 = p64.with_(precision="fp32")
    c0 = mwf.ic.gaussian_ic(p64, seed=0, kmax=16)
    cpu = cpu_port.CpuSolver(oracle_params(p64), c0, threads=THREADS)
    with mwf.Ensemble([p64, p32]) as ens:
        ens.set_state(0, c0)
        ens.set_state(1, c0)
        ens.step(20)
        cpu.step(20)
        assert rel(ens.get_state(0), cpu.c) < 1e-11
        ens.step(80)
        cpu.step(80)
        g32 = ens.get_state(1)
        e32 = ens.energy(1)
    e_ref = O.energy(oracle_params(p64), cpu.c)
    cpu.close()
    assert rel(g32, cpu.c) < 1e-4, rel(g32, cpu.c)
    assert abs(e32 - e_ref) < 1e-2 * abs(e_ref), (e32, e_ref)
