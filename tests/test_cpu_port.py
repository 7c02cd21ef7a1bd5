"""The C++ FP64 restatement (oracle/cpu_step.cpp, the timed CPU baseline) against the numpy
oracle: same steps, same coefficients to rounding."""
import numpy as np
import pytest

from oracle import mwf_oracle as O
from oracle import cpu_port


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def gaussian(p, seed):
    g = np.random.default_rng(seed)
    c = 1e-2 * (g.standard_normal((p.NN, p.M, p.K)) + 1j * g.standard_normal((p.NN, p.M, p.K)))
    c[0] = 0.0            # keep the state physical: no n = 0 column (its Hermitian rule is not imposed)
    return c


@pytest.mark.parametrize("K0,MM,NN,alpha,gamma,theta", [
    (4, 16, 16, 2 * np.pi / 12, 2 * np.pi / 6, 0.0),
    (6, 16, 24, 2 * np.pi / 12, 2 * np.pi / 8, 0.0),
    (4, 24, 18, 0.3, 0.45, 0.2),
    (6, 12, 8, 0.5, 0.7, 0.0),
])
@pytest.mark.parametrize("threads", [1, 3])
def test_cpu_port_matches_oracle(K0, MM, NN, alpha, gamma, theta, threads):
    p = O.Params(K0=K0, MM=MM, NN=NN, alpha=alpha, gamma=gamma, Re=200, dt=0.02, theta=theta)
    c0 = gaussian(p, 3)
    ref = O.Solver(p, c0)
    cpu = cpu_port.CpuSolver(p, c0, threads=threads)
    for _ in range(3):
        ref.step(1)
        cpu.step(1)
        assert rel(cpu.c, ref.c) < 1e-12, rel(cpu.c, ref.c)
    assert rel(cpu.onl, ref.onl) < 1e-12


def test_coupling_term_count():
    """Number of coupling products per point (about half the flop count of udotgradu:
    369 flops for M4 and 1043 for M6 in modes.M4.f90 / modes.M6.f90)."""
    n4 = len(cpu_port.coupling_terms(4)[1])
    n6 = len(cpu_port.coupling_terms(6)[1])
    assert 100 < n4 < 369 and 300 < n6 < 1043, (n4, n6)


def test_rejects_masks():
    p = O.Params(K0=4, MM=8, NN=8, reflect=True)
    with pytest.raises(ValueError):
        cpu_port.CpuSolver(p, np.zeros((p.NN, p.M, p.K), complex))
