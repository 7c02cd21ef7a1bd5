"""FP32 runs at the grid sizes with compile-time transform plans (MM = NN = 32..512, i.e. 64..1024
modes: x lines 96..1536, z lines 32..512; NN > 256 takes the 512-thread z pass), M4 and M6, in one
ensemble with FP64 runs on the same states (the FP64 path is itself checked against the oracle in
tests/test_gpu_parity.py): coefficients within 1e-4 after 5 steps."""
import numpy as np
import pytest

import mwf_gb300 as mwf

pytestmark = pytest.mark.gpu

SIZES = [32, 48, 64, 96, 128, 192, 256, 384, 512]   # MM = NN


@pytest.mark.parametrize("K0", [4, 6])
def test_fp32_fixed_plan_sizes(built_lib, K0):
    runs64 = [mwf.RunParams.square(K0, 2 * n, 2 * n * np.pi / 3, Re=200.0, dt=0.01) for n in SIZES]
    runs32 = [p.with_(precision="fp32") for p in runs64]
    states = [0.3 * mwf.ic.gaussian_ic(p, seed=i) for i, p in enumerate(runs64)]
    with mwf.Ensemble(runs64 + runs32) as ens:
        for i, c in enumerate(states):
            ens.set_state(i, c)
            ens.set_state(len(SIZES) + i, c)
        ens.step(5)
        states64 = [ens.get_state(i) for i in range(len(SIZES))]
        states32 = [ens.get_state(len(SIZES) + i) for i in range(len(SIZES))]
        summary = [(n, float(np.abs(x).max()), float(np.abs(y).max())) for n, x, y in zip(SIZES, states64, states32)]
        for i, n in enumerate(SIZES):
            a, b = states64[i], states32[i]
            assert np.isfinite(b).all() and np.isfinite(a).all(), f"MM = NN = {n}: state not finite {summary}"
            err = np.abs(b - a).max() / np.abs(a).max()
            assert err < 1e-4, f"MM = NN = {n}: FP32 vs FP64 relative error {err:.3e}; (MM, max|c64|, max|c32|): {summary}"


@pytest.mark.parametrize("K0,MM,NN", [(4, 16, 27), (6, 12, 9), (4, 18, 81)])
def test_odd_z_lines(built_lib, K0, MM, NN):
    """Odd NN: the rows of a z task do not all start on 16-byte boundaries, so the FP32 z pass
    stages them element by element (cp.async) instead of by bulk copies; the transforms are the
    generic engine's radix-3 plans.  FP64 against the oracle, FP32 against FP64."""
    from oracle import mwf_oracle as O
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
