"""FP32 runs at the grid sizes with compile-time transform plans (32..512 modes, MM = NN = 16..256:
x lines 48..768, z lines 16..256), M4 and M6, in one ensemble with FP64 runs on the same states (the FP64
path is itself checked against the oracle in tests/test_gpu_parity.py): coefficients within 1e-4 after
5 steps."""
import numpy as np
import pytest

import mwf_gb300 as mwf

pytestmark = pytest.mark.gpu

SIZES = [32, 48, 64, 96, 128, 192, 256, 384, 512]


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
