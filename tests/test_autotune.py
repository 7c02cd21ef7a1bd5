"""Autotuner knobs: validation on CPU, tuned handles on the GPU."""
import numpy as np
import pytest

import mwf_gb300 as mwf
from mwf_gb300 import autotune


def test_knob_validation_host_only():
    p = mwf.RunParams(K0=4, MM=48, NN=48)
    assert mwf.footprint_bytes([p.with_(z_lines=1, xf_cols=4, xi_cols=2, x_radix=8, z_radix=8)]) > 0
    assert mwf.footprint_bytes([p.with_(z_lines=10 ** 4)]) == -1       # more lines than fit a CTA
    assert mwf.footprint_bytes([p.with_(x_radix=7)]) == -1
    assert mwf.footprint_bytes([p.with_(z_radix=16)]) == -1             # above the FP64 z cap
    assert mwf.footprint_bytes([p.with_(precision="fp32", z_radix=12)]) > 0


@pytest.mark.gpu
def test_tuned_run_matches_default(built_lib, tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "tune.json"))
    autotune._mem.clear()
    p = mwf.RunParams.square(4, 96, 32 * np.pi, Re=200, dt=0.02)
    c0 = mwf.ic.gaussian_ic(p, seed=3)
    with mwf.Ensemble([p]) as a:
        a.set_state(0, c0)
        a.step(5)
        ref = a.get_state(0)
    with mwf.Ensemble([p], tune=True) as b:
        assert (tmp_path / "tune.json").exists()
        b.set_state(0, c0)
        b.step(5)
        got = b.get_state(0)
    # tiles do not change the arithmetic; a different radix plan changes rounding only
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
