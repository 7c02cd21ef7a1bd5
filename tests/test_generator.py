"""The product's analytic coupling generator against the oracle's quadrature (CPU)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import galerkin

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "mwf_gb300", "csrc")
sys.path.insert(0, CSRC)
import gen_nl  # noqa: E402


def _arr(d, shape, off):
    a = np.zeros(shape)
    for (k, i, j), c in d.items():
        a[k - off[0], i - off[1], j - off[2]] = float(c)
    return a


@pytest.mark.parametrize("K0", [4, 6])
def test_exact_tensors_match_quadrature(K0):
    Gp, Gv, Hp, Hv = gen_nl.tensors(K0)
    oGp, oGv, oHp, oHv, _ = galerkin.tensors(K0)
    b = np.pi / 2
    assert np.abs(_arr(Gp, oGp.shape, (0, 0, 0)) - oGp).max() < 1e-13
    assert np.abs(_arr(Gv, oGv.shape, (1, 0, 1)) - oGv).max() < 1e-13
    assert np.abs(_arr(Hp, oHp.shape, (0, 1, 0)) * b - oHp).max() < 1e-12
    assert np.abs(_arr(Hv, oHv.shape, (1, 1, 1)) * b - oHv).max() < 1e-12


def test_generated_header_is_current():
    out = subprocess.run([sys.executable, os.path.join(CSRC, "gen_nl.py")], capture_output=True, text=True,
                         check=True).stdout
    with open(os.path.join(CSRC, "nl_gen.cuh")) as f:
        assert f.read() == out
