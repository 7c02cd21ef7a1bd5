"""Failure detection in device code: the bounded wait of the staged FP32 z pass.

The staged z pass copies each task's input rows into shared memory with bulk copies that
complete on an mbarrier; every thread waits for the barrier's phase with a time limit, and a
copy that does not land sets an error flag instead of hanging the CTA.  The test makes that
wait run out on purpose (the barrier is armed with more bytes than the copies carry, and the
limit is shortened to 1 ms): the step must come back with MWF_ERR_DEVICE and the copy-timeout
flag, quickly, and a new handle in the same process must step correctly afterwards.
"""
import time

import numpy as np
import pytest

import mwf_gb300 as mwf
from mwf_gb300 import _lib
from oracle import mwf_oracle as O

pytestmark = pytest.mark.gpu


def test_bounded_copy_wait_runs_out(built_lib):
    lib = _lib.load()
    # a z radix cap selects the staged z pass (z_nonlinear_kernel) for this FP32 run
    p = mwf.RunParams(K0=4, MM=32, NN=32, alpha=1 / 8, gamma=1 / 8, Re=200.0, dt=0.02, precision="fp32",
                      z_radix=12)
    c0 = mwf.ic.gaussian_ic(p, seed=2, kmax=6)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        _lib.check(lib.mwf_test_copy_timeout(ens.handle, 0, 16, 1.0))
        t0 = time.perf_counter()
        with pytest.raises(mwf.MwfError) as ei:
            ens.step(1)
        elapsed = time.perf_counter() - t0
        assert ei.value.code == -5, ei.value
        assert "0x8" in str(ei.value), ei.value
        assert elapsed < 10.0, elapsed
    # the context stays usable: a new handle in the same process matches the oracle
    op = O.Params(K0=4, MM=32, NN=32, alpha=1 / 8, gamma=1 / 8, Re=200.0, dt=0.02)
    s = O.Solver(op, c0)
    s.step(2)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(2)
        g = ens.get_state(0)
    assert np.abs(g - s.c).max() / np.abs(s.c).max() <= 1e-5


def test_copy_timeout_arguments_are_checked(built_lib):
    lib = _lib.load()
    p = mwf.RunParams(K0=4, MM=16, NN=16, precision="fp32", z_radix=12)
    with mwf.Ensemble([p]) as ens:
        assert lib.mwf_test_copy_timeout(ens.handle, 0, 8, 1.0) == -1       # not a multiple of 16
        assert lib.mwf_test_copy_timeout(ens.handle, 0, 16, 5000.0) == -1   # limit above a second
        assert lib.mwf_test_copy_timeout(ens.handle, 1, 16, 1.0) == -1      # no run 1
        _lib.check(lib.mwf_test_copy_timeout(ens.handle, 0, 0, 0.0))        # normal operation
        ens.step(1)
