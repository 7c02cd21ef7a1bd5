"""mwf_step_noalloc: the time step for callers that cannot allocate device memory.

Host codes that own all of their device buffers (CUDA Fortran or OpenACC arrays, their own
pool) cannot let the library cudaMalloc state.  The entry point takes the state in the
caller's device arrays and keeps its intermediates in a fixed file-scope device array.
This file is collected last so that a stop-at-first-failure run has already run the rest.
"""
import ctypes

import numpy as np
import pytest

import mwf_gb300 as mwf
from mwf_gb300 import _lib

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def test_noalloc_matches_ensemble_two_calls(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    p = mwf.RunParams(K0=4, MM=48, NN=48, alpha=1 / 16, gamma=1 / 16, Re=200.0, dt=0.02)
    c0 = mwf.ic.gaussian_ic(p, seed=7)
    # existing entry point
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(1)
        ref1 = ens.get_state(0)
        ens.step(1)
        ref2 = ens.get_state(0)
    # no-allocation entry point on caller-owned device arrays (reference layout)
    c_re, c_im = _dev(torch, c0.real), _dev(torch, c0.imag)
    o_re, o_im = torch.zeros_like(c_re), torch.zeros_like(c_im)
    desc = p.to_c()
    args = [ctypes.byref(desc), c_re.data_ptr(), c_im.data_ptr(), o_re.data_ptr(), o_im.data_ptr()]
    _lib.check(lib.mwf_step_noalloc(*args, 1, 1))
    got1 = c_re.cpu().numpy() + 1j * c_im.cpu().numpy()
    _lib.check(lib.mwf_step_noalloc(*args, 0, 1))
    got2 = c_re.cpu().numpy() + 1j * c_im.cpu().numpy()
    for got, ref in ((got1, ref1), (got2, ref2)):
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err <= 1e-12, err


def test_noalloc_rejects_oversized_run(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    p = mwf.RunParams(K0=4, MM=256, NN=256)
    n = p.dof
    bufs = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(4)]
    desc = p.to_c()
    rc = lib.mwf_step_noalloc(ctypes.byref(desc), *[b.data_ptr() for b in bufs], 1, 1)
    assert rc == -2, rc
    assert "scratch" in _lib.last_error()
