"""mwf_step_noalloc: the time step for callers that cannot allocate device memory.

Host codes that own all of their device buffers (CUDA Fortran or OpenACC arrays, a pool they
manage) or that may not grow their device footprint after start-up cannot let the library
cudaMalloc its own state.  This entry point takes the state in the caller's device arrays and
keeps its intermediates in one fixed file-scope device array.  Its results must equal those of
the allocating entry point (mwf_create + mwf_step) and stay on the FP64 oracle, call after call.
This file is collected last so that a stop-at-first-failure run has already run the rest.
"""
import ctypes

import numpy as np
import pytest

import mwf_gb300 as mwf
from mwf_gb300 import _lib
from oracle import mwf_oracle as O

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _oracle(p, c0):
    op = O.Params(K0=p.K0, MM=p.MM, NN=p.NN, alpha=p.alpha, gamma=p.gamma, Re=p.Re, dt=p.dt,
                  drag=p.drag, vdrag=p.vdrag, hypo=p.hypo, dragall=p.dragall, theta=p.theta)
    return O.Solver(op, c0)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


class DeviceState:
    """Caller-owned device arrays in the reference layout: Re/Im of the state and of the AB2
    history, K*M*NN doubles each."""

    def __init__(self, torch, p, c, onl=None):
        def dev(a):
            return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
        self.c_re, self.c_im = dev(c.real), dev(c.imag)
        onl = np.zeros_like(c) if onl is None else onl
        self.o_re, self.o_im = dev(onl.real), dev(onl.imag)
        self.desc = p.to_c()

    def step(self, lib, first_step, nsteps):
        return lib.mwf_step_noalloc(ctypes.byref(self.desc), self.c_re.data_ptr(), self.c_im.data_ptr(),
                                    self.o_re.data_ptr(), self.o_im.data_ptr(), int(first_step), int(nsteps))

    def state(self):
        return self.c_re.cpu().numpy() + 1j * self.c_im.cpu().numpy()

    def history(self):
        return self.o_re.cpu().numpy() + 1j * self.o_im.cpu().numpy()


def test_noalloc_fp64_two_calls(built_lib):
    """cfg0 grid (M4, 96^2 modes, 144^2 grid, Re 200, dt 0.02): a first call with the Euler
    start, then a call that continues from the history the first one left, against the
    oracle (<= 1e-12) and against mwf_step on a handle (<= 1e-12)."""
    torch = _torch()
    lib = _lib.load()
    p = mwf.RunParams(K0=4, MM=48, NN=48, alpha=1 / 16, gamma=1 / 16, Re=200.0, dt=0.02)
    c0 = mwf.ic.gaussian_ic(p, seed=7)
    s = _oracle(p, c0)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(1)
        alloc1 = ens.get_state(0)
        ens.step(1)
        alloc2 = ens.get_state(0)
    st = DeviceState(torch, p, c0)
    _lib.check(st.step(lib, 1, 1))
    got1 = st.state()
    s.step(1)
    assert rel(got1, s.c) <= 1e-12, rel(got1, s.c)
    assert rel(got1, alloc1) <= 1e-12, rel(got1, alloc1)
    _lib.check(st.step(lib, 0, 1))
    got2 = st.state()
    s.step(1)
    assert rel(got2, s.c) <= 1e-12, rel(got2, s.c)
    assert rel(got2, alloc2) <= 1e-12, rel(got2, alloc2)
    assert rel(st.history(), s.onl) <= 1e-12


def test_noalloc_fp32_two_calls_100_steps(built_lib):
    """FP32 run of the same case: two calls of 50 steps (Euler start, then continued), against
    mwf_step on a handle after each call (<= 1e-5: the same FP32 arithmetic) and against the
    FP64 oracle after 100 steps at the FP32 bar (<= 1e-4 coefficients, <= 1 % energy)."""
    torch = _torch()
    lib = _lib.load()
    p = mwf.RunParams(K0=4, MM=48, NN=48, alpha=1 / 16, gamma=1 / 16, Re=200.0, dt=0.02, precision="fp32")
    c0 = mwf.ic.gaussian_ic(p, seed=11)
    with mwf.Ensemble([p]) as ens:
        ens.set_state(0, c0)
        ens.step(50)
        alloc50 = ens.get_state(0)
        ens.step(50)
        alloc100 = ens.get_state(0)
    st = DeviceState(torch, p, c0)
    _lib.check(st.step(lib, 1, 50))
    got50 = st.state()
    assert rel(got50, alloc50) <= 1e-5, rel(got50, alloc50)
    _lib.check(st.step(lib, 0, 50))
    got100 = st.state()
    assert rel(got100, alloc100) <= 1e-5, rel(got100, alloc100)
    s = _oracle(p.with_(precision="fp64"), c0)
    s.step(100)
    assert rel(got100, s.c) <= 1e-4, rel(got100, s.c)
    op = s.p
    e32, e64 = O.energy(op, got100), s.energy()
    assert abs(e32 - e64) <= 1e-2 * abs(e64), (e32, e64)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_noalloc_continues_from_given_history(built_lib, prec, tol):
    """first_step = 0 with a history the caller supplies: three oracle steps of an M6 run give
    (c, onl); one more call must match the oracle's fourth step."""
    torch = _torch()
    lib = _lib.load()
    p = mwf.RunParams(K0=6, MM=16, NN=24, alpha=2 * np.pi / 12, gamma=2 * np.pi / 8, Re=300.0, dt=0.01,
                      precision=prec)
    c0 = mwf.ic.gaussian_ic(p, seed=3, kmax=6)
    s = _oracle(p.with_(precision="fp64"), c0)
    s.step(3)
    st = DeviceState(torch, p, s.c, s.onl)
    s.step(1)
    _lib.check(st.step(lib, 0, 1))
    got = st.state()
    assert rel(got, s.c) <= tol, rel(got, s.c)
    assert rel(st.history(), s.onl) <= tol


def test_noalloc_zero_steps_and_rejections(built_lib):
    torch = _torch()
    lib = _lib.load()
    p = mwf.RunParams(K0=4, MM=16, NN=16)
    c0 = mwf.ic.gaussian_ic(p, seed=5, kmax=6)
    st = DeviceState(torch, p, c0)
    _lib.check(st.step(lib, 1, 0))
    assert np.array_equal(st.state(), c0)
    # symmetry masks are not supported by this entry point
    bad = DeviceState(torch, p.with_(reflect=True), c0)
    assert bad.step(lib, 1, 1) == -1
    assert np.array_equal(bad.state(), c0)
    # a run whose intermediates exceed the fixed array is rejected before any work
    big = mwf.RunParams(K0=4, MM=256, NN=256)
    n = big.dof
    bufs = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(4)]
    desc = big.to_c()
    rc = lib.mwf_step_noalloc(ctypes.byref(desc), *[b.data_ptr() for b in bufs], 1, 1)
    assert rc == -2, rc
    assert "scratch" in _lib.last_error()
