"""Continuous-batching server: admission, retirement, failure isolation and compaction logic (CPU,
fake device backend), and on the GPU: each result is the same alone and in the mix, a run whose
state turns non-finite fails alone, and a compacted run continues bitwise."""
import numpy as np
import pytest

import mwf_gb300 as mwf
from mwf_gb300 import serve
from mwf_gb300._lib import MwfError


class FakeEnsemble:
    """Stand-in for the C-ABI handle: counts steps per active run; a run whose params have
    Re < 0 reports a non-finite state once it has stepped."""
    created = []

    def __init__(self, runs, device=0):
        self.runs = runs
        self.steps = [0] * len(runs)
        self.active = [True] * len(runs)
        self.pending = 0
        self.closed = False
        FakeEnsemble.created.append(self)

    def set_state(self, i, c):
        assert c.shape == self.runs[i].shape

    def step_async(self, n):
        self.pending = n

    def query(self):
        return True

    def synchronize(self):
        for i in range(len(self.runs)):
            if self.active[i]:
                self.steps[i] += self.pending
        self.pending = 0

    def energy(self, i):
        if self.runs[i].Re < 0 and self.steps[i] > 0:
            raise MwfError(-6, f"run {i}: state contains NaN/Inf")
        return float(self.steps[i])

    def set_active(self, i, a):
        self.active[i] = a

    def get_state(self, i):
        return np.zeros(self.runs[i].shape, complex)

    def checkpoint(self, i):
        return ("ckpt", self.steps[i])

    def restore(self, i, ckpt):
        self.steps[i] = ckpt[1]

    def close(self):
        self.closed = True


def small(K0, n, **kw):
    return mwf.RunParams.square(K0, n, n * np.pi / 3, **kw)


def drain(srv):
    peak = 0
    while srv.busy():
        srv.tick()
        peak = max(peak, srv.in_use)
        assert srv.in_use <= srv.budget
    return peak


def test_admission_respects_budget_and_retires():
    FakeEnsemble.created.clear()
    reqs = [serve.Request(i, small(4, 64), steps=120 + 30 * i, seed=i) for i in range(6)]
    one = mwf.footprint_bytes([reqs[0].params])
    srv = serve.Server(budget_bytes=int(2.5 * one), chunk=50, backend=FakeEnsemble)
    for r in reqs:
        srv.submit(r)
    assert drain(srv) > 0
    assert all(e.closed for e in FakeEnsemble.created)
    for r in reqs:
        res = srv.results[r.rid]
        assert res.status == "done"
        assert res.energies[-1][0] == r.steps          # stepped exactly its steps
        assert res.finished >= res.admitted
    assert srv.dof_steps == sum(r.params.dof * r.steps for r in reqs)
    # FIFO: admission times are non-decreasing in submission order
    adm = [srv.results[r.rid].admitted for r in reqs]
    assert adm == sorted(adm)


def test_oversized_request_is_rejected():
    srv = serve.Server(budget_bytes=1000, backend=FakeEnsemble)
    with pytest.raises(ValueError):
        srv.submit(serve.Request(0, small(4, 64), steps=10))


def test_nonfinite_run_fails_alone():
    """A run whose state is no longer finite is marked failed and switched off; the server and
    the other runs of its cohort carry on."""
    reqs = [serve.Request(0, small(4, 64), steps=200), serve.Request(1, small(4, 64, Re=-1.0), steps=200),
            serve.Request(2, small(4, 96), steps=120)]
    srv = serve.Server(budget_bytes=2 ** 34, chunk=50, backend=FakeEnsemble)
    for r in reqs:
        srv.submit(r)
    drain(srv)
    assert srv.results[1].status == "failed: non-finite state after 50 steps"
    assert srv.results[0].status == srv.results[2].status == "done"
    assert srv.results[0].energies[-1][0] == 200 and srv.results[2].energies[-1][0] == 120
    assert srv.summary(1.0)["failed"] == 1


def test_mostly_retired_cohort_is_compacted():
    """One cohort holds a long run and several short ones; once the short ones retire and a new
    request does not fit, the long run is checkpointed, its cohort freed, and it resumes in the
    next cohort with its step count intact."""
    FakeEnsemble.created.clear()
    p = small(4, 64)
    one = mwf.footprint_bytes([p])
    first = [serve.Request(0, p, steps=400)] + [serve.Request(i, p, steps=50) for i in range(1, 4)]
    srv = serve.Server(budget_bytes=int(4.5 * one), chunk=50, backend=FakeEnsemble)
    for r in first:
        srv.submit(r)
    srv.tick()                      # admits the four together, runs one chunk, retires the short ones
    late = [serve.Request(10 + i, p, steps=100) for i in range(3)]
    for r in late:
        srv.submit(r)
    drain(srv)
    assert srv.compactions >= 1
    assert srv.results[0].status == "done" and srv.results[0].energies[-1][0] == 400
    assert all(srv.results[r.rid].status == "done" for r in late)
    assert srv.dof_steps == sum(r.params.dof * r.steps for r in first + late)


def test_poisson_trace_shapes():
    tr = serve.poisson_trace(rate=20, duration=5, seed=1)
    assert 50 <= len(tr) <= 160
    assert all(mwf.is_23_smooth(r.params.MM) for r in tr)
    assert all(500 <= r.steps <= 20000 for r in tr)
    k0 = np.array([r.params.K0 for r in tr])
    assert 0.4 < np.mean(k0 == 4) < 0.95


def _alone(r):
    with mwf.Ensemble([r.params]) as e:
        e.set_state(0, serve.initial_state(r))
        e.step(r.steps)
        return e.get_state(0)


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix(built_lib):
    reqs = [serve.Request(0, small(4, 64, Re=200, dt=0.02), steps=130, seed=1, arrival=0.0),
            serve.Request(1, small(6, 48, Re=300, dt=0.01), steps=70, seed=2, arrival=0.0),
            serve.Request(2, small(4, 96, Re=250, dt=0.02, precision="fp32"), steps=160, seed=3, arrival=0.05),
            serve.Request(3, small(6, 64, Re=180, dt=0.01, precision="fp32"), steps=90, seed=4, arrival=0.1),
            serve.Request(4, small(4, 128, Re=300, dt=0.02), steps=60, seed=5, arrival=0.12)]
    alone = {r.rid: _alone(r) for r in reqs}
    srv = serve.Server(budget_bytes=2 * 2 ** 30, chunk=50, keep_states=True)
    summ = srv.run_trace(reqs)
    assert summ["completed"] == len(reqs)
    assert summ["p99_latency_s"] >= summ["p50_latency_s"] > 0
    for r in reqs:
        got = srv.results[r.rid].state
        assert np.all(np.isfinite(got))
        assert np.array_equal(got, alone[r.rid]), r.rid


@pytest.mark.gpu
def test_nan_run_fails_alone_in_a_mixed_cohort(built_lib):
    """A request whose initial state holds a NaN (set on the host through set_state) is admitted
    with three others into one cohort; it is marked failed after its first chunk and switched
    off, and the other three finish bitwise equal to their runs alone."""
    good = [serve.Request(0, small(4, 64, Re=200, dt=0.02), steps=120, seed=1),
            serve.Request(1, small(6, 48, Re=300, dt=0.01, precision="fp32"), steps=100, seed=2),
            serve.Request(2, small(4, 96, Re=250, dt=0.02, precision="fp32"), steps=150, seed=3)]
    bad_p = small(4, 64, Re=220, dt=0.02)
    c_bad = mwf.ic.gaussian_ic(bad_p, 9)
    c_bad[3, 5, 2] = np.nan
    bad = serve.Request(3, bad_p, steps=120, ic_kind="given", state=c_bad)
    alone = {r.rid: _alone(r) for r in good}
    srv = serve.Server(budget_bytes=2 * 2 ** 30, chunk=50, keep_states=True)
    for r in good + [bad]:
        srv.submit(r)
    srv.tick()
    assert len(srv.cohorts) == 1 and len(srv.cohorts[0].reqs) == 4
    while srv.busy():
        srv.tick()
    assert srv.results[3].status.startswith("failed: non-finite"), srv.results[3].status
    for r in good:
        assert srv.results[r.rid].status == "done"
        assert np.array_equal(srv.results[r.rid].state, alone[r.rid]), r.rid


@pytest.mark.gpu
def test_compacted_run_continues_bitwise(built_lib):
    """A long run outlives the short runs of its cohort; a request that does not fit forces a
    compaction (checkpoint to the host, cohort freed, restore into a new cohort); the long run's
    final state equals its run alone bitwise, in FP64 and in FP32."""
    for prec in ("fp64", "fp32"):
        p = small(4, 64, Re=230, dt=0.02, precision=prec)
        one = mwf.footprint_bytes([p])
        long_run = serve.Request(0, p, steps=230, seed=11)
        short = [serve.Request(i, p, steps=50, seed=11 + i) for i in range(1, 4)]
        late = serve.Request(10, p, steps=60, seed=20)
        srv = serve.Server(budget_bytes=int(4.5 * one), chunk=50, keep_states=True)
        for r in [long_run] + short:
            srv.submit(r)
        srv.tick()
        srv.submit(late)
        while srv.busy():
            srv.tick()
        assert srv.compactions >= 1
        assert np.array_equal(srv.results[0].state, _alone(long_run)), prec
        assert np.array_equal(srv.results[10].state, _alone(late)), prec
