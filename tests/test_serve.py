"""Continuous-batching server: admission and retirement logic (CPU, fake device backend) and
the same-alone-and-in-the-mix property on the GPU."""
import numpy as np
import pytest

import mwf_gb300 as mwf
from mwf_gb300 import serve


class FakeEnsemble:
    """Stand-in for the C-ABI handle: counts steps per active run."""
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

    def synchronize(self):
        for i in range(len(self.runs)):
            if self.active[i]:
                self.steps[i] += self.pending
        self.pending = 0

    def energy(self, i):
        return float(self.steps[i])

    def set_active(self, i, a):
        self.active[i] = a

    def get_state(self, i):
        return np.zeros(self.runs[i].shape, complex)

    def close(self):
        self.closed = True


def small(K0, n, **kw):
    return mwf.RunParams.square(K0, n, n * np.pi / 3, **kw)


def test_admission_respects_budget_and_retires():
    FakeEnsemble.created.clear()
    reqs = [serve.Request(i, small(4, 64), steps=120 + 30 * i, seed=i) for i in range(6)]
    one = mwf.footprint_bytes([reqs[0].params])
    srv = serve.Server(budget_bytes=int(2.5 * one), chunk=50, backend=FakeEnsemble)
    for r in reqs:
        srv.submit(r)
    peak = 0
    while srv.busy():
        srv.tick()
        peak = max(peak, srv.in_use)
        assert srv.in_use <= srv.budget
    assert peak > 0
    assert all(e.closed for e in FakeEnsemble.created)
    for r in reqs:
        res = srv.results[r.rid]
        assert res.energies[-1][0] == r.steps          # stepped exactly its steps
        assert res.finished >= res.admitted
    assert srv.dof_steps == sum(r.params.dof * r.steps for r in reqs)
    # FIFO: admission times are non-decreasing in submission order
    adm = [srv.admitted_at[r.rid] for r in reqs]
    assert adm == sorted(adm)


def test_oversized_request_is_rejected():
    srv = serve.Server(budget_bytes=1000, backend=FakeEnsemble)
    srv.submit(serve.Request(0, small(4, 64), steps=10))
    with pytest.raises(ValueError):
        srv.tick()


def test_poisson_trace_shapes():
    tr = serve.poisson_trace(rate=20, duration=5, seed=1)
    assert 50 <= len(tr) <= 160
    assert all(mwf.is_23_smooth(r.params.MM) for r in tr)
    assert all(500 <= r.steps <= 20000 for r in tr)
    k0 = np.array([r.params.K0 for r in tr])
    assert 0.4 < np.mean(k0 == 4) < 0.95


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix(built_lib):
    reqs = [serve.Request(0, small(4, 64, Re=200, dt=0.02), steps=130, seed=1, arrival=0.0),
            serve.Request(1, small(6, 48, Re=300, dt=0.01), steps=70, seed=2, arrival=0.0),
            serve.Request(2, small(4, 96, Re=250, dt=0.02, precision="fp32"), steps=160, seed=3, arrival=0.05),
            serve.Request(3, small(6, 64, Re=180, dt=0.01, precision="fp32"), steps=90, seed=4, arrival=0.1),
            serve.Request(4, small(4, 128, Re=300, dt=0.02), steps=60, seed=5, arrival=0.12)]
    alone = {}
    for r in reqs:
        with mwf.Ensemble([r.params]) as e:
            e.set_state(0, mwf.ic.gaussian_ic(r.params, r.seed))
            e.step(r.steps)
            alone[r.rid] = e.get_state(0)
    srv = serve.Server(budget_bytes=2 * 2 ** 30, chunk=50, keep_states=True)
    summ = srv.run_trace(reqs)
    assert summ["completed"] == len(reqs)
    assert summ["p99_latency_s"] >= summ["p50_latency_s"] > 0
    for r in reqs:
        got = srv.results[r.rid].state
        assert np.all(np.isfinite(got))
        assert np.array_equal(got, alone[r.rid]), r.rid
