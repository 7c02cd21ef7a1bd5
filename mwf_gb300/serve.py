"""Continuous-batching server for MWF run requests on one GPU.

A request asks for one simulation: model (K0), grid, Re, number of steps, precision and IC
seed.  The server keeps every admitted run's state on the device and advances all of them in
chunks of ``chunk`` steps (the reference's energy cadence, i_save_rate2 = 50):

* admission: requests wait in FIFO order and are admitted while the device footprint of the
  admitted work (``footprint_bytes``) stays within the HBM budget;
* batching: the requests admitted at one scheduling tick form a *cohort* -- one C-ABI handle
  holding runs of different sizes, models and precisions, advanced by one CUDA-graph replay
  per step on the handle's own stream.  All live cohorts are launched asynchronously before
  the server waits on any of them, so their kernels overlap on the device;
* retirement: a run that has done its steps is switched off inside its cohort
  (``mwf_set_active``) and its final state is copied out; a cohort's memory is released when
  its last run finishes;
* diagnostics: the perturbation energy of every live run is streamed back after each chunk.

Latency = completion time - arrival time.  Each run's arithmetic does not depend on the other
runs of its cohort (the kernels of one run never read another run's data), so a result is the
same alone and in the mix.
"""
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import ic
from .solver import Ensemble, RunParams, footprint_bytes, round_23


@dataclass
class Request:
    rid: int
    params: RunParams
    steps: int
    seed: int = 0
    arrival: float = 0.0
    ic_kind: str = "gauss"


@dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    finished: float
    steps: int
    dof: int
    energies: list = field(default_factory=list)
    state: np.ndarray = None

    @property
    def latency(self):
        return self.finished - self.arrival


class _Cohort:
    def __init__(self, reqs, backend, device):
        self.reqs = list(reqs)
        self.ens = backend([r.params for r in self.reqs], device=device)
        self.done_steps = [0] * len(self.reqs)
        self.live = [True] * len(self.reqs)
        self.bytes = footprint_bytes([r.params for r in self.reqs])
        for i, r in enumerate(self.reqs):
            c0 = ic.spot_ic(r.params, r.seed) if r.ic_kind == "spot" else ic.gaussian_ic(r.params, r.seed)
            self.ens.set_state(i, c0)

    def remaining(self):
        return [r.steps - d if live else 0 for r, d, live in zip(self.reqs, self.done_steps, self.live)]


class Server:
    """Single-GPU continuous-batching loop (see the module docstring)."""

    def __init__(self, budget_bytes=150 * 2 ** 30, chunk=50, device=0, keep_states=False,
                 backend=Ensemble, clock=time.perf_counter):
        self.budget = int(budget_bytes)
        self.chunk = int(chunk)
        self.device = device
        self.keep_states = keep_states
        self.backend = backend
        self.clock = clock
        self.queue = []            # FIFO of waiting requests
        self.cohorts = []
        self.results = {}
        self.admitted_at = {}
        self.dof_steps = 0
        self.in_use = 0

    # -- admission ----------------------------------------------------------------------
    def submit(self, req):
        self.queue.append(req)

    def _admit(self, now):
        batch, need = [], 0
        while self.queue:
            r = self.queue[0]
            b = footprint_bytes([r.params])
            if b < 0:
                raise ValueError(f"request {r.rid}: unsupported run {r.params}")
            if b > self.budget:
                raise ValueError(f"request {r.rid} needs {b} bytes, more than the whole budget")
            if self.in_use + need + b > self.budget:
                break
            batch.append(self.queue.pop(0))
            need += b
        if batch:
            co = _Cohort(batch, self.backend, self.device)
            self.cohorts.append(co)
            self.in_use += co.bytes
            for r in batch:
                self.admitted_at[r.rid] = now
                self.results[r.rid] = Result(r.rid, r.arrival, now, math.nan, r.steps, r.params.dof)
        return len(batch)

    # -- one scheduling tick --------------------------------------------------------------
    def tick(self):
        now = self.clock()
        self._admit(now)
        if not self.cohorts:
            return 0
        plans = []
        for co in self.cohorts:
            rem = [x for x in co.remaining() if x > 0]
            n = min(self.chunk, min(rem)) if rem else 0
            plans.append(n)
            if n:
                co.ens.step_async(n)           # all cohorts in flight before any wait
        for co, n in zip(self.cohorts, plans):
            if not n:
                continue
            co.ens.synchronize()
            for i, r in enumerate(co.reqs):
                if not co.live[i]:
                    continue
                co.done_steps[i] += n
                self.dof_steps += r.params.dof * n
                res = self.results[r.rid]
                res.energies.append((co.done_steps[i], co.ens.energy(i)))
        t = self.clock()
        for co in self.cohorts:
            for i, r in enumerate(co.reqs):
                if co.live[i] and co.done_steps[i] >= r.steps:
                    co.live[i] = False
                    co.ens.set_active(i, False)
                    res = self.results[r.rid]
                    res.finished = t
                    if self.keep_states:
                        res.state = co.ens.get_state(i)
        keep = []
        for co in self.cohorts:
            if any(co.live):
                keep.append(co)
            else:
                co.ens.close()
                self.in_use -= co.bytes
        self.cohorts = keep
        return sum(plans)

    def busy(self):
        return bool(self.queue or self.cohorts)

    # -- trace driver -------------------------------------------------------------------
    def run_trace(self, trace, max_wall=None):
        """Feed requests at their arrival times (seconds from start) and run until done."""
        pending = sorted(trace, key=lambda r: r.arrival)
        t0 = self.clock()
        k = 0
        while k < len(pending) or self.busy():
            now = self.clock() - t0
            while k < len(pending) and pending[k].arrival <= now:
                r = pending[k]
                r.arrival = t0 + r.arrival
                self.submit(r)
                k += 1
            if not self.busy():
                time.sleep(min(0.001, max(0.0, pending[k].arrival - now)))
                continue
            self.tick()
            if max_wall is not None and self.clock() - t0 > max_wall:
                break
        wall = self.clock() - t0
        return self.summary(wall)

    def summary(self, wall):
        lat = np.array([r.latency for r in self.results.values() if not math.isnan(r.finished)])
        return {
            "completed": int(lat.size),
            "submitted": len(self.results) + len(self.queue),
            "p50_latency_s": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if lat.size else None,
            "dof_steps_per_s": self.dof_steps / wall if wall > 0 else None,
            "wall_s": wall,
        }


def poisson_trace(rate, duration, seed=0, steps_range=(500, 20000), n_range=(64, 512),
                  m4_frac=0.7, fp32_frac=0.8, re_range=(150.0, 400.0)):
    """Requests arriving as a Poisson process: model M4/M6, N x N modes log-uniform in n_range
    (rounded to 2^a 3^b, domain L = N pi / 3), Re uniform, steps log-uniform, FP32/FP64."""
    rng = np.random.default_rng(seed)
    t, rid, out = 0.0, 0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        K0 = 4 if rng.random() < m4_frac else 6
        n = round_23(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1]))))
        n = max(4, 2 * (round_23(n // 2)))
        L = n * math.pi / 3.0
        prec = "fp32" if rng.random() < fp32_frac else "fp64"
        if K0 == 6 and prec == "fp64":
            n = min(n, 1024)
        p = RunParams.square(K0, n, L, Re=float(rng.uniform(*re_range)), dt=0.02 if K0 == 4 else 0.01,
                             precision=prec)
        steps = int(round(math.exp(rng.uniform(math.log(steps_range[0]), math.log(steps_range[1])))))
        out.append(Request(rid, p, steps, seed=rid, arrival=t))
        rid += 1
    return out
