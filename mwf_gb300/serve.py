"""Continuous-batching server for MWF run requests on one GPU.

A request asks for one simulation: model (K0), grid, Re, number of steps, precision and initial
condition (a seed, or a state of its own).  The server keeps every admitted run's state on the
device and advances runs in chunks of ``chunk`` steps (the reference's energy cadence,
i_save_rate2 = 50):

* batching: the requests admitted together form a *cohort* -- one C-ABI handle holding runs of
  different sizes, models and precisions, advanced by one CUDA-graph replay per step on the
  handle's own stream.  Cohorts run concurrently on the device;
* an event loop (``poll``): a cohort whose chunk has finished (``mwf_query``, no waiting) is
  processed on its own -- energies streamed back, finished runs retired inside the cohort
  (``mwf_set_active``), a run whose state is no longer finite marked failed and switched off
  while the others continue -- and its next chunk is launched at once; requests are admitted
  as soon as memory frees, without waiting for the other cohorts;
* admission: FIFO while the device footprint of the admitted work (``footprint_bytes``) stays
  within the HBM budget.  A cohort's memory is released when its last run ends; when the queue
  head does not fit, cohorts whose runs have mostly retired are compacted: their live runs are
  checkpointed exactly (state, AB2 history, Euler flag) to the host, the cohort is freed, and
  the runs are restored into the next cohort, where they continue bitwise as before.

Latency = completion time - arrival time.  Each run's arithmetic does not depend on the other
runs of its cohort (the kernels of one run never read another run's data), so a result is the
same alone, in the mix, and after a compaction.  A failed run stops the reference's way
(io_write_energy stops a run whose energy leaves the valid range, io.f90:462-465) without
stopping the server.
"""
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import ic
from ._lib import MwfError
from .solver import Ensemble, RunParams, footprint_bytes, round_23

MWF_ERR_NONFINITE = -6


@dataclass
class Request:
    rid: int
    params: RunParams
    steps: int
    seed: int = 0
    arrival: float = 0.0
    ic_kind: str = "gauss"          # "gauss", "spot", or "given" (state below)
    state: np.ndarray = None


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
    status: str = "running"         # "running", "done", or "failed: <why>"
    done_steps: int = 0

    @property
    def latency(self):
        return self.finished - self.arrival


def initial_state(r):
    if r.ic_kind == "given":
        return r.state
    if r.ic_kind == "spot":
        return ic.spot_ic(r.params, r.seed)
    return ic.gaussian_ic(r.params, r.seed)


class _Cohort:
    """One handle and the bookkeeping of its runs.  entries: (request, steps done, checkpoint or
    None)."""

    def __init__(self, entries, backend, device):
        self.reqs = [e[0] for e in entries]
        self.ens = backend([r.params for r in self.reqs], device=device)
        self.done_steps = [e[1] for e in entries]
        self.live = [True] * len(self.reqs)
        self.run_bytes = [footprint_bytes([r.params]) for r in self.reqs]
        self.bytes = footprint_bytes([r.params for r in self.reqs])
        self.inflight = 0               # steps launched and not yet accounted
        for i, (r, _, ckpt) in enumerate(entries):
            if ckpt is not None:
                self.ens.restore(i, ckpt)
            else:
                self.ens.set_state(i, initial_state(r))

    def remaining(self):
        return [r.steps - d if live else 0 for r, d, live in zip(self.reqs, self.done_steps, self.live)]

    def live_bytes(self):
        return sum(b for b, live in zip(self.run_bytes, self.live) if live)


class Server:
    """Single-GPU continuous-batching loop (see the module docstring)."""

    def __init__(self, budget_bytes=150 * 2 ** 30, chunk=50, device=0, keep_states=False,
                 backend=Ensemble, clock=time.perf_counter, compact_below=0.5, admit_interval=0.0):
        self.budget = int(budget_bytes)
        self.chunk = int(chunk)
        self.device = device
        self.keep_states = keep_states
        self.backend = backend
        self.clock = clock
        self.compact_below = compact_below
        # seconds between admissions while runs are in flight: arrivals in between join one cohort
        self.admit_interval = admit_interval
        self._last_admit = -math.inf
        self.queue = []            # FIFO of waiting requests
        self.resume = []           # checkpointed runs of compacted cohorts: (request, done, ckpt)
        self.cohorts = []
        self.results = {}
        self.dof_steps = 0
        self.in_use = 0
        self.compactions = 0

    # -- admission ----------------------------------------------------------------------
    def submit(self, req):
        b = footprint_bytes([req.params])
        if b < 0:
            raise ValueError(f"request {req.rid}: unsupported run {req.params}")
        if b > self.budget:
            raise ValueError(f"request {req.rid} needs {b} bytes, more than the whole budget")
        self.queue.append(req)

    def _compact(self, need):
        """Checkpoint the live runs of idle cohorts whose live share of memory is at most
        compact_below to the host and free those cohorts, most reclaimable first, until `need`
        more bytes are free."""
        cands = [co for co in self.cohorts if not co.inflight and co.live_bytes() <= self.compact_below * co.bytes]
        cands.sort(key=lambda co: co.bytes - co.live_bytes(), reverse=True)
        for co in cands:
            if self.budget - self.in_use >= need:
                break
            for i, r in enumerate(co.reqs):
                if co.live[i]:
                    self.resume.append((r, co.done_steps[i], co.ens.checkpoint(i)))
            co.ens.close()
            self.in_use -= co.bytes
            self.cohorts.remove(co)
            self.compactions += 1

    def _admit(self, now):
        """Admit resumed runs first, then the FIFO queue, while they fit; compact first if the
        next one does not fit."""
        if self.resume:
            head = self.resume[0][0]
        elif self.queue:
            head = self.queue[0]
        else:
            return 0
        free = self.budget - self.in_use
        if footprint_bytes([head.params]) > free:
            self._compact(footprint_bytes([head.params]))
            free = self.budget - self.in_use
        entries, need = [], 0
        while self.resume and need + footprint_bytes([self.resume[0][0].params]) <= free:
            e = self.resume.pop(0)
            entries.append(e)
            need += footprint_bytes([e[0].params])
        if not self.resume:
            while self.queue and need + footprint_bytes([self.queue[0].params]) <= free:
                r = self.queue.pop(0)
                entries.append((r, 0, None))
                need += footprint_bytes([r.params])
                self.results[r.rid] = Result(r.rid, r.arrival, now, math.nan, r.steps, r.params.dof)
        if not entries:
            return 0
        co = _Cohort(entries, self.backend, self.device)
        self.cohorts.append(co)
        self.in_use += co.bytes
        return len(entries)

    # -- the event loop -------------------------------------------------------------------
    def _finish_chunk(self, co):
        n = co.inflight
        co.inflight = 0
        co.ens.synchronize()
        t = self.clock()
        for i, r in enumerate(co.reqs):
            if not co.live[i]:
                continue
            co.done_steps[i] += n
            self.dof_steps += r.params.dof * n
            res = self.results[r.rid]
            res.done_steps = co.done_steps[i]
            try:
                res.energies.append((co.done_steps[i], co.ens.energy(i)))
            except MwfError as e:
                if e.code != MWF_ERR_NONFINITE:
                    raise
                co.live[i] = False
                co.ens.set_active(i, False)
                res.status = f"failed: non-finite state after {co.done_steps[i]} steps"
                res.finished = t
                continue
            if co.done_steps[i] >= r.steps:
                co.live[i] = False
                co.ens.set_active(i, False)
                res.status = "done"
                res.finished = t
                if self.keep_states:
                    res.state = co.ens.get_state(i)

    def _launch(self, co):
        rem = [x for x in co.remaining() if x > 0]
        if rem and not co.inflight:
            n = min(self.chunk, min(rem))
            co.ens.step_async(n)
            co.inflight = n

    def poll(self):
        """One pass of the loop: account every finished chunk, free empty cohorts, admit, and
        launch the next chunk of every idle cohort.  Returns True if anything progressed."""
        progressed = False
        for co in list(self.cohorts):
            if co.inflight and co.ens.query():
                self._finish_chunk(co)
                progressed = True
        for co in list(self.cohorts):
            if not any(co.live) and not co.inflight:
                co.ens.close()
                self.in_use -= co.bytes
                self.cohorts.remove(co)
        now = self.clock()
        if not self.cohorts or now - self._last_admit >= self.admit_interval:
            if self._admit(now):
                self._last_admit = now
                progressed = True
        for co in self.cohorts:
            if not co.inflight:
                self._launch(co)
                progressed = True
        return progressed

    def tick(self):
        """poll() until at least one chunk has been accounted (or nothing is running)."""
        while True:
            before = self.dof_steps
            self.poll()
            if self.dof_steps != before or not self.cohorts:
                return self.dof_steps - before
            time.sleep(2e-4)

    def busy(self):
        return bool(self.queue or self.resume or self.cohorts)

    # -- trace driver -------------------------------------------------------------------
    def run_trace(self, trace, max_wall=None):
        """Feed requests at their arrival times (seconds from start) and run until done (or
        until max_wall seconds have passed)."""
        pending = sorted(trace, key=lambda r: r.arrival)
        t0 = self.clock()
        k = 0
        self.offered_dof_steps = 0
        while k < len(pending) or self.busy():
            now = self.clock() - t0
            while k < len(pending) and pending[k].arrival <= now:
                r = pending[k]
                r.arrival = t0 + r.arrival
                self.submit(r)
                self.offered_dof_steps += r.params.dof * r.steps
                k += 1
            if not self.busy():
                time.sleep(min(0.001, max(0.0, pending[k].arrival - now)))
                continue
            if not self.poll():
                time.sleep(2e-4)
            if max_wall is not None and self.clock() - t0 > max_wall:
                break
        wall = self.clock() - t0
        return self.summary(wall)

    def summary(self, wall):
        done = [r for r in self.results.values() if r.status == "done"]
        lat = np.array([r.latency for r in done])
        return {
            "completed": len(done),
            "failed": sum(1 for r in self.results.values() if r.status.startswith("failed")),
            "submitted": len(self.results) + len(self.queue),
            "waiting": len(self.queue) + len(self.resume),
            "p50_latency_s": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if lat.size else None,
            "dof_steps_per_s": self.dof_steps / wall if wall > 0 else None,
            "compactions": self.compactions,
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
