#!/usr/bin/env python
"""Throughput of the Model Waleffe Flow timestep on GB300, in dof-steps/s.

Default workload (one replica per GPU, runs shard across GPUs with no collective):
  M6 model, 1024 x 1024 Fourier modes (MM = NN = 512) on a 1536 x 1536 dealiased grid,
  Lx = Lz = 256 pi, Re = 300, dt = 0.01, plain FP64, seeded localized-spot initial
  condition (Gaussian spectrum |k| <= 8 times a width-20 Gaussian envelope).
A step is one vel_TS over that state (dof = 11 * 1023 * 512 complex MPT coefficients).

  value      dof-steps/s with the state resident on the device, CUDA events on the
             library's own stream around the graph launches, max over ranks
  e2e        the same metric through the C ABI with host buffers: every step copies the
             state in from pinned host memory, advances one step and copies it back
  roofline   the dominant pass (the z pass: z transforms + nonlinear term) against HBM,
             plus its FP64 arithmetic rate against the measured FP64 FMA peak
  cpu_baseline  the C++ FP64 / OpenMP restatement of the step (oracle/cpu_step.cpp) on
             a bounded sample of the same workload (about 10 s on all host cores, plus about
             6 s on one core; rank 0, N = 1)

  --impl reference   times that C++ restatement with all host cores (the Fortran reference
                     cannot be built here) on the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PI = 3.1415926535897931
HBM_FALLBACK_GBS = 6800.0


def workload_params(name):
    import mwf_gb300 as mwf
    if name == "m6-1024-fp64":
        p = mwf.RunParams.square(6, 1024, 256 * PI, Re=300.0, dt=0.01)
        return [p], "spot"
    if name == "m6-512-fp64":
        p = mwf.RunParams.square(6, 512, 128 * PI, Re=300.0, dt=0.01)
        return [p], "spot"
    if name == "m4-96-fp64":
        p = mwf.RunParams.square(4, 96, 32 * PI, Re=200.0, dt=0.02)
        return [p], "gauss"
    if name == "m4-2048-fp32":
        p = mwf.RunParams.square(4, 2048, 512 * PI, Re=250.0, dt=0.01, precision="fp32")
        return [p], "gauss16"
    if name in ("ensemble512-fp32", "ensemble64-fp32"):
        rng = np.random.default_rng(12345)
        sizes = [64, 96, 128, 192, 256]
        runs = []
        for i in range(512 if name == "ensemble512-fp32" else 64):
            n = int(rng.choice(sizes))
            L = n * PI / 3.0
            runs.append(mwf.RunParams.square(4, n, L, Re=float(rng.uniform(150, 350)), dt=0.02,
                                             precision="fp32"))
        return runs, "gauss"
    raise SystemExit(f"unknown workload {name}")


def initial_state(p, kind, seed):
    import mwf_gb300 as mwf
    if kind == "spot":
        return mwf.ic.spot_ic(p, seed)
    if kind == "gauss16":
        return mwf.ic.gaussian_ic(p, seed, kmax=16)
    return mwf.ic.gaussian_ic(p, seed)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.f is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        rows = [ln.strip().split(", ") for ln in open(self.f.name) if ln.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return HBM_FALLBACK_GBS, "fallback"


def zpass_alg(p):
    """Algorithmic bytes and flops of one z-pass launch for run p.

    bytes: read the x-transformed u and d/dx u (2KK fields of X*NN complex), write the
    z-transformed nonlinear term (KK fields of X*NN complex).
    flops: 2.5 * 4KK * X * Z * log2(Z) for the c2r of 3KK fields and the r2c of KK fields
    (real transforms of length Z), plus c_NL * X * Z for the pointwise coupling
    (c_NL = 369 for M4, 1043 for M6, counted from the reference's expressions).
    """
    cb = 16 if p.precision == "fp64" else 8
    nbytes = 3 * p.KK * p.X * p.NN * cb
    cnl = 369 if p.K0 == 4 else 1043
    flops = 2.5 * 4 * p.KK * p.X * p.Z * np.log2(p.Z) + cnl * p.X * p.Z
    return nbytes, flops


def step_alg_bytes(p):
    """B_alg per run-step: state traffic 4*K*M*NN plus the two transposes 6*KK*X*NN (complex)."""
    cb = 16 if p.precision == "fp64" else 8
    return cb * (4 * p.K * p.M * p.NN + 6 * p.KK * p.X * p.NN)


def config_dict(workload, runs, kind, world):
    """The `config` object of the JSON line, identical for both arms (same workload)."""
    p = runs[0]
    return {"workload": workload, "runs_per_gpu": len(runs), "dof_per_gpu": sum(q.dof for q in runs),
            "K0": p.K0, "MM": p.MM, "NN": p.NN, "grid": f"{p.X}x{p.Z}", "Re": p.Re, "dt": p.dt,
            "ic": kind, "l2": "inputs larger than L2 (step working set "
            f"{sum(step_alg_bytes(q) for q in runs) / 1e9:.2f} GB > 129 MB)",
            "parallelism": f"replicas x{world} (runs shard, no collective)"}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def allreduce_max(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


def cufft_transforms_ms(runs, device, reps=5):
    """Comparison only, not the product path: the transforms of one step done by cuFFT through
    torch.fft, batched the way a library-FFT implementation would call them (runs of one grid
    size in one batch): x c2c backward of the 2KK fields u, du/dx (NN lines of X), z c2r of the
    3KK fields u, du/dx, du/dz (X lines, Z points), z r2c of the KK products, x c2c forward of
    the KK fields.  Transforms alone -- no padding copies, nonlinear term or update -- so this
    is a lower bound for a cuFFT-based step.  Milliseconds per step, CUDA events on torch's
    current stream."""
    import torch
    dev = torch.device("cuda", device)
    groups = {}
    for p in runs:
        groups.setdefault((p.K0, p.MM, p.NN, p.precision), []).append(p)
    bufs = []
    for (K0, MM, NN, prec), ps in groups.items():
        p, c = ps[0], len(ps)
        dc = torch.complex128 if prec == "fp64" else torch.complex64
        dr = torch.float64 if prec == "fp64" else torch.float32
        bufs.append((p.Z,
                     torch.zeros(c * 2 * p.KK, NN, p.X, dtype=dc, device=dev),
                     torch.zeros(c * 3 * p.KK, p.X, p.Z // 2 + 1, dtype=dc, device=dev),
                     torch.zeros(c * p.KK, p.X, p.Z, dtype=dr, device=dev),
                     torch.zeros(c * p.KK, NN, p.X, dtype=dc, device=dev)))

    def step():      # unnormalised in both directions, as the step's transforms
        for Z, a, zin, zr, b in bufs:
            torch.fft.ifft(a, dim=-1, norm="forward")
            torch.fft.irfft(zin, n=Z, dim=-1, norm="forward")
            torch.fft.rfft(zr, dim=-1)
            torch.fft.fft(b, dim=-1)

    with torch.cuda.device(dev):
        step()
        step()
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            step()
        e1.record()
        e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    del bufs
    torch.cuda.empty_cache()
    return ms


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_port_solver(runs, kind, threads):
    """The C++ FP64 / OpenMP restatement of the step (oracle/cpu_step.cpp) on the first run of
    the workload: the CPU implementation of the path, since the Fortran reference (FFTW3,
    netCDF, MPI, a Fortran compiler) cannot be built on these machines."""
    from oracle import mwf_oracle as O
    from oracle import cpu_port
    p = runs[0]
    op = O.Params(K0=p.K0, MM=p.MM, NN=p.NN, alpha=p.alpha, gamma=p.gamma, Re=p.Re, dt=p.dt,
                  drag=p.drag, vdrag=p.vdrag, hypo=p.hypo, dragall=p.dragall, theta=p.theta)
    return p, cpu_port.CpuSolver(op, initial_state(p, kind, 0), threads=threads)


def cpu_port_rate_bounded(runs, kind, threads, budget_s, max_steps=500):
    """cpu_port_rate over as many steps as fit in about budget_s seconds (after one timed
    warm-up step that sizes the sample): (dof-steps/s, seconds, steps)."""
    p, s = cpu_port_solver(runs, kind, threads)
    t0 = time.perf_counter()
    s.step(1)
    t1 = time.perf_counter() - t0
    n = int(max(1, min(max_steps, budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    s.step(n)
    dt = time.perf_counter() - t0
    s.close()
    return p.dof * n / dt, dt, n


def cpu_port_rate(runs, kind, steps, threads, warmup=1):
    """dof-steps/s of the C++ restatement over `steps` steps (after `warmup`) of run 0."""
    p, s = cpu_port_solver(runs, kind, threads)
    s.step(warmup)
    t0 = time.perf_counter()
    s.step(steps)
    dt = time.perf_counter() - t0
    s.close()
    return p.dof * steps / dt, dt


def run_reference(args, world, rank, pg):
    runs, kind = workload_params(args.workload)
    if rank != 0:
        return
    threads = host_cores()
    # warm-up steps, then K timed steps of the C++ restatement on the first run of the workload
    p = runs[0]
    v, dt = cpu_port_rate(runs, kind, args.steps, threads, warmup=args.warmup)
    line = {
        "metric": "dof-steps/s", "value": v, "unit": "dof-steps/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args.workload, runs, kind, world),
        "cpu_baseline": {"value": v, "unit": "dof-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full steps of the workload's first run after "
                                   f"{args.warmup} warm-up steps: C++ FP64 restatement with OpenMP "
                                   "(oracle/cpu_step.cpp), not the reference binary, which does not "
                                   "build here (no Fortran compiler, FFTW3, netCDF)"},
        "e2e": {"value": v, "unit": "dof-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


PASS_NAMES = ["x_forward", "z_nonlinear", "x_inverse"]


def pass_alg_bytes(runs, i):
    """Algorithmic bytes of pass i over all runs: x forward reads c and writes T (2KK fields);
    z reads T and writes the KK nonlinear fields; x inverse reads those, c, onl and the
    tables and writes c and onl."""
    tot = 0
    for p in runs:
        cb = 16 if p.precision == "fp64" else 8
        if i == 0:
            tot += (2 * p.KK * p.X * p.NN + p.K * p.M * p.NN) * cb
        elif i == 1:
            tot += zpass_alg(p)[0]
        else:
            tot += (p.KK * p.X * p.NN + 4 * p.K * p.M * p.NN) * cb + 2 * p.K * p.M * p.NN * 8
    return tot


def measure_resident(ens, args, pg, world, dev):
    """Device-resident throughput of an Ensemble over K steps (CUDA events on the library's
    stream, max over ranks), with clocks sampled during the timed region, per-pass device
    times and the rooflines of the dominant pass."""
    runs = ens.runs
    dof = sum(p.dof for p in runs)
    ens.step(args.warmup)
    barrier(pg)
    with ClockSampler(dev) as clk:
        t_host0 = time.perf_counter()
        ms = ens.step_timed(args.steps)
        t_host = time.perf_counter() - t_host0
    ms = allreduce_max(pg, ms)
    barrier(pg)
    pass_ms = ens.profile_passes(3)
    dom = int(np.argmax(pass_ms))
    hbm, hbm_src = measured_peaks()
    achieved = pass_alg_bytes(runs, dom) / (pass_ms[dom] * 1e-3) / 1e9
    fp64 = all(p.precision == "fp64" for p in runs)
    peak_fma = mwf_solver().measure_fma_peak(dev, fp64=fp64)
    zf = sum(zpass_alg(p)[1] for p in runs)
    z_tflops = zf / (pass_ms[1] * 1e-3) / 1e12
    return {
        "value": world * dof * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
        "clocks": clk.summary(), "host_wall_s": t_host,
        "gpu_launches": ens.kernels_per_step() * args.steps,
        "pass_ms": dict(zip(PASS_NAMES, pass_ms)),
        "step_alg_bytes": sum(step_alg_bytes(p) for p in runs),
        "roofline": {"bound": "hbm", "kernel": PASS_NAMES[dom], "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                     "peak_source": f"{hbm_src} hbm_gbs"},
        "alu_roofline": {"kernel": "z_nonlinear", "achieved": z_tflops, "peak": peak_fma,
                         "unit": "TFLOP/s", "frac": z_tflops / peak_fma, "pipe": "fp64" if fp64 else "fp32",
                         "peak_source": "measured FMA-chain probe on this GPU"},
    }


def mwf_solver():
    from mwf_gb300 import solver
    return solver


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of the z pass per launch, from single-
# kernel ncu captures of smaller cases (profiles/z_nonlinear_fp64_m6_768sq.md,
# profiles/batched_dram_fp32_ensemble64.md) scaled by the points processed:
#  - FP64 M6: the 768^2 grid read 108.07 MB and wrote 129.06 MB; the 1536^2 grid has 4x the points;
#  - batched FP32 M4 z pass: DRAM read per run of MM = NN = 32, 48, 64, 96, 128 (the capture's
#    reads divided by its runs of each size; 0.2-1.1 % above the algorithmic read of T), plus the
#    algorithmic write KK X NN 8 B, which at the capture's size stays in L2.
ZPASS_TRAFFIC = {"m6-1024-fp64": 4 * (108.07e6 + 129.06e6)}
ZB_READ_PER_RUN = {32: 7115520 / 13, 48: 19553536 / 16, 64: 19536640 / 9, 96: 78002432 / 16, 128: 86641408 / 10}


def zpass_traffic_fp32(runs):
    """Estimated DRAM bytes of the batched FP32 z pass over these runs (None if a size was not captured)."""
    tot = 0.0
    for p in runs:
        if p.K0 != 4 or p.MM != p.NN or p.MM not in ZB_READ_PER_RUN:
            return None
        tot += ZB_READ_PER_RUN[p.MM] + p.KK * p.X * p.NN * 8
    return tot


def run_gpu(args, world, rank, local, pg):
    import mwf_gb300 as mwf
    from mwf_gb300 import build, _lib
    build.build()
    runs, kind = workload_params(args.workload)
    dev = local
    t_tune = time.perf_counter()
    ens = mwf.Ensemble(runs, device=dev, tune=not args.no_tune)   # autotuned tiles/radices
    t_tune = time.perf_counter() - t_tune
    if args.persistent:
        ens.set_persistent(True)
    runs = ens.runs
    for i, p in enumerate(runs):
        ens.set_state(i, initial_state(p, kind, 1000 * rank + i))
    res = measure_resident(ens, args, pg, world, dev)
    if res["roofline"]["kernel"] == "z_nonlinear":
        res["roofline"]["traffic"] = ZPASS_TRAFFIC.get(args.workload)
    # ---- end to end through the C ABI with host buffers ----
    e2e = None
    if len(runs) == 1:
        p = runs[0]
        lib = _lib.load()
        import ctypes
        nbytes = p.dof * 8
        ptrs = []
        arrs = []
        for _ in range(2):
            ptr = ctypes.c_void_p()
            _lib.check(lib.mwf_host_alloc(nbytes, ctypes.byref(ptr)))
            ptrs.append(ptr)
            arrs.append(np.ctypeslib.as_array((ctypes.c_double * p.dof).from_address(ptr.value)))
        re, im = arrs
        c0 = ens.get_state(0)
        re[:] = c0.real.ravel()
        im[:] = c0.imag.ravel()
        ke = max(3, min(args.steps, 10))
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(ke):
            ens.set_state_ref(0, re, im)
            ens.step(1)
            ens.get_state_ref(0, re, im)
        te = allreduce_max(pg, time.perf_counter() - t0)
        for ptr in ptrs:
            lib.mwf_host_free(ptr)
        e2e = {"value": world * p.dof * ke / te, "unit": "dof-steps/s",
               "h2d_bytes_per_step": 2 * nbytes, "d2h_bytes_per_step": 2 * nbytes,
               "steps": ke, "path": "mwf_set_state + mwf_step(1) + mwf_get_state, pinned host"}
    fp64 = all(p.precision == "fp64" for p in runs)
    line = {
        "metric": "dof-steps/s", "value": res["value"], "unit": "dof-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if fp64 else "f32", "data": "synthetic",
        "config": config_dict(args.workload, runs, kind, world),
        "step_mode": "persistent" if args.persistent else "per-pass launches",
        "tuning": {"autotuned": not args.no_tune, "setup_s": round(t_tune, 2),
                   "knobs_run0": {k: getattr(runs[0], k) for k in
                                  ("xf_cols", "xi_cols", "z_lines", "x_radix", "z_radix")}},
    }
    for k in ("clocks", "gpu_launches", "pass_ms", "step_alg_bytes", "roofline", "alu_roofline", "host_wall_s"):
        line[k] = res[k]
    if e2e:
        line["e2e"] = e2e
    ens.close()
    del ens
    if rank == 0:
        cf = cufft_transforms_ms(runs, dev)
        line["cufft_comparison"] = {
            "transforms_ms_per_step": cf, "mwf_step_ms": res["ms_per_step"],
            "note": "cuFFT (torch.fft) doing only the step's batched transforms, no nonlinear term, "
                    "padding or update: a lower bound for a library-FFT step; comparison only"}
    # ---- the batched FP32 form beside the plain FP64 headline (same process, same GPU) ----
    if args.workload == "m6-1024-fp64" and not args.no_fp32_batch:
        eruns, ekind = workload_params("ensemble512-fp32")
        t_e = time.perf_counter()
        ens = mwf.Ensemble(eruns, device=dev, tune=not args.no_tune)
        t_e = time.perf_counter() - t_e
        for i, p in enumerate(ens.runs):
            ens.set_state(i, initial_state(p, ekind, 1000 * rank + i))
        fr = measure_resident(ens, args, pg, world, dev)
        if fr["roofline"]["kernel"] == "z_nonlinear":
            fr["roofline"]["traffic"] = zpass_traffic_fp32(ens.runs)
        # the same step as one persistent launch (same results; slower on GB300: see mwf_set_persistent)
        ens.set_persistent(True)
        ens.step(args.warmup)
        persistent_ms = allreduce_max(pg, ens.step_timed(args.steps)) / args.steps
        ens.set_persistent(False)
        ens.close()
        del ens
        line["fp32_batched"] = {
            "workload": "ensemble512-fp32", "runs_per_gpu": len(eruns),
            "dof_per_gpu": sum(p.dof for p in eruns),
            "grids": "M4, N x N modes with N uniform over {64, 96, 128, 192, 256} (MM = NN = N/2), "
                     "L = N pi/3, Re U(150, 350), dt 0.02, Gaussian IC |k| <= 8, seeds 0..511",
            "value": fr["value"], "unit": "dof-steps/s", "ms_per_step": fr["ms_per_step"],
            "pass_ms": fr["pass_ms"], "roofline": fr["roofline"], "alu_roofline": fr["alu_roofline"],
            "clocks": fr["clocks"], "gpu_launches": fr["gpu_launches"], "setup_s": round(t_e, 2),
            "persistent_launch_ms_per_step": persistent_ms,
            "l2": "inputs larger than L2 (step working set "
                  f"{fr['step_alg_bytes'] / 1e9:.2f} GB > 129 MB)"}
        line["fp32_over_fp64"] = fr["value"] / res["value"]
        line["gpu_launches"] += fr["gpu_launches"]
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = host_cores()
        # bounded samples: about 10 s on all cores and 6 s on one core
        rate, dt, ns = cpu_port_rate_bounded(runs, kind, cores, 10.0)
        rate1, dt1, ns1 = cpu_port_rate_bounded(runs, kind, 1, 6.0)
        line["cpu_baseline"] = {"value": rate, "unit": "dof-steps/s", "cores": cores, "kind": "port",
                                "sample": f"{ns} full steps of the workload's first run after 1 warm-up step "
                                          f"in {dt:.2f} s: C++ FP64 restatement with OpenMP "
                                          "(oracle/cpu_step.cpp), not the reference binary",
                                "single_core": {"value": rate1,
                                                "sample": f"{ns1} steps in {dt1:.2f} s, 1 thread"}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_precision(args, world, rank, local, pg):
    """FP32 beside FP64 on the M4 precision case: 2048 x 2048 modes on a 3072 x 3072 grid,
    Lx = Lz = 512 pi, Re = 250, dt = 0.01, Gaussian IC with |k| <= 16, amplitude 0.3; both
    runs in one handle from the same state.  Reported: relative coefficient error of FP32
    against FP64 after 10 and 100 steps, and over the run (every 50 steps, before the step
    as in io_write2files) the mean-energy error and the turbulent-fraction error with the
    fixed threshold epos > 0.1.  The FP64 GPU path stands in for the FP64 oracle here (it
    matches the numpy oracle to 1e-11 after 100 steps on smaller grids; the numpy oracle
    would need days for 2000 steps of this grid)."""
    import mwf_gb300 as mwf
    from mwf_gb300 import build
    build.build()
    total = args.steps if args.steps > 100 else 2000
    ct = 0.1
    p64 = mwf.RunParams.square(4, 2048, 512 * PI, Re=250.0, dt=0.01)
    p32 = p64.with_(precision="fp32")
    c0 = mwf.ic.gaussian_ic(p64, seed=local, kmax=16)
    ens = mwf.Ensemble([p64, p32], device=local)
    ens.set_state(0, c0)
    ens.set_state(1, c0)

    def coef_err():
        a, b = ens.get_state(0), ens.get_state(1)
        return float(np.abs(b - a).max() / np.abs(a).max())

    errs, e64, e32, f64, f32 = {}, [], [], [], []
    t0 = time.perf_counter()
    done = 0
    while done < total:
        if done % 50 == 0:
            e64.append(ens.energy(0))
            e32.append(ens.energy(1))
            f64.append(ens.turbulent_fraction(0, ct))
            f32.append(ens.turbulent_fraction(1, ct))
        n = 10 if done < 10 else (90 if done < 100 else 50)
        n = min(n, 50 - done % 50, total - done)
        ens.step(n)
        done += n
        if done in (10, 100):
            errs[done] = coef_err()
    wall = time.perf_counter() - t0
    pm = ens.profile_passes(3)
    ens.close()
    line = {
        "metric": "fp32_vs_fp64_error", "config": {"workload": "precision-m4-2048", "K0": 4, "MM": 1024,
                                                   "NN": 1024, "grid": "3072x3072", "Re": 250.0, "dt": 0.01,
                                                   "steps": total, "ic": "gauss |k|<=16 amp 0.3",
                                                   "turb_threshold": ct},
        "coef_rel_err_10": errs.get(10), "coef_rel_err_100": errs.get(100),
        "mean_energy_fp64": float(np.mean(e64)), "mean_energy_fp32": float(np.mean(e32)),
        "mean_energy_rel_err": float(abs(np.mean(e32) - np.mean(e64)) / abs(np.mean(e64))),
        "turb_frac_mean_fp64": float(np.mean(f64)), "turb_frac_mean_fp32": float(np.mean(f32)),
        "turb_frac_mean_abs_err": float(abs(np.mean(f32) - np.mean(f64))),
        "energy_series_fp64": e64, "energy_series_fp32": e32,
        "wall_s": wall, "pass_ms_both": dict(zip(["x_forward", "z_nonlinear", "x_inverse"], pm)),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_serve(args, world, rank, local, pg):
    """Continuous-batching serving on the configured Poisson trace: 50 requests/s, M4/M6
    70/30, N x N modes log-uniform in 64..512 (rounded to 2^a 3^b), Re U(150, 400), steps
    log-uniform in 500..20000, FP32/FP64 80/20, 150 GiB HBM admission budget.
    Phase A runs the configured arrival process for --serve-window seconds of wall time and
    reports the offered load (dof-steps of the requests that arrived, per second of arrivals)
    against the served load (dof-steps/s the server completed), which is far lower: the
    configured trace asks for orders of magnitude more than one GPU delivers.  Phase B
    offers requests of the same distribution at a rate the GPU sustains (70 % of phase A's
    served dof-steps/s divided by the mean work per request) for --serve-sustain-window seconds,
    drains them, and reports p50/p99 completion latency and the aggregate dof-steps/s."""
    from mwf_gb300 import build, serve
    build.build()
    budget = 150 * 2 ** 30
    # phase A: the configured trace, bounded wall time
    trace = serve.poisson_trace(rate=50.0, duration=args.serve_window, seed=1000 + rank)
    mean_work = float(np.mean([r.params.dof * r.steps for r in trace]))
    srv = serve.Server(budget_bytes=budget, chunk=50, device=local, admit_interval=0.1)
    barrier(pg)
    a = srv.run_trace(trace, max_wall=args.serve_window)
    offered = srv.offered_dof_steps / args.serve_window
    served = a["dof_steps_per_s"]
    for co in srv.cohorts:
        co.ens.close()
    # phase B: a load the GPU sustains, drained
    rate_b = max(0.05, 0.7 * served / mean_work)
    trace_b = serve.poisson_trace(rate=rate_b, duration=args.serve_sustain_window, seed=2000 + rank)
    srv_b = serve.Server(budget_bytes=budget, chunk=50, device=local, admit_interval=0.1)
    b = srv_b.run_trace(trace_b, max_wall=args.serve_max_wall)
    wall = allreduce_max(pg, b["wall_s"])
    line = {
        "metric": "dof-steps/s", "value": b["dof_steps_per_s"] * world, "unit": "dof-steps/s",
        "n_gpus": world, "steps": b["completed"], "warmup": 0, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "mixed f32/f64", "data": "synthetic",
        "config": {"workload": "serve-poisson", "hbm_budget_gib": 150, "steps_range": [500, 20000],
                   "modes_range": [64, 512], "m4_fraction": 0.7, "fp32_fraction": 0.8, "re_range": [150, 400]},
        "configured_trace": {"rate_per_s": 50.0, "window_s": args.serve_window, "requests": len(trace),
                             "offered_dof_steps_per_s": offered, "served_dof_steps_per_s": served,
                             "served_fraction": served / offered if offered else None,
                             "completed": a["completed"], "failed": a["failed"], "still_waiting": a["waiting"],
                             "mean_dof_steps_per_request": mean_work},
        "sustained_trace": {"rate_per_s": rate_b, "arrival_window_s": args.serve_sustain_window,
                            "requests": len(trace_b), "completed": b["completed"], "failed": b["failed"],
                            "p50_latency_s": b["p50_latency_s"], "p99_latency_s": b["p99_latency_s"],
                            "dof_steps_per_s": b["dof_steps_per_s"], "compactions": b["compactions"],
                            "wall_s": wall, "drained": b["waiting"] == 0 and b["completed"] + b["failed"] == len(trace_b)},
        "p50_latency_s": b["p50_latency_s"], "p99_latency_s": b["p99_latency_s"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mwf", choices=["mwf", "reference"])
    ap.add_argument("--workload", default="m6-1024-fp64")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="use the planner's default tiles/radices")
    ap.add_argument("--serve-window", type=float, default=60.0,
                    help="serving: seconds of the configured 50 req/s trace (offered vs served load)")
    ap.add_argument("--serve-sustain-window", type=float, default=120.0,
                    help="serving: arrival window of the sustainable-load trace (latency percentiles)")
    ap.add_argument("--serve-max-wall", type=float, default=900.0,
                    help="serving: wall-time limit of the sustainable-load phase, drain included")
    ap.add_argument("--persistent", action="store_true",
                    help="step the workload in the persistent step mode (one launch per step)")
    ap.add_argument("--no-fp32-batch", action="store_true",
                    help="skip the 512-run FP32 ensemble measured beside the FP64 headline")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
    elif args.workload.startswith("serve"):
        run_serve(args, world, rank, local, pg)
    elif args.workload.startswith("precision"):
        run_precision(args, world, rank, local, pg)
    else:
        run_gpu(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
