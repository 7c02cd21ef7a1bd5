"""Autotuner for the per-run knobs of the passes, chosen by timing them on the device.

Knobs (fields of RunParams / mwf_run_desc, 0 = planner default):
    xf_cols, xi_cols   columns n per CTA of the x-forward / x-inverse pass
    z_lines            x lines per CTA of the z pass
    x_radix, z_radix   largest radix of the x / z transforms (8, 12, 16 within the caps)
The x knobs and the z knobs are tuned separately: every candidate is one handle holding 1, 8
or 32 copies of the run (the batch context: the best tiles of a run alone and of a run in a
large batch differ) whose passes are timed with CUDA events (mwf_profile_passes); the
default configuration is always a candidate, so tuning never picks a slower one in that
context.  Results are cached in a JSON file keyed by precision, model, grid and context
(MWF_TUNE_CACHE, default ~/.cache/mwf_gb300/tuning.json).  This plays the part of the FFTW_PATIENT planning the
reference does at start-up (transform.fftw5.f90:33-59).
"""
import json
import os

import numpy as np

from .solver import Ensemble, footprint_bytes

CACHE = os.environ.get("MWF_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "mwf_gb300",
                                                      "tuning.json"))
_mem = {}


def batch_bucket(copies):
    """Tuning context: a run alone (1), in a small batch (8) or in a large batch (32)."""
    return 1 if copies <= 1 else (8 if copies <= 8 else 32)


KERNEL_VERSION = 3      # bumped when the kernels' tiling changes, so old cache entries are ignored


def key(p, copies=1):
    return f"v{KERNEL_VERSION}:{p.precision}:M{p.K0}:{p.MM}x{p.NN}:b{batch_bucket(copies)}"


def _load():
    if _mem:
        return _mem
    try:
        with open(CACHE) as f:
            _mem.update(json.load(f))
    except (OSError, ValueError):
        pass
    return _mem


def _store():
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        with open(CACHE, "w") as f:
            json.dump(_mem, f, indent=1, sort_keys=True)
    except OSError:
        pass


def _valid(p):
    return footprint_bytes([p]) > 0


def _time(p, device, reps, copies):
    runs = [p] * copies
    with Ensemble(runs, device=device) as e:
        rng = np.random.default_rng(0)
        for i in range(copies):
            c = 1e-3 * (rng.standard_normal(p.shape) + 1j * rng.standard_normal(p.shape))
            c[0] = c[0].real
            e.set_state(i, c)
        e.step(2)
        return e.profile_passes(reps)


def tune(p, device=0, reps=3, copies=1):
    """Time the candidates for run p (in a handle of `copies` such runs, the tuning context)
    and return the best knob settings (a dict)."""
    copies = batch_bucket(copies)
    base = p.with_(xf_cols=0, xi_cols=0, z_lines=0, x_radix=0, z_radix=0)
    x_radices = [8, 12, 16] if p.precision == "fp32" else [8, 12]
    z_radices = [8, 12] if p.precision == "fp32" else [8]
    widths = [1, 2, 4, 8, 16]
    best_x, best_xt = {}, None
    for xr in [0] + x_radices:
        # the two x passes are timed separately, so their column tiles are chosen separately
        # (their capacities differ: x-forward tiles up to twice as many columns in FP32)
        tf, ti = {}, {}
        for cols in [0] + widths:
            for xf, xi in ((cols, cols), (cols, 0), (0, cols)):
                q = base.with_(x_radix=xr, xf_cols=xf, xi_cols=xi)
                if _valid(q):
                    t = _time(q, device, reps, copies)
                    tf.setdefault(xf, t[0])
                    ti.setdefault(xi, t[2])
                    break
        if tf and ti:
            cf, ci = min(tf, key=tf.get), min(ti, key=ti.get)
            if best_xt is None or tf[cf] + ti[ci] < best_xt:
                best_xt, best_x = tf[cf] + ti[ci], {"x_radix": xr, "xf_cols": cf, "xi_cols": ci}
    best_z, best_zt = {}, None
    for zr in [0] + z_radices:
        for lines in [0] + widths:
            q = base.with_(z_radix=zr, z_lines=lines)
            if not _valid(q):
                continue
            t = _time(q, device, reps, copies)
            if best_zt is None or t[1] < best_zt:
                best_zt, best_z = t[1], {"z_radix": zr, "z_lines": lines}
    out = dict(best_x)
    out.update(best_z)
    out["ms"] = {"x": best_xt, "z": best_zt, "copies": copies}
    return out


def tuned(p, device=0, reps=3, retune=False, copies=1):
    """p with its knobs from the cache, tuning (and caching) first if needed; copies = how
    many runs of this configuration the batch holds."""
    db = _load()
    k = key(p, copies)
    if retune or k not in db:
        db[k] = tune(p, device=device, reps=reps, copies=copies)
        _store()
    knobs = {n: db[k][n] for n in ("xf_cols", "xi_cols", "z_lines", "x_radix", "z_radix")}
    return p.with_(**knobs)
