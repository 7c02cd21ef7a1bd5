"""Host-side mirror of the reference's ``velocity`` module over the C ABI.

``RunParams`` is the runtime copy of program/parameters.f90:7-72; ``Ensemble`` owns the
device state of one or more runs (one C-ABI handle); ``Velocity`` is the single-run view
with the reference's routine names (``vel_TS``, ``vel_energy``, ``vel_c``).

State arrays on the Python side are complex128 ``c[n, m, k]`` of shape (NN, M, K), which
has the same memory order as the Fortran ``mpt%Re/Im(K, 0:M-1, 0:NN-1)`` arrays.
"""
import ctypes
import math
from dataclasses import dataclass, replace

import numpy as np

from . import _lib

PI = 3.1415926535897931


@dataclass
class RunParams:
    K0: int = 4
    MM: int = 32
    NN: int = 32
    alpha: float = 2 * PI / 12.0
    gamma: float = 2 * PI / 6.0
    Re: float = 200.0
    dt: float = 0.01
    drag: float = 1e-2
    vdrag: float = 0.0
    hypo: float = 0.0
    dragall: bool = True
    theta: float = 0.0
    reflect: bool = False
    uvreflect: bool = False
    wreflect: bool = False
    precision: str = "fp64"        # "fp64" (plain path) or "fp32"
    # tuning knobs (0 = planner default): x-forward / x-inverse columns per CTA, z-pass x
    # lines per CTA, largest radix of the x / z transforms
    xf_cols: int = 0
    xi_cols: int = 0
    z_lines: int = 0
    x_radix: int = 0
    z_radix: int = 0

    @property
    def K(self):
        return 2 * self.K0 - 1

    @property
    def KK(self):
        return 3 * self.K0 - 1

    @property
    def M(self):
        return 2 * (self.MM - 1) + 1

    @property
    def X(self):
        return 3 * self.MM

    @property
    def Z(self):
        return 3 * self.NN

    @property
    def dof(self):
        """complex MPT coefficients K*(2MM-1)*NN of the prognostic state"""
        return self.K * self.M * self.NN

    @property
    def shape(self):
        return (self.NN, self.M, self.K)

    def with_(self, **kw):
        return replace(self, **kw)

    def to_c(self):
        if self.precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        return _lib.RunDescC(
            self.K0, self.MM, self.NN, _lib.MWF_FP64 if self.precision == "fp64" else _lib.MWF_FP32,
            self.alpha, self.gamma, self.Re, self.dt, self.drag, self.vdrag, self.hypo,
            int(bool(self.dragall)), int(bool(self.reflect)), int(bool(self.uvreflect)),
            int(bool(self.wreflect)), self.theta, int(self.xf_cols), int(self.xi_cols),
            int(self.z_lines), int(self.x_radix), int(self.z_radix))

    @classmethod
    def square(cls, K0, N_modes, L, **kw):
        """A run of N_modes x N_modes Fourier modes (MM = NN = N_modes/2, grid 3N/2) on Lx = Lz = L."""
        return cls(K0=K0, MM=N_modes // 2, NN=N_modes // 2, alpha=2 * PI / L, gamma=2 * PI / L, **kw)


def footprint_bytes(runs):
    """Device bytes that an Ensemble of these runs allocates (admission control)."""
    lib = _lib.load()
    arr = (_lib.RunDescC * len(runs))(*[r.to_c() for r in runs])
    return int(lib.mwf_footprint_bytes(arr, len(runs)))


def describe_run(p):
    """The kernels and tiling the library would step run p with (mwf_describe_run), as a dict:
    batched_x / batched_z, columns or lines per work item, CTAs per SM, shared memory per CTA
    and work items per step of each pass.  Host only; raises MwfError for a run the kernels
    cannot take."""
    lib = _lib.load()
    d = p.to_c()
    out = _lib.RunPlanC()
    _lib.check(lib.mwf_describe_run(ctypes.byref(d), ctypes.byref(out)))
    return {name: getattr(out, name) for name, _ in _lib.RunPlanC._fields_}


class Ensemble:
    """Independent runs of possibly different sizes, precisions and parameters, advanced
    together: every step is one CUDA-graph replay of the three passes over all runs."""

    def __init__(self, runs, device=0, tune=False):
        """tune=True: take each run's tile/radix knobs from the autotuner (timing them on
        first use of a grid, cached per precision/model/grid)."""
        self.lib = _lib.load()
        runs = list(runs)
        if tune:
            from . import autotune
            count = {}
            for r in runs:
                k = autotune.key(r)
                count[k] = count.get(k, 0) + 1
            seen = {}
            for i, r in enumerate(runs):
                k = (autotune.key(r), r.xf_cols, r.xi_cols, r.z_lines, r.x_radix, r.z_radix)
                if k not in seen:
                    seen[k] = autotune.tuned(r, device=device, copies=count[autotune.key(r)])
                t = seen[k]
                runs[i] = r.with_(xf_cols=t.xf_cols, xi_cols=t.xi_cols, z_lines=t.z_lines,
                                  x_radix=t.x_radix, z_radix=t.z_radix)
        self.runs = runs
        arr = (_lib.RunDescC * len(self.runs))(*[r.to_c() for r in self.runs])
        h = ctypes.c_void_p()
        _lib.check(self.lib.mwf_create(arr, len(self.runs), device, ctypes.byref(h)))
        self._h = h
        self.device = device

    @property
    def handle(self):
        if self._h is None:
            raise RuntimeError("ensemble is closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            _lib.check(self.lib.mwf_destroy(self._h))
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ------------------------------------------------------------------------
    def set_state(self, run, c):
        p = self.runs[run]
        c = np.asarray(c)
        if c.shape != p.shape:
            raise ValueError(f"state shape {c.shape} != {p.shape}")
        re = np.ascontiguousarray(c.real, dtype=np.float64)
        im = np.ascontiguousarray(c.imag, dtype=np.float64)
        self.set_state_ref(run, re, im)

    def set_state_ref(self, run, re, im):
        """re/im: float64 arrays in the reference layout (K, M, NN) Fortran order, given as any
        C-contiguous array whose flat order matches it (e.g. shape (NN, M, K))."""
        n = self.runs[run].dof
        if re.size != n or im.size != n or not re.flags.c_contiguous or not im.flags.c_contiguous:
            raise ValueError("re/im must be C-contiguous float64 arrays of K*M*NN elements")
        _lib.check(self.lib.mwf_set_state(self.handle, run, re.ctypes.data, im.ctypes.data))

    def get_state(self, run):
        p = self.runs[run]
        re = np.empty(p.shape)
        im = np.empty(p.shape)
        self.get_state_ref(run, re, im)
        return re + 1j * im

    def get_state_ref(self, run, re, im):
        n = self.runs[run].dof
        if re.size != n or im.size != n or not re.flags.c_contiguous or not im.flags.c_contiguous:
            raise ValueError("re/im must be C-contiguous float64 arrays of K*M*NN elements")
        _lib.check(self.lib.mwf_get_state(self.handle, run, re.ctypes.data, im.ctypes.data))

    def get_history(self, run):
        """(AB2 history as complex (NN, M, K), Euler-start flag of the next step)."""
        p = self.runs[run]
        re = np.empty(p.shape)
        im = np.empty(p.shape)
        flag = ctypes.c_int()
        _lib.check(self.lib.mwf_get_history(self.handle, run, re.ctypes.data, im.ctypes.data, ctypes.byref(flag)))
        return re + 1j * im, bool(flag.value)

    def set_history(self, run, onl, euler_next):
        p = self.runs[run]
        onl = np.asarray(onl)
        if onl.shape != p.shape:
            raise ValueError(f"history shape {onl.shape} != {p.shape}")
        re = np.ascontiguousarray(onl.real, dtype=np.float64)
        im = np.ascontiguousarray(onl.imag, dtype=np.float64)
        _lib.check(self.lib.mwf_set_history(self.handle, run, re.ctypes.data, im.ctypes.data, int(bool(euler_next))))

    def checkpoint(self, run):
        """Everything a run needs to continue exactly: (state, history, Euler-start flag)."""
        onl, flag = self.get_history(run)
        return self.get_state(run), onl, flag

    def restore(self, run, ckpt):
        c, onl, flag = ckpt
        self.set_state(run, c)
        self.set_history(run, onl, flag)

    def query(self):
        """True when every queued step has finished (does not wait)."""
        idle = ctypes.c_int()
        _lib.check(self.lib.mwf_query(self.handle, ctypes.byref(idle)))
        return bool(idle.value)

    # -- time stepping -----------------------------------------------------------------
    def step(self, nsteps=1):
        _lib.check(self.lib.mwf_step(self.handle, int(nsteps)))

    def step_async(self, nsteps=1):
        _lib.check(self.lib.mwf_step_async(self.handle, int(nsteps)))

    def synchronize(self):
        _lib.check(self.lib.mwf_synchronize(self.handle))

    def reset_history(self, run):
        _lib.check(self.lib.mwf_reset_history(self.handle, run))

    def set_active(self, run, active):
        """Stop (False) or resume (True) stepping one run inside the batch."""
        _lib.check(self.lib.mwf_set_active(self.handle, run, int(bool(active))))

    def step_timed(self, nsteps):
        """Advance nsteps; returns device milliseconds (CUDA events on the library's stream)."""
        ms = ctypes.c_double()
        _lib.check(self.lib.mwf_step_timed(self.handle, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def set_persistent(self, on):
        """Step the FP32 runs with batched passes in one persistent launch (True) or with one
        launch per pass and grid size (False, the default, faster on GB300); same results."""
        _lib.check(self.lib.mwf_set_persistent(self.handle, int(bool(on))))

    def kernels_per_step(self):
        """Kernel launches one step makes (the grouped passes and any symmetry masks)."""
        n = ctypes.c_int()
        _lib.check(self.lib.mwf_kernels_per_step(self.handle, ctypes.byref(n)))
        return n.value

    def profile_passes(self, nreps):
        """Mean device ms per step of (x-forward, z nonlinear, x-inverse+update); advances nreps steps."""
        arr = (ctypes.c_double * 3)()
        _lib.check(self.lib.mwf_profile_passes(self.handle, int(nreps), arr))
        return tuple(arr)

    def phys_diagnostics(self, run, threshold):
        """(points with epos > threshold, physical-space energy) of the current state."""
        cnt, e = ctypes.c_double(), ctypes.c_double()
        _lib.check(self.lib.mwf_phys_diagnostics(self.handle, run, float(threshold), ctypes.byref(cnt),
                                                 ctypes.byref(e)))
        return cnt.value, e.value

    def turbulent_fraction(self, run, threshold):
        """The reference's turbulent fraction: count / ((3MM+1)(3NN+1)) (io.f90:597-615)."""
        p = self.runs[run]
        cnt, _ = self.phys_diagnostics(run, threshold)
        return cnt / ((p.X + 1) * (p.Z + 1))

    def energy(self, run):
        e = ctypes.c_double()
        _lib.check(self.lib.mwf_energy(self.handle, run, ctypes.byref(e)))
        return e.value

    # -- state operations and diagnostics outside the timestep ---------------------------
    def get_phys(self, run):
        """vel_mpt2phys without the base flow: float64 array (X, Z, KK), i.e. the reference's
        phys%Re(KK, 0:Z-1, 0:X-1) in C order."""
        p = self.runs[run]
        out = np.empty((p.X, p.Z, p.KK))
        _lib.check(self.lib.mwf_get_phys(self.handle, run, out.ctypes.data))
        return out

    def spectrum_maxima(self, run):
        """io_save_Uspec: (m_max over |m| = 0..MM-1, n_max over n = 0..NN-1)."""
        p = self.runs[run]
        m_max, n_max = np.empty(p.MM), np.empty(p.NN)
        _lib.check(self.lib.mwf_spectrum_maxima(self.handle, run, m_max.ctypes.data, n_max.ctypes.data))
        return m_max, n_max

    def history(self, run, y=0.0, n_probes=32):
        """vel_history: rows (z position, u, v, w) of the probes at x = 0, height y."""
        H = np.empty((int(n_probes), 4))
        _lib.check(self.lib.mwf_history(self.handle, run, float(y), int(n_probes), H.ctypes.data))
        return H

    def remap_x(self, run, factor):
        """var_quadX (factor 4) / var_doubleX (factor 2): x wavenumber m -> factor*m."""
        _lib.check(self.lib.mwf_remap_x(self.handle, run, int(factor)))

    def blend_state(self, run, other, d):
        """utils/interpstate: state[run] := (1-d) state[run] + d state[other]."""
        _lib.check(self.lib.mwf_blend_state(self.handle, run, int(other), float(d)))

    def add_noise(self, run, scale, seed=0):
        """var_randadd with a seeded counter-based generator."""
        _lib.check(self.lib.mwf_add_noise(self.handle, run, float(scale), int(seed) & (2 ** 64 - 1)))


class Velocity:
    """One run with the reference's velocity-module names (program/velocity.f90)."""

    def __init__(self, params: RunParams, device=0):
        self.params = params
        self.ens = Ensemble([params], device=device)
        self.tim_t = 0.0
        self.tim_step = 0

    @property
    def vel_c(self):
        return self.ens.get_state(0)

    @vel_c.setter
    def vel_c(self, c):
        self.ens.set_state(0, c)

    def vel_TS(self, nsteps=1):
        """vel_imposesym + vel_TS, nsteps times (main.f90:22-26)."""
        self.ens.step(nsteps)
        self.tim_t += nsteps * self.params.dt
        self.tim_step += nsteps

    def vel_energy(self):
        """vel_energy(vel_mpt2phys(vel_c)) (velocity.f90:84-90, 144-162)"""
        return self.ens.energy(0)

    def reset_history(self):
        self.ens.reset_history(0)

    def vel_mpt2phys(self):
        """vel_mpt2phys(vel_c) (velocity.f90:84-90): (X, Z, KK) float64."""
        return self.ens.get_phys(0)

    def vel_history(self, y=0.0, n_probes=32):
        """vel_history (velocity.f90:164-180): (n_probes, 4) rows of io_write_history."""
        return self.ens.history(0, y, n_probes)

    def vel_spec(self):
        """The two columns of io_save_Uspec's vel_spec file (io.f90:345-372)."""
        return self.ens.spectrum_maxima(0)

    def var_doubleX(self):
        self.ens.remap_x(0, 2)

    def var_quadX(self):
        self.ens.remap_x(0, 4)

    def var_randadd(self, scl, seed=0):
        self.ens.add_noise(0, scl, seed)

    def close(self):
        self.ens.close()


def spec2phys(p, s):
    """tra_spec2phys on the device: spectral u, v, w (NN, M, KK) complex -> the physical fields
    (X, Z, KK) float64 of the 3MM x 3NN grid (the reference's type(phys) in C order)."""
    lib = _lib.load()
    s = np.asarray(s)
    if s.shape != (p.NN, p.M, p.KK):
        raise ValueError(f"spectral shape {s.shape} != {(p.NN, p.M, p.KK)}")
    re = np.ascontiguousarray(s.real, dtype=np.float64)
    im = np.ascontiguousarray(s.imag, dtype=np.float64)
    out = np.empty((p.X, p.Z, p.KK))
    d = p.to_c()
    _lib.check(lib.mwf_spec2phys(ctypes.byref(d), re.ctypes.data, im.ctypes.data, out.ctypes.data))
    return out


def phys2spec(p, ph):
    """tra_phys2spec on the device: physical fields (X, Z, KK) -> spectral (NN, M, KK) complex."""
    lib = _lib.load()
    ph = np.ascontiguousarray(ph, dtype=np.float64)
    if ph.shape != (p.X, p.Z, p.KK):
        raise ValueError(f"physical shape {ph.shape} != {(p.X, p.Z, p.KK)}")
    re = np.empty((p.NN, p.M, p.KK))
    im = np.empty((p.NN, p.M, p.KK))
    d = p.to_c()
    _lib.check(lib.mwf_phys2spec(ctypes.byref(d), ph.ctypes.data, re.ctypes.data, im.ctypes.data))
    return re + 1j * im


def measure_fma_peak(device=0, fp64=True):
    """Measured FMA peak of the device in TFLOP/s (FP64 or FP32 pipe)."""
    lib = _lib.load()
    v = ctypes.c_double()
    _lib.check(lib.mwf_measure_fma_peak(device, 0 if fp64 else 1, ctypes.byref(v)))
    return v.value


def dof_steps(runs, steps):
    return sum(r.dof for r in runs) * steps


def is_23_smooth(n):
    if n < 1:
        return False
    while n % 2 == 0:
        n //= 2
    while n % 3 == 0:
        n //= 3
    return n == 1


def round_23(n):
    """Nearest 2^a 3^b >= 2 to n (log distance), for grid sizes drawn from a continuous range."""
    best = None
    for a in range(0, 16):
        for b in range(0, 10):
            v = 2 ** a * 3 ** b
            if v < 2:
                continue
            d = abs(math.log(v) - math.log(n))
            if best is None or d < best[0]:
                best = (d, v)
    return best[1]
