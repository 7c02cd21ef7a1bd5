"""ctypes wrapper of oracle/cpu_step.cpp, the C++ FP64 / OpenMP restatement of the timestep
(test and baseline infrastructure, not the product).  Only ``tests/`` and ``bench.py``'s
CPU-baseline / reference legs use it.  It takes its tables from the numpy oracle
(``lhsrhs``, ``tables``) and its mode-coupling terms from the Galerkin tensors of
``oracle/galerkin.py``, and is checked against ``mwf_oracle.Solver`` in tests/test_cpu_port.py.
Symmetry masks (vel_imposesym) are not restated here."""
import ctypes
import os
import subprocess
import threading

import numpy as np

from . import galerkin
from . import mwf_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_step.cpp")
OUT = os.path.join(HERE, "_build", "libmwfcpu.so")
_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile cpu_step.cpp with g++ -O3 -fopenmp (no target-specific flags)."""
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    tmp = OUT + ".tmp"
    subprocess.run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", SRC, "-o", tmp], check=True)
    os.replace(tmp, OUT)
    return OUT


def load():
    global _lib
    with _lock:
        if _lib is None:
            lib = ctypes.CDLL(build())
            dp = ctypes.POINTER(ctypes.c_double)
            lib.mwfcpu_create.restype = ctypes.c_void_p
            lib.mwfcpu_create.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 5 + [dp] * 5 + [
                ctypes.c_int, ctypes.POINTER(ctypes.c_int), dp]
            lib.mwfcpu_destroy.argtypes = [ctypes.c_void_p]
            lib.mwfcpu_step.restype = ctypes.c_int
            lib.mwfcpu_step.argtypes = [ctypes.c_void_p, dp, dp, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                        ctypes.c_int]
            _lib = lib
    return _lib


def coupling_terms(K0, tol=1e-14):
    """udotgradu (modes.M4.f90:14-36, modes.M6.f90:14-20, 22-79) as terms out[d] += c * P[a] * P[b]
    over the 3KK physical fields P = (u, du/dx, du/dz), each KK long in the order u 0..K0-1,
    v 1..K0-1, w 0..K0-1 -- the contraction of mwf_oracle.udotgradu written out."""
    Gp, Gv, Hp, Hv, _ = galerkin.tensors(K0)
    KK = 3 * K0 - 1
    U, V, W = 0, K0, 2 * K0 - 1              # offsets of u, v, w inside a block of KK
    DX, DZ = KK, 2 * KK                      # offsets of the d/dx and d/dz blocks
    idx, coef = [], []

    def add(T, dbase, abase, bbase):
        for d, i, j in zip(*np.nonzero(np.abs(T) > tol)):
            idx.append((dbase + d, abase + i, bbase + j))
            coef.append(T[d, i, j])

    add(Gp, U, U, DX + U); add(Hp, U, V, U); add(Gp, U, W, DZ + U)
    add(Gv, V, U, DX + V); add(Hv, V, V, V); add(Gv, V, W, DZ + V)
    add(Gp, W, U, DX + W); add(Hp, W, V, W); add(Gp, W, W, DZ + W)
    return np.array(idx, np.int32).reshape(-1, 3), np.array(coef, np.float64)


class CpuSolver:
    """mwf_oracle.Solver's interface over the C++ step (no symmetry masks)."""

    def __init__(self, p: O.Params, c0, threads=1):
        if p.reflect or p.uvreflect or p.wreflect:
            raise ValueError("the C++ restatement has no symmetry masks")
        lib = load()
        self.p, self.threads = p, int(threads)
        L, R = O.lhsrhs(p)
        m1, _, n1, _, k1, _ = O.tables(p)
        self._keep = [np.ascontiguousarray(a, np.float64) for a in (L, R, m1, n1, k1)]
        tidx, tcoef = coupling_terms(p.K0)
        self.nterms = len(tcoef)
        self._keep += [np.ascontiguousarray(tidx), np.ascontiguousarray(tcoef)]
        dp = ctypes.POINTER(ctypes.c_double)
        ptr = [a.ctypes.data_as(dp) for a in self._keep[:5]]
        self.h = lib.mwfcpu_create(p.K0, p.MM, p.NN, p.alpha, p.gamma, p.dt, np.cos(p.theta), np.sin(p.theta),
                                   *ptr, self.nterms, self._keep[5].ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   self._keep[6].ctypes.data_as(dp))
        if not self.h:
            raise ValueError("cpu restatement: 3MM and 3NN must be of the form 2^a 3^b")
        self.c = np.ascontiguousarray(np.array(c0, dtype=np.complex128))
        self.onl = np.zeros_like(self.c)
        self.nst = ctypes.c_int(1)

    def step(self, n=1):
        dp = ctypes.POINTER(ctypes.c_double)
        rc = load().mwfcpu_step(self.h, self.c.ctypes.data_as(dp), self.onl.ctypes.data_as(dp),
                                ctypes.byref(self.nst), int(n), self.threads)
        if rc:
            raise RuntimeError("mwfcpu_step failed")
        return self.c

    def close(self):
        if self.h:
            load().mwfcpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
