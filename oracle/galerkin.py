"""Oracle (test infrastructure only): wall-normal Galerkin coupling tensors by quadrature.

This module is part of the CPU oracle.  Only the tests, ``__graft_entry__.smoke`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.

The reference's mode-coupling functions (``nluw``, ``nluv``, ``nluyv``, ``nlvvy``, ``nlvv`` in
program/modes.M4.f90:38-72 and program/modes.M6.f90:22-79, combined by ``udotgradu`` at
modes.M4.f90:14-36 / modes.M6.f90:14-20) are the Galerkin projections of the quadratic
products onto the free-slip y-basis

    u, w :  phi_0 = 1, phi_k = sin(k b y) (k odd), cos(k b y) (k even)      b = pi/2
    v    :  psi_k = cos(k b y) (k odd), sin(k b y) (k even),   k = 1..K0-1

(the y-expansions of ``velU``/``velV``/``velW``, modes.M4.f90:83-107).  The oracle derives the
projection tensors independently of the reference's expanded formulas, by Gauss-Legendre
quadrature on [-1, 1]; the tests check the result against the reference's own expressions
(golden vectors in tests/golden/, made by evaluating the Fortran expressions).
"""
from functools import lru_cache

import numpy as np

BETA = np.pi / 2.0  # d_beta, program/parameters.f90:55


def _phi(k, y):
    return np.cos(k * BETA * y) if k % 2 == 0 else np.sin(k * BETA * y)


def _dphi(k, y):
    return -k * BETA * np.sin(k * BETA * y) if k % 2 == 0 else k * BETA * np.cos(k * BETA * y)


def _psi(k, y):
    return np.cos(k * BETA * y) if k % 2 == 1 else np.sin(k * BETA * y)


def _dpsi(k, y):
    return -k * BETA * np.sin(k * BETA * y) if k % 2 == 1 else k * BETA * np.cos(k * BETA * y)


@lru_cache(maxsize=None)
def tensors(K0):
    """Return the projection tensors for K0 wall-normal modes.

    Gp[k,i,j] = <phi_k, phi_i phi_j>      (u*ux, w*uz products onto u/w modes: nluw)
    Gv[k,i,j] = <psi_k, phi_i psi_j>      (u*vx, w*vz onto v modes: nluv)
    Hp[k,i,j] = <phi_k, psi_i dphi_j>     (v * d/dy of u or w: nluyv)
    Hv[k,i,j] = <psi_k, psi_i dpsi_j>     (v * d/dy v: nlvvy)
    Ev[k,i,j] = <phi_k, psi_i psi_j>      (v*v onto the mean modes: nlvv)
    with <f, g> = (1/|f|^2) int_{-1}^{1} f g dy.  Index ranges: phi 0..K0-1, psi 1..K0-1
    (stored at 0..K0-2).
    """
    y, wq = np.polynomial.legendre.leggauss(96)
    ph = np.array([_phi(k, y) for k in range(K0)])
    dph = np.array([_dphi(k, y) for k in range(K0)])
    ps = np.array([_psi(k, y) for k in range(1, K0)])
    dps = np.array([_dpsi(k, y) for k in range(1, K0)])
    nph = np.einsum("kq,kq,q->k", ph, ph, wq)
    nps = np.einsum("kq,kq,q->k", ps, ps, wq)
    Gp = np.einsum("kq,iq,jq,q->kij", ph, ph, ph, wq) / nph[:, None, None]
    Gv = np.einsum("kq,iq,jq,q->kij", ps, ph, ps, wq) / nps[:, None, None]
    Hp = np.einsum("kq,iq,jq,q->kij", ph, ps, dph, wq) / nph[:, None, None]
    Hv = np.einsum("kq,iq,jq,q->kij", ps, ps, dps, wq) / nps[:, None, None]
    Ev = np.einsum("kq,iq,jq,q->kij", ph, ps, ps, wq) / nph[:, None, None]
    out = []
    for t in (Gp, Gv, Hp, Hv, Ev):
        t = t.copy()
        t[np.abs(t) < 1e-12] = 0.0
        out.append(t)
    return tuple(out)
