"""Seeded initial conditions (the reference's IC generator utils/randIC.f90 is not shipped).

gaussian_ic: every MPT coefficient with integer |k| = sqrt(m^2 + n^2) <= kmax is a complex
Gaussian times amp*exp(-|k|^2/decay); all others are zero.  The draws are made in a fixed
(n, m, k) order over the |k| <= kmax window, independent of the grid, so the same seed gives
the same low modes on every grid.  The n = 0 column is made Hermitian
(c(-m,0) = conj(c(m,0))), the (0,0) coefficients are real and psi_0(0,0) = 0 (the mode the
update pins to zero, velocity.f90:36-38).  The MPT representation is divergence-free by
construction, so no projection is needed.

spot_ic: the same spectrum, with each MPT potential multiplied in physical space by
exp(-r^2 / (2 w^2)) centred in the domain and truncated back to the retained modes.
"""
import numpy as np


def _window(kmax):
    for n in range(0, kmax + 1):
        for m in range(-kmax, kmax + 1):
            if m * m + n * n <= kmax * kmax:
                yield m, n


def gaussian_ic(p, seed, kmax=8, amp=0.3, decay=16.0):
    """p: RunParams-like object with K0, MM, NN.  Returns complex (NN, M, K)."""
    K0, MM, NN = p.K0, p.MM, p.NN
    K, M = 2 * K0 - 1, 2 * (MM - 1) + 1
    rng = np.random.Generator(np.random.PCG64(seed))
    c = np.zeros((NN, M, K), complex)
    for m, n in _window(kmax):
        draw = rng.standard_normal(K) + 1j * rng.standard_normal(K)
        if abs(m) >= MM or n >= NN:
            continue
        if n == 0 and m < 0:
            continue                      # filled from the Hermitian mirror below
        c[n, m % M, :] = draw * amp * np.exp(-(m * m + n * n) / decay)
    for m in range(1, MM):
        c[0, (-m) % M, :] = np.conj(c[0, m, :])
    c[0, 0, :] = c[0, 0, :].real
    c[0, 0, 0] = 0.0
    return c


def _to_phys(p, a):
    """2D real field per component from its half spectrum a (NN, M, nf) on the 3/2 grid."""
    X, Z, NN, MM, M = 3 * p.MM, 3 * p.NN, p.NN, p.MM, 2 * (p.MM - 1) + 1
    ms = np.arange(-(MM - 1), MM)
    t = np.zeros((NN, X, a.shape[2]), complex)
    t[:, ms % X, :] = a[:, ms % M, :]
    t = np.fft.ifft(t, axis=1) * X
    mid = np.zeros((X, Z // 2 + 1, a.shape[2]), complex)
    mid[:, :NN, :] = t.transpose(1, 0, 2)
    mid[:, 0, :] = mid[:, 0, :].real
    return np.fft.irfft(mid, n=Z, axis=1) * Z


def _to_spec(p, f):
    X, Z, NN, MM, M = 3 * p.MM, 3 * p.NN, p.NN, p.MM, 2 * (p.MM - 1) + 1
    mid = np.fft.rfft(f / (X * Z), axis=1)
    t = np.fft.fft(np.ascontiguousarray(mid[:, :NN, :].transpose(1, 0, 2)), axis=1)
    ms = np.arange(-(MM - 1), MM)
    out = np.zeros((NN, M, f.shape[2]), complex)
    out[:, ms % M, :] = t[:, ms % X, :]
    return out


def spot_ic(p, seed, width=20.0, kmax=8, amp=0.3, decay=16.0):
    c = gaussian_ic(p, seed, kmax=kmax, amp=amp, decay=decay)
    X, Z = 3 * p.MM, 3 * p.NN
    Lx, Lz = 2 * np.pi / p.alpha, 2 * np.pi / p.gamma
    x = np.arange(X) * Lx / X
    z = np.arange(Z) * Lz / Z
    env = np.exp(-((x[:, None] - Lx / 2) ** 2 + (z[None, :] - Lz / 2) ** 2) / (2 * width ** 2))
    f = _to_phys(p, c) * env[:, :, None]
    out = _to_spec(p, f)
    out[0, 0, 0] = 0.0
    return out
