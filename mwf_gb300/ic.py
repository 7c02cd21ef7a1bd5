"""Seeded initial conditions (the reference's IC generator utils/randIC.f90 is not shipped).

gaussian_ic: every MPT coefficient with integer |k| = sqrt(m^2 + n^2) <= kmax is a complex
Gaussian times amp*exp(-|k|^2/decay); all others are zero.  The draws are made in a fixed
(n, m, k) order over the |k| <= kmax window, independent of the grid, so the same seed gives
the same low modes on every grid.  The n = 0 column is made Hermitian
(c(-m,0) = conj(c(m,0))), the (0,0) coefficients are real and psi_0(0,0) = 0 (the mode the
update pins to zero, velocity.f90:36-38).  The MPT representation is divergence-free by
construction, so no projection is needed.

spot_ic: the localised spot of the M6 benchmark configuration: the same spectrum is turned into
the velocity field (u, v, w; var_mpt2spec, program/variables.f90:390-434, without the base
flow), which is multiplied in physical space by exp(-r^2 / (2 w^2)) centred in the domain,
truncated back to the retained modes and re-projected divergence-free by the inverse of
var_mpt2spec: phi_k from v_k and psi_k from the vertical vorticity (uvw_to_mpt).
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


def _wavenumbers(p):
    """alpha m per x slot (slot m > MM-1 holds m - M), gamma n per column, (-1)^k k beta per k."""
    MM, NN, K0 = p.MM, p.NN, p.K0
    M = 2 * (MM - 1) + 1
    ms = np.arange(M)
    m = np.where(ms < MM, ms, ms - M)
    beta = np.pi / 2
    k = np.arange(K0)
    return p.alpha * m, p.gamma * np.arange(NN), np.where(k % 2 == 1, -k, k) * beta


def mpt_to_uvw(p, c):
    """u, v, w spectral coefficients (NN, M, KK) of an MPT state (NN, M, K), the formulas of
    var_mpt2spec (program/variables.f90:390-434) without the laminar base flow:
        u_k = -i gamma n psi_k + i kappa_k alpha m phi_k,   v_k = h phi_k,
        w_k =  i alpha m psi_k + i kappa_k gamma n phi_k,
    h = (alpha m)^2 + (gamma n)^2, kappa_k = (-1)^k k beta, phi_0 = 0; at (m, n) = (0, 0) the mean
    flows u_k = psi_k, w_k = phi_k (k >= 1) and u_0 = w_0 = 0."""
    K0 = p.K0
    m1, n1, kap = _wavenumbers(p)
    M1 = m1[None, :, None]
    N1 = n1[:, None, None]
    c = np.asarray(c, complex)
    psi = c[:, :, :K0]
    phi = np.concatenate([np.zeros_like(c[:, :, :1]), c[:, :, K0:]], axis=2)
    h = M1 ** 2 + N1 ** 2
    u = -1j * N1 * psi + 1j * kap * M1 * phi
    v = (h * phi)[:, :, 1:]
    w = 1j * M1 * psi + 1j * kap * N1 * phi
    u[0, 0, :] = 0.0
    w[0, 0, :] = 0.0
    u[0, 0, 1:] = psi[0, 0, 1:]
    w[0, 0, 1:] = phi[0, 0, 1:]
    return np.concatenate([u, v, w], axis=2)


def uvw_to_mpt(p, s):
    """The inverse of mpt_to_uvw on divergence-free fields, and the projection of any u, v, w
    (NN, M, KK) onto the MPT representation: phi_k = v_k / h and psi_k = i (gamma n u_k -
    alpha m w_k) / h (the vertical vorticity over h) for (m, n) != (0, 0); the mean flows
    psi_k = u_k, phi_k = w_k (k >= 1) at (0, 0), psi_0(0, 0) = 0."""
    K0 = p.K0
    m1, n1, _ = _wavenumbers(p)
    M1 = m1[None, :, None]
    N1 = n1[:, None, None]
    s = np.asarray(s, complex)
    u, v, w = s[:, :, :K0], s[:, :, K0:2 * K0 - 1], s[:, :, 2 * K0 - 1:]
    h = M1 ** 2 + N1 ** 2
    h[0, 0, 0] = 1.0                            # (0, 0) is set separately below
    psi = 1j * (N1 * u - M1 * w) / h
    phi = v / h
    psi[0, 0, :] = 0.0
    psi[0, 0, 1:] = u[0, 0, 1:]
    phi[0, 0, :] = w[0, 0, 1:]
    return np.concatenate([psi, phi], axis=2)


def spot_ic(p, seed, width=20.0, kmax=8, amp=0.3, decay=16.0):
    """Localised spot: the Gaussian spectrum's velocity field times a Gaussian envelope of
    width `width` (exp(-r^2 / (2 width^2)), r measured from the centre of the domain),
    re-projected onto the MPT representation."""
    c = gaussian_ic(p, seed, kmax=kmax, amp=amp, decay=decay)
    X, Z = 3 * p.MM, 3 * p.NN
    Lx, Lz = 2 * np.pi / p.alpha, 2 * np.pi / p.gamma
    x = np.arange(X) * Lx / X
    z = np.arange(Z) * Lz / Z
    env = np.exp(-((x[:, None] - Lx / 2) ** 2 + (z[None, :] - Lz / 2) ** 2) / (2 * width ** 2))
    f = _to_phys(p, mpt_to_uvw(p, c)) * env[:, :, None]
    out = uvw_to_mpt(p, _to_spec(p, f))
    out[0, 0, 0] = 0.0
    return out
