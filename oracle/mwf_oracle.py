"""FP64 CPU oracle for the MWF timestep hot path (test infrastructure, not the product).

Only ``tests/``, ``__graft_entry__.smoke`` and ``bench.py``'s CPU-baseline / reference legs may
import this module.  It restates, in numpy FP64, the reference's timestep routines so that
the CUDA path can be checked against them:

    tables            program/variables.f90:516-531   (var_precompute, wavenumber tables)
    lhsrhs            program/variables.f90:565-597   (var_LHSRHS)
    mpt2spec          program/variables.f90:390-434   (var_mpt2spec)
    addlam            program/velocity.f90:76-82      (vel_addlam)
    spec_grad         program/variables.f90:600-612   (var_spec_grad)
    spec2phys         program/transform.fftw5.f90:64-87, 33-59, 210-218 (tra_spec2phys)
    phys2spec         program/transform.fftw5.f90:122-145, 151-159      (tra_phys2spec)
    udotgradu         program/modes.M4.f90:14-36, program/modes.M6.f90:14-20 (helpers 22-79)
    spec2mpt          program/variables.f90:440-480   (var_spec2mpt)
    Solver.step       program/velocity.f90:21-41, 92-113 (vel_TS, vel_nonlinear)
    energy            program/velocity.f90:84-90, 115-126, 144-162 (vel_mpt2phys, epos, vel_energy)
    turbulent_count   program/io.f90:597-615          (io_writeVTK_txz threshold count)
    reflect masks     program/variables.f90:42-131    (var_uvreflect, var_wreflect, var_reflect)

Parity status: the reference ships no tests, golden vectors or state files, and it cannot be
built here (no Fortran compiler, FFTW3 or netCDF-Fortran), so the oracle is pinned only by
(a) golden vectors made by evaluating the reference's own mode-coupling expressions
(tests/golden/make_golden.py) and (b) physics known-answer tests.  The FFTW boundary is
**parity unpinned**: FFTW 3.3.8 is not vendored; the oracle uses numpy's pocketfft with
FFTW's conventions (backward = e^{+i}, forward = e^{-i}, unnormalised, c2r ignores the
imaginary part of the DC term).

Array layout (same memory order as the reference's Fortran arrays):
    MPT  c[n, m, k]   complex, shape (NN, M, K)   == Fortran mpt%Re/Im(K, 0:M-1, 0:NN-1)
    spec s[n, m, k]   complex, shape (NN, M, KK)  == Fortran spec%Re/Im(KK, 0:M-1, 0:NN-1)
    phys p[x, z, k]   real,    shape (X, Z, KK)   == Fortran phys%Re(KK, 0:3NN-1, 0:3MM-1)
"""
from dataclasses import dataclass, field

import numpy as np

from . import galerkin

PI = 3.1415926535897931  # d_PI, program/parameters.f90:14
BETA = PI / 2.0

# Host threads for the transforms (scipy.fft workers) and the pointwise term.  1 = numpy only.
_THREADS = 1


def set_threads(n):
    """Use n host threads (scipy.fft workers for the FFTs, thread chunks for the NL term)."""
    global _THREADS
    _THREADS = max(1, int(n))


def _fft(a, axis, inverse=False, real=None, n=None):
    if _THREADS > 1:
        import scipy.fft as sf
        if real == "r2c":
            return sf.rfft(a, axis=axis, workers=_THREADS)
        if real == "c2r":
            return sf.irfft(a, n=n, axis=axis, workers=_THREADS)
        return (sf.ifft if inverse else sf.fft)(a, axis=axis, workers=_THREADS)
    if real == "r2c":
        return np.fft.rfft(a, axis=axis)
    if real == "c2r":
        return np.fft.irfft(a, n=n, axis=axis)
    return (np.fft.ifft if inverse else np.fft.fft)(a, axis=axis)


@dataclass
class Params:
    """Runtime copy of the compile-time parameters of program/parameters.f90:7-72."""
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
    theta: float = 0.0           # radians (d_theta = d_thdeg/180*pi)
    reflect: bool = False
    uvreflect: bool = False
    wreflect: bool = False

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


# ----------------------------------------------------------------------------------------
# tables: program/variables.f90:516-531
# ----------------------------------------------------------------------------------------
def tables(p: Params):
    M, MM, NN, K0 = p.M, p.MM, p.NN, p.K0
    m1 = np.zeros(M)
    m2 = np.zeros(M)
    for m in range(MM):
        if m > 0:
            m1[M - m] = -p.alpha * m
            m2[M - m] = -p.alpha * m * p.alpha * m
        m1[m] = p.alpha * m
        m2[m] = -p.alpha * m * p.alpha * m
    n = np.arange(NN, dtype=float)
    n2 = -p.gamma * n * p.gamma * n
    n1 = p.gamma * n
    k = np.arange(K0)
    k1 = (-1.0) ** k * k * BETA
    k2 = -k * k * BETA * BETA * 1.0
    return m1, m2, n1, n2, k1, k2


# ----------------------------------------------------------------------------------------
# LHS/RHS of the implicit update: program/variables.f90:565-597.  The k loop runs in the
# reference's order so that the slot shared by psi_{K0-1} and phi_0 (index K0) ends with
# the psi_{K0-1} value, and the 0/0 at (m,n,k)=(0,0,0) is overwritten as in the reference.
# ----------------------------------------------------------------------------------------
def lhsrhs(p: Params):
    m1, m2, n1, n2, k1t, k2t = tables(p)
    NN, M, K, K0 = p.NN, p.M, p.K, p.K0
    L = np.zeros((NN, M, K))
    R = np.zeros((NN, M, K))
    m2g = m2[None, :]
    n2g = n2[:, None]
    mean = np.zeros((NN, M), bool)
    mean[0, 0] = True
    with np.errstate(divide="ignore", invalid="ignore"):
        for k in range(K0):
            a, b = k, k + K0 - 1               # 0-based slots of k1=k+1, k2=k+K0
            lap = m2g + k2t[k] + n2g
            hlap = m2g + n2g
            ilap16 = p.hypo / (m2g + k2t[k] + n2g)
            if p.dragall or k == 0:
                tvl = 1.0 - p.dt * (lap / p.Re + ilap16 - p.drag)
            else:
                tvl = 1.0 - p.dt * (lap / p.Re + ilap16)
            if p.dragall:
                lk2 = tvl * hlap * lap + p.dt * (p.vdrag - p.drag) * hlap * hlap
            else:
                lk2 = tvl * hlap * lap
            L[:, :, a] = np.where(mean, tvl, tvl * hlap)
            L[:, :, b] = np.where(mean, tvl, lk2)
            R[:, :, a] = np.where(mean, 1.0, hlap)
            R[:, :, b] = np.where(mean, 1.0, hlap * lap)
            L[0, 0, 0] = 1.0
            R[0, 0, 0] = 0.0
    return L, R


# ----------------------------------------------------------------------------------------
# MPT <-> uvw maps
# ----------------------------------------------------------------------------------------
def mpt2spec(p: Params, c):
    """program/variables.f90:390-434 (var_mpt2spec)."""
    m1, m2, n1, n2, k1t, _ = tables(p)
    NN, M, K0, KK = p.NN, p.M, p.K0, p.KK
    s = np.zeros((NN, M, KK), complex)
    M1 = m1[None, :]
    N1 = n1[:, None]
    H = m2[None, :] + n2[:, None]
    for k in range(K0):
        a, b, d = k, k + K0 - 1, k + 2 * K0 - 1     # k1, k2, k3 (0-based)
        psi, phi = c[:, :, a], c[:, :, b]
        # s(k1) = i*(-gamma n psi + k1 alpha m phi)
        s[:, :, a] = (-(-psi.imag * N1 + phi.imag * k1t[k] * M1)
                      + 1j * (-psi.real * N1 + phi.real * k1t[k] * M1))
        s[:, :, b] = -phi.real * H - 1j * (phi.imag * H)
        s[:, :, d] = (-(psi.imag * M1 + phi.imag * k1t[k] * N1)
                      + 1j * (psi.real * M1 + phi.real * k1t[k] * N1))
    s[0, 0, 0] = 0.0
    s[0, 0, 2 * K0 - 1] = 0.0
    for k in range(1, K0):
        a, b, d = k, k + K0 - 1, k + 2 * K0 - 1
        s[0, 0, a] = c[0, 0, a]
        s[0, 0, d] = c[0, 0, b]
    return s


def addlam(p: Params, s):
    """program/velocity.f90:76-82 (vel_addlam)."""
    s = s.copy()
    s[0, 0, 1] += np.cos(p.theta)
    s[0, 0, 2 * p.K0] += np.sin(p.theta)
    return s


def spec_grad(p: Params, s):
    """program/variables.f90:600-612 (var_spec_grad): ux = i alpha m s, uz = i gamma n s."""
    m1, _, n1, _, _, _ = tables(p)
    ux = (-s.imag * m1[None, :, None]) + 1j * (s.real * m1[None, :, None])
    uz = (-s.imag * n1[:, None, None]) + 1j * (s.real * n1[:, None, None])
    return ux, uz


def spec2mpt(p: Params, s):
    """program/variables.f90:440-480 (var_spec2mpt)."""
    m1, m2, n1, n2, k1t, _ = tables(p)
    NN, M, K0, K = p.NN, p.M, p.K0, p.K
    c = np.zeros((NN, M, K), complex)
    M1 = m1[None, :]
    N1 = n1[:, None]
    H = m2[None, :] + n2[:, None]
    for k in range(K0):
        a, b, d = k, k + K0 - 1, k + 2 * K0 - 1
        su, sv, sw = s[:, :, a], s[:, :, b], s[:, :, d]
        re2 = -(su.imag * M1 * k1t[k] + sw.imag * N1 * k1t[k]) + sv.real * H
        im2 = (su.real * M1 * k1t[k] + sw.real * N1 * k1t[k]) + sv.imag * H
        c[:, :, b] = re2 + 1j * im2
        re1 = sw.imag * M1 - su.imag * N1
        im1 = -(sw.real * M1 - su.real * N1)
        c[:, :, a] = re1 + 1j * im1
    c[0, 0, 0] = 0.0
    for k in range(1, K0):
        a, b, d = k, k + K0 - 1, k + 2 * K0 - 1
        c[0, 0, a] = -s[0, 0, a]
        c[0, 0, b] = -s[0, 0, d]
    return c


# ----------------------------------------------------------------------------------------
# Transforms (FFTW conventions restated with numpy's pocketfft)
# ----------------------------------------------------------------------------------------
def _mrange(p):
    return np.arange(-(p.M - p.MM), p.MM)          # m = -(i_M-i_MM) .. i_MM1


def spec2phys(p: Params, s):
    """program/transform.fftw5.f90:64-87: pad m to 3MM, c2c e^{+i}; pad n to 3NN/2+1, c2r."""
    X, Z, NN = p.X, p.Z, p.NN
    nf = s.shape[2]
    ms = _mrange(p)
    a = np.zeros((NN, X, nf), complex)
    a[:, ms % X, :] = s[:, ms % p.M, :]
    a = _fft(a, 1, inverse=True) * X                # unnormalised backward (sgn=+1)
    mid = np.zeros((X, Z // 2 + 1, nf), complex)
    mid[:, :NN, :] = a.transpose(1, 0, 2)
    mid[:, 0, :] = mid[:, 0, :].real                # c2r uses Re of the DC term (FFTW)
    return _fft(mid, 1, real="c2r", n=Z) * Z      # (X, Z, nf)


def phys2spec(p: Params, ph):
    """program/transform.fftw5.f90:122-145: scale 1/(3MM*3NN), r2c e^{-i}, c2c e^{-i}, truncate."""
    X, Z, NN = p.X, p.Z, p.NN
    scale = 1.0 / float(X * Z)
    mid = _fft(scale * ph, 1, real="r2c")           # (X, Z//2+1, nf)
    t = np.ascontiguousarray(mid[:, :NN, :].transpose(1, 0, 2))
    t = _fft(t, 1)
    ms = _mrange(p)
    s = np.zeros((NN, p.M, ph.shape[2]), complex)
    s[:, ms % p.M, :] = t[:, ms % X, :]
    return s


# ----------------------------------------------------------------------------------------
# Mode coupling
# ----------------------------------------------------------------------------------------
def split_uvw(K0, a):
    """Split the KK y-coefficients of a point: u 0..K0-1, v 1..K0-1, w 0..K0-1."""
    return a[..., :K0], a[..., K0:2 * K0 - 1], a[..., 2 * K0 - 1:]


def udotgradu(K0, v, vx, vz):
    """u.grad(u) projected onto the y-modes (modes.M4.f90:30-36 / modes.M6.f90:14-20).

    v, vx, vz: (..., KK) physical-space y-coefficients of u, d/dx u, d/dz u.
    """
    if _THREADS > 1 and v.ndim >= 2 and v.shape[0] >= 2 * _THREADS:
        from concurrent.futures import ThreadPoolExecutor
        chunks = np.array_split(np.arange(v.shape[0]), _THREADS)
        with ThreadPoolExecutor(_THREADS) as ex:
            parts = list(ex.map(lambda ix: _udotgradu(K0, v[ix], vx[ix], vz[ix]), chunks))
        return np.concatenate(parts, axis=0)
    return _udotgradu(K0, v, vx, vz)


def _udotgradu(K0, v, vx, vz):
    Gp, Gv, Hp, Hv, _ = galerkin.tensors(K0)
    u, vv, w = split_uvw(K0, v)
    ux, vxx, wx = split_uvw(K0, vx)
    uz, vzz, wz = split_uvw(K0, vz)
    e = np.einsum
    out_u = e("kij,...i,...j->...k", Gp, u, ux) + e("kij,...i,...j->...k", Hp, vv, u) \
        + e("kij,...i,...j->...k", Gp, w, uz)
    out_v = e("kij,...i,...j->...k", Gv, u, vxx) + e("kij,...i,...j->...k", Hv, vv, vv) \
        + e("kij,...i,...j->...k", Gv, w, vzz)
    out_w = e("kij,...i,...j->...k", Gp, u, wx) + e("kij,...i,...j->...k", Hp, vv, w) \
        + e("kij,...i,...j->...k", Gp, w, wz)
    return np.concatenate([out_u, out_v, out_w], axis=-1)


def epos(K0, a):
    """program/velocity.f90:115-126: y-mean of u^2+v^2+w^2 at each physical point."""
    Gp, _, _, _, Ev = galerkin.tensors(K0)
    u, v, w = split_uvw(K0, a)
    return (np.einsum("ij,...i,...j->...", Gp[0], u, u)
            + np.einsum("ij,...i,...j->...", Ev[0], v, v)
            + np.einsum("ij,...i,...j->...", Gp[0], w, w))


def spectrum_maxima(p: Params, c):
    """io_save_Uspec (io.f90:345-372): max |u,v,w coefficient| per |m| (0..MM-1) and per n,
    with the modulus computed as the reference writes it, dsqrt(dRe*dRe + dIm*dIm)."""
    s = mpt2spec(p, c)
    a = np.sqrt(s.real * s.real + s.imag * s.imag).max(axis=2)     # (NN, M)
    n_max = a.max(axis=1)
    m_abs = np.array([m if m <= p.MM - 1 else p.M - m for m in range(p.M)])
    m_max = np.zeros(p.MM)
    for m in range(p.M):
        m_max[m_abs[m]] = max(m_max[m_abs[m]], a[:, m].max())
    return m_max, n_max


def remap_x(p: Params, c, factor):
    """var_quadX (variables.f90:168-185) for any factor, in its loop order: the coefficient of
    x wavenumber m moves to slot factor*m (m <= MM-1) or M - factor*(M - m) (negative m),
    skipped when the positive target passes MM-1 or the negative one falls below MM-1.
    var_doubleX (147-165) is the same routine with factor 2, except that its negative branch
    computes M - 2*(m - M), which lies past the end of the array for every negative m; the
    restatement uses quadX's mirror rule for it.  Kept from the reference: a negative target
    of exactly MM-1 (wavenumber -MM, when factor divides MM) overwrites the positive mode in
    that slot, since negative m come later in the loop."""
    out = np.zeros_like(c)
    for m in range(p.M):
        if m <= p.MM - 1:
            mm = factor * m
            if mm > p.MM - 1:
                continue
        else:
            mm = p.M - factor * (p.M - m)
            if mm < p.MM - 1:
                continue
        out[:, mm, :] = c[:, m, :]
    return out


def blend(c1, c2, d):
    """utils/interpstate.f90:32-33: (1 - d) * state1 + d * state2, per Re and Im part."""
    e = 1.0 - d
    return (e * c1.real + d * c2.real) + 1j * (e * c1.imag + d * c2.imag)


_SM_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_SM_M1 = np.uint64(0xBF58476D1CE4E5B9)
_SM_M2 = np.uint64(0x94D049BB133111EB)


def _splitmix64(x):
    x = np.asarray(x, np.uint64) + _SM_GAMMA
    x = (x ^ (x >> np.uint64(30))) * _SM_M1
    x = (x ^ (x >> np.uint64(27))) * _SM_M2
    return x ^ (x >> np.uint64(31))


def add_noise(p: Params, c, scale, seed):
    """var_randadd (variables.f90:253-269): scale * r added to Re and Im of every coefficient
    with m != 0 and n != 0, r uniform in [0, 1).  The reference's r comes from Fortran's
    RANDOM_NUMBER; the device kernel and this restatement both draw r as the top 53 bits of
    SplitMix64(seed ^ SplitMix64(i)), i = 2e (Re) or 2e + 1 (Im), e the coefficient's index in
    the reference order (k fastest, then m, then n)."""
    NN, M, K = c.shape
    e = np.arange(NN * M * K, dtype=np.uint64).reshape(NN, M, K)
    s = np.uint64(seed)
    with np.errstate(over="ignore"):
        r_re = (_splitmix64(s ^ _splitmix64(np.uint64(2) * e)) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
        r_im = (_splitmix64(s ^ _splitmix64(np.uint64(2) * e + np.uint64(1))) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    live = np.ones((NN, M, 1), bool)
    live[0] = False
    live[:, 0] = False
    re = np.where(live, c.real + scale * r_re, c.real)
    im = np.where(live, c.imag + scale * r_im, c.imag)
    return re + 1j * im


def phys_field(p: Params, c):
    """vel_mpt2phys (velocity.f90:84-90): the perturbation velocity on the grid, in the
    reference's phys order (KK, Z, X) with the field index fastest: returned as (X, Z, KK)."""
    return spec2phys(p, mpt2spec(p, c))


def history(p: Params, c, y, n_probes=32):
    """vel_history (velocity.f90:164-180) with velU/velV/velW (modes.M4.f90:83-107,
    modes.M6.f90:81-111): at x = 0 and z index ji = j * Z / n_probes + 1 (integer division), the position
    ji * Lz / Z and u, v, w at height y.  Returns H as (n_probes, 4)."""
    ph = phys_field(p, c)
    K0 = p.K0
    beta = np.pi / 2.0
    bu = np.array([1.0] + [np.sin(k * beta * y) if k % 2 else np.cos(k * beta * y) for k in range(1, K0)])
    bv = np.array([np.cos(k * beta * y) if k % 2 else np.sin(k * beta * y) for k in range(1, K0)])
    out = np.zeros((n_probes, 4))
    Lz = 2.0 * np.pi / p.gamma
    for j in range(n_probes):
        ji = j * p.Z // n_probes + 1
        V = ph[0, ji]
        out[j, 0] = ji * Lz / p.Z
        out[j, 1] = bu @ V[:K0]
        out[j, 2] = bv @ V[K0:2 * K0 - 1]
        out[j, 3] = bu @ V[2 * K0 - 1:]
    return out


def turbulent_count(p: Params, c, ct):
    """io_writeVTK_txz (io.f90:597-615) on the full grid: points with epos > ct of the
    perturbation field; also returns the physical-space energy.  The reference's turbulent
    fraction is count / ((X+1)(Z+1)) (io.f90:615)."""
    P = spec2phys(p, mpt2spec(p, c))
    e = epos(p.K0, P)
    return int(np.sum(e > ct)), float(np.sum(e) / (p.X * p.Z))


# ----------------------------------------------------------------------------------------
# Symmetry masks (off by default): program/variables.f90:42-131, velocity.f90:68-74
# ----------------------------------------------------------------------------------------
def _neg_m_index(p):
    m = np.arange(p.M)
    return np.where(m > p.MM - 1, np.abs(m - p.M), m)


def uvreflect(p: Params, c):
    assert p.K0 == 4, "the reference's var_uvreflect hard-codes K=7"
    c = c.copy()
    mm = _neg_m_index(p)
    for n in range(p.NN):
        for m in range(p.M):
            if m == 0:
                if n == 0:
                    c[n, m, [0, 2, 4, 6]] = 1j * c[n, m, [0, 2, 4, 6]].imag
                else:
                    c[n, m, [0, 2, 4, 6]] = 0
            elif m > p.MM - 1:
                sgn = np.array([-1, 1, -1, 1, -1, 1, -1.0])
                c[n, m, :] = sgn * c[n, mm[m], :]
    return c


def wreflect(p: Params, c):
    assert p.K0 == 4, "the reference's var_wreflect hard-codes K=7"
    c = c.copy()
    mm = _neg_m_index(p)
    for n in range(p.NN):
        for m in range(p.M):
            if n == 0:
                if m == 0:
                    c[n, m, 4:7] = 1j * c[n, m, 4:7].imag
                else:
                    c[n, m, 0:4] = 0
            elif m > p.MM - 1:
                src = c[n, mm[m], :]
                out = np.empty(7, complex)
                out[0:4] = -src[0:4].real + 1j * src[0:4].imag
                out[4:7] = src[4:7].real - 1j * src[4:7].imag
                c[n, m, :] = out
    return c


def reflect(p: Params, c):
    assert p.K0 == 4, "the reference's var_reflect hard-codes K=7"
    c = c.copy()
    for n in range(p.NN):
        for m in range(p.M):
            if m == 0 and n == 0:
                for k in (0, 2, 5):
                    c[n, m, k] = 1j * c[n, m, k].imag
            else:
                for k in (0, 2, 5):
                    c[n, m, k] = c[n, m, k].real
                for k in (1, 3, 4, 6):
                    c[n, m, k] = 1j * c[n, m, k].imag
    return c


def imposesym(p: Params, c):
    if p.reflect:
        c = reflect(p, c)
    if p.uvreflect:
        c = uvreflect(p, c)
    if p.wreflect:
        c = wreflect(p, c)
    return c


# ----------------------------------------------------------------------------------------
# Timestepper
# ----------------------------------------------------------------------------------------
def nonlinear(p: Params, c):
    """program/velocity.f90:92-113 (vel_nonlinear)."""
    u = addlam(p, mpt2spec(p, c))
    ux, uz = spec_grad(p, u)
    P = spec2phys(p, u)
    PX = spec2phys(p, ux)
    PZ = spec2phys(p, uz)
    ans = udotgradu(p.K0, P, PX, PZ)
    return spec2mpt(p, phys2spec(p, ans))


def energy(p: Params, c):
    """program/velocity.f90:144-162 on vel_mpt2phys(vel_c) (perturbation only, no addlam)."""
    P = spec2phys(p, mpt2spec(p, c))
    return float(np.sum(epos(p.K0, P)) / (p.X * p.Z))


@dataclass
class Solver:
    """Module state of program/velocity.f90:15-17 with vel_TS / vel_precompute semantics."""
    p: Params
    c: np.ndarray
    onl: np.ndarray = None
    nst: bool = True
    lhs: np.ndarray = field(default=None, repr=False)
    rhs: np.ndarray = field(default=None, repr=False)

    def __post_init__(self):
        self.c = np.array(self.c, dtype=complex)
        self.lhs, self.rhs = lhsrhs(self.p)
        if self.onl is None:
            self.onl = np.zeros_like(self.c)

    def step(self, n=1):
        """vel_TS (program/velocity.f90:21-41), n times (with vel_imposesym before each)."""
        p = self.p
        for _ in range(n):
            self.c = imposesym(p, self.c)
            nl = nonlinear(p, self.c)
            if self.nst:
                self.onl = nl.copy()
                self.nst = False
            c2 = self.rhs * self.c
            c2 = c2 + p.dt / 2.0 * (3.0 * nl - self.onl)
            c2 = c2 / self.lhs
            c2[0, 0, 0] = 1j * c2[0, 0, 0].imag
            self.onl = nl
            self.c = c2
        return self.c

    def energy(self):
        return energy(self.p, self.c)
