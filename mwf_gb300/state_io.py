"""The reference's netCDF state files (io.f90:122-340), read and written with scipy.

Format (classic netCDF): global attributes t, Re, alpha, gamma; dimensions N = NN, M = M,
K = K, ReIm = 2; variable ``mpt`` (double) with Fortran dimensions (K, M, N, ReIm), i.e.
C-order (ReIm, N, M, K), carrying integer attributes K, MM, NN.  Re is written first.
An optional ``onl`` variable of the same shape holds the AB2 history (a compatible
superset: the reference's loader only reads ``mpt``).
"""
import numpy as np
from scipy.io import netcdf_file


class StateFileError(RuntimeError):
    pass


def save_state(path, c, K0, MM, NN, t=0.0, Re=0.0, alpha=0.0, gamma=0.0, onl=None):
    K, M = 2 * K0 - 1, 2 * (MM - 1) + 1
    c = np.asarray(c)
    if c.shape != (NN, M, K):
        raise StateFileError(f"state shape {c.shape} != {(NN, M, K)}")
    with netcdf_file(path, "w", version=1) as f:
        f.t = np.float64(t)
        f.Re = np.float64(Re)
        f.alpha = np.float64(alpha)
        f.gamma = np.float64(gamma)
        f.createDimension("N", NN)
        f.createDimension("M", M)
        f.createDimension("K", K)
        f.createDimension("ReIm", 2)
        for name, arr in (("mpt", c), ("onl", onl)):
            if arr is None:
                continue
            v = f.createVariable(name, "d", ("ReIm", "N", "M", "K"))
            v.K = np.int32(K)
            v.MM = np.int32(MM)
            v.NN = np.int32(NN)
            v[0, :, :, :] = np.asarray(arr).real
            v[1, :, :, :] = np.asarray(arr).imag


def load_state(path, K0=None, MM=None, NN=None):
    """Returns (c, attrs).  Like io_load_mpt (io.f90:166-204) it stops on a size mismatch."""
    try:
        f = netcdf_file(path, "r", mmap=False)
    except (OSError, TypeError, ValueError) as e:
        raise StateFileError(f"state file not found or unreadable: {path}: {e}") from e
    with f:
        if "mpt" not in f.variables:
            raise StateFileError("Field mpt not found!")
        v = f.variables["mpt"]
        K_, MM_, NN_ = int(v.K), int(v.MM), int(v.NN)
        if K0 is not None and (K_ != 2 * K0 - 1 or MM_ != MM or NN_ != NN):
            raise StateFileError(f"wrong state size: K {K_}, MM {MM_}, NN {NN_}")
        data = np.array(v[:], dtype=np.float64)
        if data.shape != (2, NN_, 2 * (MM_ - 1) + 1, K_):
            raise StateFileError(f"mpt has shape {data.shape}")
        c = data[0] + 1j * data[1]
        attrs = {k: float(getattr(f, k)) for k in ("t", "Re", "alpha", "gamma") if hasattr(f, k)}
        if "onl" in f.variables:
            o = np.array(f.variables["onl"][:], dtype=np.float64)
            attrs["onl"] = o[0] + 1j * o[1]
    return c, attrs


# ---- text output in the reference's formats (io.f90) -------------------------------------

def fortran_e20_12(v):
    """Fortran's Ew.d edit descriptor for w = 20, d = 12 (the reference's '(2e20.12)' and
    '(6e20.12)'): optional minus sign, "0.", twelve digits, exponent "E+dd" (or "+ddd" without
    the E from 100 on), right-justified in 20 columns."""
    v = float(v)
    if v == 0.0:
        s = "-0.000000000000E+00" if np.signbit(v) else "0.000000000000E+00"
    elif not np.isfinite(v):
        s = "NaN" if np.isnan(v) else ("Infinity" if v > 0 else "-Infinity")
    else:
        sci = f"{abs(v):.11e}"                    # d.ddddddddddde+XX: 12 significant digits
        mant, ex = sci.split("e")
        ex = int(ex) + 1                          # 0.dddddddddddd x 10^ex
        digits = mant.replace(".", "")
        sign = "-" if v < 0 else ""
        es = "-" if ex < 0 else "+"
        s = f"{sign}0.{digits}E{es}{abs(ex):02d}" if -99 <= ex <= 99 else f"{sign}0.{digits}{es}{abs(ex):03d}"
    return f"{s:>20}"


def energy_row(t, E):
    """One row of vel_energy.dat: write(io_KE, '(2e20.12)') tim_t, E (io.f90:453-467)."""
    return fortran_e20_12(t) + fortran_e20_12(E)


def parse_energy_rows(text):
    """(t, E) pairs of vel_energy.dat text."""
    out = []
    for ln in text.splitlines():
        if ln.strip():
            out.append((float(ln[:20]), float(ln[20:40])))
    return out
