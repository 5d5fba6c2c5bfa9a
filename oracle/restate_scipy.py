"""Independent numpy/scipy.fft restatement of solver_cpu (src/solver_cpu.f90:20-115).

TEST INFRASTRUCTURE ONLY: used by the tests to cross-check the C oracle.  It
shares no code with it: the r2r transforms come from scipy.fft, whose
unnormalised ``dct``/``dst`` of types 1-4 equal FFTW's REDFT00/10/01/11 and
RODFT00/10/01/11, and R2HC/HC2R are built from ``rfft``/``irfft``.
Arrays use the layout of oracle/oracle.py: shape (nz+2, ny+2, nx+2), x fastest.
"""
from __future__ import annotations

import numpy as np
import scipy.fft as sf


def eigenvalues(n, bc, c_or_f="c"):
    """initsolver.f90:122-186 (natural order), unscaled."""
    l = np.arange(1, n + 1, dtype=np.float64)
    pair = bc[0] + bc[1]
    if pair == "PP":
        return -4.0 * np.sin((l - 1) * np.pi / n) ** 2
    if pair == "NN":
        return -4.0 * np.sin((l - 1) * np.pi / (2.0 * n)) ** 2
    if pair == "DD":
        lam = -4.0 * np.sin(l * np.pi / (2.0 * n)) ** 2
        if c_or_f == "f":
            lam[-1] = 0.0
        return lam
    if pair in ("ND", "DN"):
        return -4.0 * np.sin((2 * l - 1) * np.pi / (4.0 * n)) ** 2
    raise ValueError(pair)


def _r2hc(x, axis):
    n = x.shape[axis]
    X = sf.rfft(x, axis=axis)
    out = np.empty_like(x)
    idx = [slice(None)] * x.ndim
    for k in range(n // 2 + 1):
        idx[axis] = k
        src = [slice(None)] * x.ndim
        src[axis] = k
        out[tuple(idx)] = X[tuple(src)].real
    for k in range(1, (n - 1) // 2 + 1):
        idx[axis] = n - k
        src = [slice(None)] * x.ndim
        src[axis] = k
        out[tuple(idx)] = X[tuple(src)].imag
    return out


def _hc2r(h, axis):
    n = h.shape[axis]
    h = np.moveaxis(h, axis, -1)
    X = np.zeros(h.shape[:-1] + (n // 2 + 1,), dtype=np.complex128)
    X[..., 0] = h[..., 0]
    for k in range(1, (n - 1) // 2 + 1):
        X[..., k] = h[..., k] + 1j * h[..., n - k]
    if n % 2 == 0:
        X[..., n // 2] = h[..., n // 2]
    y = sf.irfft(X, n=n, axis=-1) * n
    return np.moveaxis(y, -1, axis)


def transform(x, bc, fwd, axis, c_or_f="c"):
    pair = bc[0] + bc[1]
    if c_or_f != "c":
        raise NotImplementedError("cell-centred only in this restatement")
    if pair == "PP":
        return _r2hc(x, axis) if fwd else _hc2r(x, axis)
    if pair == "NN":
        return sf.dct(x, type=2 if fwd else 3, axis=axis)
    if pair == "DD":
        return sf.dst(x, type=2 if fwd else 3, axis=axis)
    if pair == "ND":
        return sf.dct(x, type=4, axis=axis)
    if pair == "DN":
        return sf.dst(x, type=4, axis=axis)
    raise ValueError(pair)


def tridmatrix(bc, dzci, dzfi, nz, nh_d=1):
    k = np.arange(1, nz + 1)
    a = dzfi[k - 1 + nh_d] * dzci[k - 2 + nh_d]
    c = dzfi[k - 1 + nh_d] * dzci[k - 1 + nh_d]
    b = -(a + c)
    f = {"P": 0.0, "D": -1.0, "N": 1.0}
    b[0] += f[bc[0]] * a[0]
    b[-1] += f[bc[1]] * c[-1]
    return a, b, c


def thomas_batched(a, bb, c, rhs):
    """dgtsv_homebrewed (solver_cpu.f90:187-223) vectorised over the trailing axes."""
    n = rhs.shape[0]
    p = rhs.copy()
    d = np.empty_like(p)
    z = 1.0 / bb[0]
    d[0] = c[0] * z
    p[0] = p[0] * z
    for l in range(1, n - 1):
        z = 1.0 / (bb[l] - a[l] * d[l - 1])
        d[l] = c[l] * z
        p[l] = (p[l] - a[l] * p[l - 1]) * z
    z = bb[n - 1] - a[n - 1] * d[n - 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        last = np.where(z != 0.0, (p[n - 1] - a[n - 1] * p[n - 2]) / np.where(z != 0.0, z, 1.0), 0.0)
    p[n - 1] = last
    for l in range(n - 2, -1, -1):
        p[l] = p[l] - d[l] * p[l + 1]
    return p


def solve(f_interior, cbc, dli, dzci, dzfi, nh_d=1):
    """Solve the cell-centred problem for an interior RHS of shape (nz, ny, nx).

    Returns the interior pressure, normalised as solver_cpu does.
    """
    nz, ny, nx = f_interior.shape
    lx = eigenvalues(nx, cbc[0:2]) * dli[0] ** 2
    ly = eigenvalues(ny, cbc[2:4]) * dli[1] ** 2
    lam = ly[:, None] + lx[None, :]
    x = transform(f_interior, cbc[0:2], True, axis=2)
    x = transform(x, cbc[2:4], True, axis=1)
    a, b, c = tridmatrix(cbc[4:6], dzci, dzfi, nz, nh_d)
    if cbc[4:6] == "PP":
        raise NotImplementedError("periodic z is checked through the C oracle")
    bb = b[:, None, None] + lam[None, :, :]
    x = thomas_batched(a[:, None, None], bb, c[:, None, None], x)
    x = transform(x, cbc[2:4], False, axis=1)
    x = transform(x, cbc[0:2], False, axis=2)
    norm = 1.0
    for n, pair in ((nx, cbc[0:2]), (ny, cbc[2:4])):
        norm *= n if pair == "PP" else 2.0 * n
    return x / norm
