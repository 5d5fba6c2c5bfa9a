"""Generates the known-answer fixtures in tests/golden/ (run from the repo root:
``python tests/golden/make_golden.py``).

The reference's own tests hold no golden vectors for the Poisson path (they
are end-to-end physics regressions), and the reference solver cannot be built
here (no gfortran, no FFTW).  These fixtures are exact discrete solutions
written in closed form instead: for each x/y BC pair the discrete eigenvectors
of the 3-point operator with the ghost rules of src/bound.f90 set_bc are
known (cos/sin of the cell-centre coordinate), with the eigenvalues of
src/initsolver.f90:122-186; along z any profile Z(k) works, because the RHS is
built by applying the z tridiagonal matrix of src/initsolver.f90:188-246
directly.  So p = sum_m c_m X_m(i) Y_m(j) Z_m(k) solves the discrete problem
exactly, and f = sum_m c_m X_m Y_m [(lx+ly) Z_m + A_z Z_m].  Only numpy is
used; nothing here shares code with the oracle or the CUDA kernels.
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def eigvec(pair: str, n: int, m: int):
    """Discrete eigenvector (cells i = 1..n) and unscaled eigenvalue, mode m."""
    xc = np.arange(1, n + 1) - 0.5
    if pair == "PP":
        v = np.cos(2 * np.pi * m * xc / n + 0.3 * m)
        lam = -4 * np.sin(np.pi * m / n) ** 2
    elif pair == "NN":
        v = np.cos(np.pi * m * xc / n)
        lam = -4 * np.sin(np.pi * m / (2 * n)) ** 2
    elif pair == "DD":
        v = np.sin(np.pi * (m + 1) * xc / n)
        lam = -4 * np.sin(np.pi * (m + 1) / (2 * n)) ** 2
    elif pair == "ND":
        v = np.cos(np.pi * (2 * m + 1) * xc / (2 * n))
        lam = -4 * np.sin(np.pi * (2 * m + 1) / (4 * n)) ** 2
    elif pair == "DN":
        v = np.sin(np.pi * (2 * m + 1) * xc / (2 * n))
        lam = -4 * np.sin(np.pi * (2 * m + 1) / (4 * n)) ** 2
    else:
        raise ValueError(pair)
    return v, lam


def zgrid(nz: int, gr: float, lz: float = 1.0):
    """Cell spacings with one ghost each side (tanh clustering at both walls)."""
    k = np.arange(0, nz + 1)
    z0 = k / nz
    zf = 0.5 * (1 + np.tanh((z0 - 0.5) * gr) / np.tanh(gr / 2)) * lz if gr else z0 * lz
    dzf = np.empty(nz + 2)
    dzf[1:nz + 1] = np.diff(zf)
    dzf[0], dzf[nz + 1] = dzf[1], dzf[nz]
    dzc = np.empty(nz + 2)
    dzc[0:nz + 1] = 0.5 * (dzf[0:nz + 1] + dzf[1:nz + 2])
    dzc[nz + 1] = dzc[nz]
    return 1.0 / dzc, 1.0 / dzf


def apply_az(zbc: str, Z, dzci, dzfi):
    nz = Z.size
    k = np.arange(1, nz + 1)
    a = dzfi[k] * dzci[k - 1]
    c = dzfi[k] * dzci[k]
    lo = {"P": Z[-1], "N": Z[0], "D": -Z[0]}[zbc[0]]
    hi = {"P": Z[0], "N": Z[-1], "D": -Z[-1]}[zbc[1]]
    zm = np.concatenate([[lo], Z[:-1]])
    zp = np.concatenate([Z[1:], [hi]])
    return a * zm - (a + c) * Z + c * zp


def make_case(name, n, cbc, gr, modes, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    dli = np.array([nx * 1.0, ny * 1.3, nz * 1.0])
    dzci, dzfi = zgrid(nz, gr)
    p = np.zeros((nz, ny, nx))
    f = np.zeros((nz, ny, nx))
    for (mx, my) in modes:
        X, lx = eigvec(cbc[0:2], nx, mx)
        Y, ly = eigvec(cbc[2:4], ny, my)
        lam = lx * dli[0] ** 2 + ly * dli[1] ** 2
        Z = rng.standard_normal(nz)
        coef = rng.uniform(0.5, 1.5)
        p += coef * np.einsum("k,j,i->kji", Z, Y, X)
        f += coef * np.einsum("k,j,i->kji", lam * Z + apply_az(cbc[4:6], Z, dzci, dzfi), Y, X)
    np.savez(os.path.join(HERE, f"kat_{name}.npz"), n=np.array(n), cbc=np.array(cbc), dli=dli,
             dzci=dzci, dzfi=dzfi, f=f, p=p)


CASES = [
    # name, n, cbc, z stretching, (mx, my) modes (none is the singular zero mode)
    ("pp_pp_nn_uniform", (16, 12, 10), "PPPPNN", 0.0, [(1, 2), (3, 0), (0, 5)]),
    ("pp_pp_nn_stretched", (16, 16, 12), "PPPPNN", 2.0, [(2, 1), (7, 3), (8, 8)]),
    ("nn_pp_nd_stretched", (12, 16, 9), "NNPPND", 2.0, [(1, 0), (5, 3), (11, 15)]),
    ("dd_nn_dd", (10, 12, 8), "DDNNDD", 1.5, [(0, 0), (4, 7), (9, 11)]),
    ("nd_dn_nn", (8, 10, 12), "NDDNNN", 0.0, [(0, 0), (3, 2), (7, 9)]),
    ("pp_dd_dn", (18, 14, 7), "PPDDDN", 1.0, [(0, 0), (4, 6), (9, 13)]),
    ("nn_nn_pp", (12, 10, 16), "NNNNPP", 0.0, [(1, 0), (2, 3), (11, 9)]),
    ("pp_pp_pp", (16, 16, 16), "PPPPPP", 0.0, [(1, 1), (3, 0), (5, 7)]),
    ("odd_sizes", (15, 9, 11), "NNPPNN", 2.0, [(1, 0), (4, 4), (14, 8)]),
    ("radix_mix", (48, 80, 6), "PPNNDD", 0.5, [(5, 3), (17, 40), (24, 79)]),
    ("radix_7_11", (28, 22, 5), "DDPPNN", 0.0, [(3, 1), (20, 11), (27, 21)]),
]


if __name__ == "__main__":
    for i, (name, n, cbc, gr, modes) in enumerate(CASES):
        make_case(name, n, cbc, gr, modes, seed=1000 + i)
    print(f"wrote {len(CASES)} fixtures to {HERE}")
