"""Shared fixtures and helpers.

Markers: ``gpu`` -- needs a CUDA device (the parity tests proper; run on the
GB300 machine).  Everything else runs on CPU.
"""
from __future__ import annotations

import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")


def have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if have_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def lib():
    """The CUDA library, built in-tree (fails loudly if it cannot be built)."""
    from flutas_gb300 import build as B
    B.build()
    import flutas_gb300 as F
    F.load()
    return F


def golden_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "kat_*.npz")))


def singular(cbc: str) -> bool:
    """x and y admit a zero eigenvalue and z is N/N or P/P: p is defined up to a constant."""
    return cbc[0:2] in ("PP", "NN") and cbc[2:4] in ("PP", "NN") and cbc[4:6] in ("NN", "PP")


def rel_l2(a, b, remove_mean=False):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if remove_mean:
        a = a - a.mean()
        b = b - b.mean()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def zgrid(nz, gr, lz=1.0, nh_d=1):
    """dzci, dzfi (1-nh_d:nz+nh_d) from the oracle's restatement of initgrid."""
    from oracle import oracle as O
    dzc, dzf, zc, zf = O.initgrid(nz, gr, lz, nh_d)
    return 1.0 / dzc, 1.0 / dzf, dzc, dzf


def compatible_rhs(rng, n, cbc, dzf, nh_d=1):
    """Random RHS (halo-1 array) that satisfies the solvability condition of singular cases."""
    nx, ny, nz = n
    f = rng.uniform(-1.0, 1.0, (nz, ny, nx))
    if singular(cbc):
        w = dzf[nh_d:nh_d + nz][:, None, None]
        f -= (f * w).sum() / (w.sum() * nx * ny)
    p = np.zeros((nz + 2, ny + 2, nx + 2))
    p[1:-1, 1:-1, 1:-1] = f
    return p


def random_velocity(rng, n, nh_u=1):
    nx, ny, nz = n
    shp = (nz + 2 * nh_u, ny + 2 * nh_u, nx + 2 * nh_u)
    return [rng.uniform(-1.0, 1.0, shp) for _ in range(3)]


def velocity_ghosts(u, v, w, n, cbc, nh_u=1):
    """Velocity ghosts as bounduvw leaves them for the pressure BCs of cbc:
    periodic directions are wrapped, N-pressure walls get zero normal velocity
    on the wall faces (src/bound.f90:17-144 semantics for no-slip walls)."""
    nx, ny, nz = n
    h = nh_u
    for f in (u, v, w):
        if cbc[0] == "P":
            f[:, :, :h] = f[:, :, nx:nx + h]
            f[:, :, h + nx:] = f[:, :, h:2 * h]
        if cbc[2] == "P":
            f[:, :h, :] = f[:, ny:ny + h, :]
            f[:, h + ny:, :] = f[:, h:2 * h, :]
        if cbc[4] == "P":
            f[:h] = f[nz:nz + h]
            f[h + nz:] = f[h:2 * h]
    if cbc[0] == "N":
        u[:, :, h - 1] = 0.0
        u[:, :, h + nx - 1] = 0.0
    if cbc[2] == "N":
        v[:, h - 1, :] = 0.0
        v[:, h + ny - 1, :] = 0.0
    if cbc[4] == "N":
        w[h - 1] = 0.0
        w[h + nz - 1] = 0.0
    return u, v, w
