"""Face-centred transforms (c_or_f = 'f', src/fft.f90:265-287 and
src/initsolver.f90:164-181, 188-246, 248-298) and odd-length ND/DN axes on the
GPU's FP64 solver, against the oracle.

Tolerance: relative L2 <= 1e-12 over every point (the points the face-centred
DD transform leaves untouched included: the oracle and the GPU both pass them
through, with lambda(n) = 0 where the reference leaves it unset).  The
coefficient tables (eigenvalues, tridiagonal a/b/c, boundary right-hand sides,
normfft) are bit-equal.  None of the cases is singular (a Dirichlet side, or an
ND/DN pair, in every column), so no mean is removed.
"""
import numpy as np
import pytest

from conftest import random_velocity, rel_l2, zgrid

pytestmark = pytest.mark.gpu

CASES = [
    ((33, 24, 16), "NNPPDD", "fcc", 0.0),   # REDFT00 in x (DFT of 64)
    ((32, 48, 20), "DDNNND", "fcc", 1.5),   # RODFT00 on 31 of 32 points in x (DFT of 64)
    ((48, 33, 12), "DNNNDD", "ffc", 0.0),   # RODFT01/RODFT10 in x, REDFT00 in y
    ((24, 32, 18), "NDDDNN", "ffc", 2.0),   # REDFT10/01 with ND eigenvalues in x, RODFT00 in y
    ((32, 32, 24), "PPPPND", "ccf", 1.0),   # face-centred z: Dirichlet top solves nz-1 levels
    ((32, 25, 16), "PPNNDD", "fff", 0.5),   # every axis face-centred
    ((40, 16, 17), "DDPPND", "fcf", 1.2),   # face z, Neumann bottom, Dirichlet top
    ((15, 16, 12), "NDPPDD", "ccc", 0.0),   # odd-length DCT-IV in x (DFT of 30)
    ((16, 21, 10), "PPDNNN", "ccc", 1.0),   # odd-length DST-IV in y (DFT of 42)
    ((45, 27, 9), "DNNDDD", "ccc", 0.0),    # both odd
]


@pytest.mark.parametrize("n,cbc,cf,gr", CASES, ids=[f"{c}-{f}-{n[0]}x{n[1]}x{n[2]}" for n, c, f, _ in CASES])
def test_gpu_face_and_odd_solver_matches_oracle(lib, oracle, n, cbc, cf, gr):
    rng = np.random.default_rng(sum(n) + len(cf))
    dzci, dzfi, dzc, dzf = zgrid(n[2], gr)
    dli = [n[0] * 1.0, n[1] * 1.3, n[2] * 1.0]
    bc = list(rng.uniform(-1, 1, 6))
    P = lib.initsolver(n, dli, 1, dzci, dzfi, cbc, bc, cf)
    S = oracle.SolverSetup(n, dli, 1, dzci, dzfi, cbc, bc, cf)
    assert np.array_equal(P.lambdaxy, S.lambdaxy)
    assert np.array_equal(P.a, S.a) and np.array_equal(P.b, S.b) and np.array_equal(P.c, S.c)
    assert P.normfft == S.normfft
    for a, b in ((P.rhsbx, S.rhsbx), (P.rhsby, S.rhsby), (P.rhsbz, S.rhsbz)):
        assert np.array_equal(a, b)
    f = rng.uniform(-1.0, 1.0, (n[2] + 2, n[1] + 2, n[0] + 2))
    ref = f.copy()
    S.solve(ref)
    got = f.copy()
    P.solver(got)
    e = rel_l2(got[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1])
    print(f"{cbc} {cf} {n}: rel L2 {e:.2e}")
    assert e <= 1e-12, e
    # halo untouched, as solver_cpu writes p(1:n) only
    assert np.array_equal(got[0], f[0]) and np.array_equal(got[:, :, -1], f[:, :, -1])
    # the FP64 solver only: the mixed path refuses with a clear status
    with pytest.raises(lib.FlutasError) as e:
        P.solve_mixed(f.copy(), tol=1e-8)
    assert e.value.code == lib.FLUTAS_EUNSUPPORTED


def test_gpu_odd_nd_projection_fp64(lib, oracle):
    """The fused FP64 projection on a grid with an odd-length ND axis (extended-FFT
    passes inside the projection) against the oracle's fillps, solve, boundp,
    correc, p update."""
    n, cbc = [15, 24, 20], "NDPPNN"
    rng = np.random.default_rng(15)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 1.0)
    dxi, dyi, dt, rho0 = 15.0, 24.0, 1e-3, 1.0
    P = lib.initsolver(n, [dxi, dyi, 20.0], 1, dzci, dzfi, cbc, [0.0] * 6, "ccc")
    S = oracle.SolverSetup(n, [dxi, dyi, 20.0], 1, dzci, dzfi, cbc, [0.0] * 6, "ccc")
    u, v, w = random_velocity(rng, n)
    pold = rng.standard_normal((n[2] + 2, n[1] + 2, n[0] + 2))
    uo, vo, wo = u.copy(), v.copy(), w.copy()
    phi = np.zeros_like(pold)
    oracle.fillps(n, 1, 1, dxi, dyi, 20.0, dzfi, 1 / dt, rho0, uo, vo, wo, phi)
    S.solve(phi)
    oracle.boundp(cbc, n, [0.0] * 6, 1, [1 / dxi, 1 / dyi, 1.0], dzc, dzf, phi)
    oracle.correc(n, 1, 1, dxi, dyi, 20.0, dzci, dt, rho0, phi, uo, vo, wo)
    po = pold.copy()
    po[1:-1, 1:-1, 1:-1] += phi[1:-1, 1:-1, 1:-1]
    oracle.boundp(cbc, n, [0.0] * 6, 1, [1 / dxi, 1 / dyi, 1.0], dzc, dzf, po)
    p = pold.copy()
    P.projection(1, dxi, dyi, dzci, dzfi, [0.0] * 6, dt, rho0, u, v, w, p, precision=0)
    for a, b in ((u, uo), (v, vo), (w, wo)):
        assert rel_l2(a, b) <= 1e-12
    assert rel_l2(p[1:-1, 1:-1, 1:-1] - pold[1:-1, 1:-1, 1:-1], phi[1:-1, 1:-1, 1:-1]) <= 1e-12
    with pytest.raises(lib.FlutasError) as e:
        P.projection(1, dxi, dyi, dzci, dzfi, [0.0] * 6, dt, rho0, u, v, w, p, precision=1, tol=1e-8)
    assert e.value.code == lib.FLUTAS_EUNSUPPORTED
