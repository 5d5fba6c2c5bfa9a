"""CPU tests of the FP64 oracle (the CUDA path is checked against it).

The oracle is pinned three ways: (1) every r2r kind against FFTW's published
O(n^2) definitions; (2) the whole solver against the closed-form discrete
known answers in tests/golden/; (3) against an independent scipy.fft
restatement.  Then the projection (fillps -> solver -> boundp -> correc) must
leave a divergence-free field (src/chkdiv.f90 criterion).
"""
import numpy as np
import pytest

from conftest import (compatible_rhs, golden_cases, random_velocity, rel_l2, singular,
                      velocity_ghosts, zgrid)


def r2r_direct(kind, x):
    """FFTW's unnormalised r2r definitions, summed directly."""
    from oracle import oracle as O
    n = x.size
    j = np.arange(n)[None, :]
    k = np.arange(n)[:, None]
    if kind == O.R2HC:
        X = np.exp(-2j * np.pi * j * k / n) @ x
        out = np.empty(n)
        for kk in range(n // 2 + 1):
            out[kk] = X[kk].real
        for kk in range(1, (n - 1) // 2 + 1):
            out[n - kk] = X[kk].imag
        return out
    if kind == O.HC2R:
        Z = np.zeros(n, complex)
        Z[0] = x[0]
        for kk in range(1, (n - 1) // 2 + 1):
            Z[kk] = x[kk] + 1j * x[n - kk]
            Z[n - kk] = x[kk] - 1j * x[n - kk]
        if n % 2 == 0:
            Z[n // 2] = x[n // 2]
        return (np.exp(2j * np.pi * j.T * k.T / n) @ Z).real
    if kind == O.REDFT10:
        return 2 * (np.cos(np.pi * (j + 0.5) * k / n) @ x)
    if kind == O.REDFT01:
        return x[0] + 2 * (np.cos(np.pi * j[:, 1:] * (k + 0.5) / n) @ x[1:])
    if kind == O.REDFT11:
        return 2 * (np.cos(np.pi * (j + 0.5) * (k + 0.5) / n) @ x)
    if kind == O.RODFT10:
        return 2 * (np.sin(np.pi * (j + 0.5) * (k + 1) / n) @ x)
    if kind == O.RODFT01:
        return (-1.0) ** k[:, 0] * x[n - 1] + 2 * (np.sin(np.pi * (j[:, :-1] + 1) * (k + 0.5) / n) @ x[:-1])
    if kind == O.RODFT11:
        return 2 * (np.sin(np.pi * (j + 0.5) * (k + 0.5) / n) @ x)
    if kind == O.REDFT00:
        return x[0] + (-1.0) ** k[:, 0] * x[n - 1] + 2 * (np.cos(np.pi * j[:, 1:-1] * k / (n - 1)) @ x[1:-1])
    if kind == O.RODFT00:
        return 2 * (np.sin(np.pi * (j + 1) * (k + 1) / (n + 1)) @ x)
    raise ValueError(kind)


@pytest.mark.parametrize("n", [2, 3, 5, 8, 12, 17, 48, 64, 97])
def test_r2r_matches_fftw_definitions(oracle, n):
    O = oracle
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    for kind in (O.R2HC, O.HC2R, O.REDFT10, O.REDFT01, O.REDFT11, O.RODFT10, O.RODFT01, O.RODFT11,
                 O.REDFT00, O.RODFT00):
        ref = r2r_direct(kind, x)
        got = O.r2r(kind, x)
        assert np.abs(got - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max()), kind


@pytest.mark.parametrize("fn", golden_cases(), ids=lambda s: s.split("kat_")[-1][:-4])
def test_oracle_known_answers(oracle, fn):
    d = np.load(fn)
    n = [int(x) for x in d["n"]]
    cbc = str(d["cbc"])
    S = oracle.SolverSetup(n, d["dli"], 1, d["dzci"], d["dzfi"], cbc, [0] * 6, "ccc")
    p = np.zeros((n[2] + 2, n[1] + 2, n[0] + 2))
    p[1:-1, 1:-1, 1:-1] = d["f"]
    S.solve(p)
    assert rel_l2(p[1:-1, 1:-1, 1:-1], d["p"], remove_mean=singular(cbc)) <= 1e-13


CBCS = ["PPPPNN", "NNPPND", "DDNNDD", "NDDNNN", "PPDDDN", "NNNNNN", "DNNDDN"]


@pytest.mark.parametrize("cbc", CBCS)
@pytest.mark.parametrize("n,gr", [((8, 6, 5), 0.0), ((12, 10, 9), 2.0), ((15, 9, 7), 1.0)])
def test_oracle_vs_scipy(oracle, cbc, n, gr):
    from oracle import restate_scipy as R
    if cbc[0:2] in ("ND", "DN") and n[0] % 2:
        pytest.skip("scipy restatement and GPU need even n for DCT-IV; oracle covered by KATs")
    rng = np.random.default_rng(7)
    dzci, dzfi, dzc, dzf = zgrid(n[2], gr)
    dli = [n[0] * 1.0, n[1] * 0.9, 1.0]
    S = oracle.SolverSetup(n, dli, 1, dzci, dzfi, cbc, [0] * 6, "ccc")
    p = compatible_rhs(rng, n, cbc, dzf)
    f = p[1:-1, 1:-1, 1:-1].copy()
    S.solve(p)
    ref = R.solve(f, cbc, dli, dzci, dzfi)
    assert rel_l2(p[1:-1, 1:-1, 1:-1], ref, remove_mean=singular(cbc)) <= 1e-13
    # and the solution satisfies the 7-point problem
    fh = np.zeros_like(p)
    fh[1:-1, 1:-1, 1:-1] = f
    r = oracle.residual(n, cbc, dli[0], dli[1], 1, dzci, dzfi, fh, p)
    assert np.linalg.norm(r) <= 1e-12 * np.linalg.norm(f)


def test_oracle_initsolver_tables(oracle):
    n = [8, 6, 5]
    dzci, dzfi, _, _ = zgrid(5, 1.5)
    S = oracle.SolverSetup(n, [8.0, 6.0, 5.0], 1, dzci, dzfi, "PPNNND", [0, 0, 0, 0, 1.0, 2.0], "ccc")
    lx = -4 * np.sin(np.arange(8) * np.pi / 8) ** 2 * 64
    ly = -4 * np.sin(np.arange(6) * np.pi / 12) ** 2 * 36
    assert np.allclose(S.lambdaxy, ly[:, None] + lx[None, :], rtol=0, atol=1e-12)
    k = np.arange(1, 6)
    a = dzfi[k] * dzci[k - 1]
    c = dzfi[k] * dzci[k]
    assert np.allclose(S.a, a) and np.allclose(S.c, c)
    b = -(a + c)
    b[0] += a[0]     # N bottom
    b[-1] -= c[-1]   # D top
    assert np.allclose(S.b, b)
    assert S.normfft == pytest.approx(1.0 / (8 * 12))
    # bc_rhs: N bottom with value 1 -> +dzc(0)*1/dzc(0)/dzf(1); D top value 2 -> -2*2/dzc(n)/dzf(n)
    assert np.allclose(S.rhsbz[0], 1.0 * dzfi[1])
    assert np.allclose(S.rhsbz[1], -4.0 * dzci[5] * dzfi[5])


@pytest.mark.parametrize("cbc,nh_u", [("PPPPNN", 1), ("NNPPNN", 1), ("NNNNNN", 1), ("PPPPNN", 3)])
def test_oracle_projection_is_divergence_free(oracle, cbc, nh_u):
    """fillps -> updt_rhs_b -> solver -> boundp -> correc; chkdiv max |div| <= 1e-11 U/dx."""
    O = oracle
    n = [16, 12, 10]
    rng = np.random.default_rng(3)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 1.5, nh_d=nh_u)
    dxi, dyi = 16.0, 12.0
    u, v, w = velocity_ghosts(*random_velocity(rng, n, nh_u), n, cbc, nh_u)
    S = O.SolverSetup(n, [dxi, dyi, 1.0], nh_u, dzci, dzfi, cbc, [0] * 6, "ccc")
    dt, rho0 = 1e-3, 1.0
    p = np.zeros((n[2] + 2, n[1] + 2, n[0] + 2))
    O.fillps(n, nh_u, nh_u, dxi, dyi, 1.0, dzfi, 1.0 / dt, rho0, u, v, w, p)
    O.updt_rhs_b(n, "ccc", cbc, S.rhsbx, S.rhsby, S.rhsbz, p)
    S.solve(p)
    O.boundp(cbc, n, [0] * 6, nh_u, [1 / dxi, 1 / dyi, 1.0], dzc, dzf, p)
    O.correc(n, nh_u, nh_u, dxi, dyi, 1.0, dzci, dt, rho0, p, u, v, w)
    velocity_ghosts(u, v, w, n, cbc, nh_u)
    tot, mx = O.chkdiv(n, dxi, dyi, 1.0, nh_u, nh_u, dzfi, u, v, w)
    assert mx <= 1e-11 * 1.0 * dxi


@pytest.mark.parametrize("gr", [0.0, 1.0, 2.0])
def test_bench_grid_matches_initgrid(oracle, gr):
    """bench.py's stretched z grid (configuration C3) is initgrid's (src/initgrid.f90)."""
    import bench
    n = 64
    dzci, dzfi = bench.zgrid_stretched(n, gr)
    dzc, dzf, zc, zf = oracle.initgrid(n, gr, 1.0, 1)
    # equal up to the last bits of libm tanh (numpy vs C)
    assert np.allclose(1.0 / dzci, dzc, rtol=1e-12, atol=0) and np.allclose(1.0 / dzfi, dzf, rtol=1e-12, atol=0)


@pytest.mark.parametrize("side", range(6))
def test_oracle_outflow_zero_divergence(oracle, side):
    """outflow (src/bound.f90:649-773) makes the cells next to an outflow face divergence-free."""
    n = [10, 8, 6]
    rng = np.random.default_rng(side)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 1.0)
    u, v, w = random_velocity(rng, n, 1)
    flags = [0] * 6
    flags[side] = 1
    oracle.bounduvw("PPPPDD" * 3, n, [0.0] * 18, 1, 1, [1 / 10, 1 / 8, 1.0], dzc, dzf, u, v, w, isoutflow=flags)
    # divergence of the interior cells; arrays are [k, j, i] with one halo layer
    div = ((u[1:-1, 1:-1, 1:-1] - u[1:-1, 1:-1, :-2]) * 10 + (v[1:-1, 1:-1, 1:-1] - v[1:-1, :-2, 1:-1]) * 8
           + (w[1:-1, 1:-1, 1:-1] - w[:-2, 1:-1, 1:-1]) * dzfi[1:-1, None, None])
    face = [div[:, :, 0], div[:, :, -1], div[:, 0, :], div[:, -1, :], div[0], div[-1]][side]
    assert np.abs(face).max() <= 1e-12 * np.abs(div).max()
