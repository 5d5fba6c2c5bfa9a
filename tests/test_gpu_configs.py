"""Parity at the full sizes of the benchmark workloads, against the FP64 oracle.

  128^3 single-phase projection, FP64 (fillps -> solver -> boundp -> correc ->
        bounduvw as separate drop-in calls, and the fused call)
  256^3 two-phase Dodd-Ferrante projection (the headline step), FP64 and mixed
  512x512x256 tanh-stretched solve (gr = 2), BC NN/PP/ND, k^-5/3 RHS, FP64 and
        mixed to 1e-6 and 1e-10

Tolerances (the path's targets): FP64 relative L2 <= 1e-12 against the oracle
(pressure with the mean removed where the problem is singular), max|div u| <=
1e-11 U/dx with U = 1 after an FP64 projection; mixed: relative residual of
the returned solution <= the requested tolerance (recomputed by the oracle),
and its error against the FP64 oracle bounded per case below.
"""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, rel_l2, singular

pytestmark = pytest.mark.gpu

if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _dl(n):
    return [1.0 / n[0], 1.0 / n[1], 0.0]


def test_c1_projection_128_fp64(lib, oracle):
    """128^3 uniform, periodic x,y, walls in z, u,v,w ~ U[-1,1] with no-slip walls,
    dt = 1e-3, rho0 = 1: one fillps -> solver -> correc projection."""
    import bench
    n, cbc, cbcvel = [128, 128, 128], "PPPPNN", "PPPPDD" * 3
    dzci, dzfi, dz = bench.zgrid(128)
    dxi = dyi = dzi = 128.0
    dt, rho0 = 1e-3, 1.0
    rng = np.random.default_rng(128)
    shp = (130, 130, 130)
    u, v, w = (rng.uniform(-1.0, 1.0, shp) for _ in range(3))
    oracle.bounduvw(cbcvel, n, [0.0] * 18, 1, 1, _dl(n), dz, dz, u, v, w)
    S = oracle.SolverSetup(n, [dxi, dyi, dzi], 1, dzci, dzfi, cbc, [0.0] * 6, "ccc")
    uo, vo, wo = u.copy(), v.copy(), w.copy()
    po = np.zeros(shp)
    oracle.fillps(n, 1, 1, dxi, dyi, dzi, dzfi, 1 / dt, rho0, uo, vo, wo, po)
    S.solve(po)
    oracle.boundp(cbc, n, [0.0] * 6, 1, _dl(n), dz, dz, po)
    oracle.correc(n, 1, 1, dxi, dyi, dzi, dzci, dt, rho0, po, uo, vo, wo)
    oracle.bounduvw(cbcvel, n, [0.0] * 18, 1, 1, _dl(n), dz, dz, uo, vo, wo)
    _, mx_o = oracle.chkdiv(n, dxi, dyi, dzi, 1, 1, dzfi, uo, vo, wo)
    # drop-in calls
    P = lib.initsolver(n, [dxi, dyi, dzi], 1, dzci, dzfi, cbc, [0.0] * 6, "ccc")
    ug, vg, wg = u.copy(), v.copy(), w.copy()
    pg = np.zeros(shp)
    lib.fillps(n, 1, 1, dxi, dyi, dzi, dzfi, 1 / dt, rho0, ug, vg, wg, pg)
    P.solver(pg)
    lib.boundp(cbc, n, [0.0] * 6, 1, _dl(n), dz, dz, pg)
    lib.correc(n, 1, 1, dxi, dyi, dzi, dzci, dt, rho0, pg, ug, vg, wg)
    lib.bounduvw(cbcvel, n, [0.0] * 18, 1, 1, _dl(n), dz, dz, ug, vg, wg)
    e_p = rel_l2(pg[1:-1, 1:-1, 1:-1], po[1:-1, 1:-1, 1:-1], remove_mean=True)
    e_u = max(rel_l2(a, b) for a, b in ((ug, uo), (vg, vo), (wg, wo)))
    _, mx = lib.chkdiv(n, dxi, dyi, dzi, 1, 1, dzfi, ug, vg, wg)
    print(f"C1 drop-in: rel L2 p {e_p:.2e}, u {e_u:.2e}, max|div| {mx:.2e} (oracle {mx_o:.2e})")
    assert e_p <= 1e-12 and e_u <= 1e-12
    assert mx <= 1e-11 * dxi
    # the fused call: p holds pold + phi on exit (pold = 0 here)
    uf, vf, wf = u.copy(), v.copy(), w.copy()
    pf = np.zeros(shp)
    P.projection(1, dxi, dyi, dzci, dzfi, [0.0] * 6, dt, rho0, uf, vf, wf, pf, precision=0,
                 cbcvel=cbcvel, bcvel=[0.0] * 18)
    assert rel_l2(pf[1:-1, 1:-1, 1:-1], po[1:-1, 1:-1, 1:-1], remove_mean=True) <= 1e-12
    assert max(rel_l2(a, b) for a, b in ((uf, uo), (vf, vo), (wf, wo))) <= 1e-12
    _, mxf = lib.chkdiv(n, dxi, dyi, dzi, 1, 1, dzfi, uf, vf, wf)
    assert mxf <= 1e-11 * dxi


@pytest.fixture(scope="module")
def c2_case(oracle):
    """The headline step's inputs (256^3, 64 VoF spheres, density ratio 1000, Fourier-mode
    pressures) and the oracle's result of one step on them."""
    import bench
    fields = {k: t.numpy() for k, t in bench.make_fields(256, 2024, "cpu").items()}
    O, S, dzci, dzfi, dz = bench.cpu_setup(256)
    fo = {k: a.copy() for k, a in fields.items()}
    bench.cpu_step(O, S, 256, fo, dzci, dzfi, dz)
    _, mx_o = O.chkdiv([256] * 3, 256.0, 256.0, 256.0, 1, 1, dzfi, fo["u"], fo["v"], fo["w"])
    return fields, fo, (dzci, dzfi, dz), mx_o


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed-1e-10"])
def test_c2_two_phase_projection_256(lib, c2_case, precision):
    import bench
    fields, fo, (dzci, dzfi, dz), mx_o = c2_case
    n = 256
    P = lib.initsolver([n] * 3, [float(n)] * 3, 1, dzci, dzfi, bench.CBC, [0.0] * 6, "ccc")
    f = {k: a.copy() for k, a in fields.items()}
    P.projection_df(1, float(n), float(n), dzci, dzfi, [0.0] * 6, bench.DT, bench.DT, 1.0, f["rho"], f["pold"],
                    f["u"], f["v"], f["w"], f["p"], precision=precision, tol=1e-10, max_iter=12,
                    cbcvel=bench.CBCVEL, bcvel=bench.BCVEL)
    relres, iters = P.last_solve()
    p0 = fields["p"]
    e_phi = rel_l2((f["p"] - p0)[1:-1, 1:-1, 1:-1], (fo["p"] - p0)[1:-1, 1:-1, 1:-1], remove_mean=True)
    e_u = max(rel_l2(f[k], fo[k]) for k in ("u", "v", "w"))
    _, mx = lib.chkdiv([n] * 3, float(n), float(n), float(n), 1, 1, dzfi, f["u"], f["v"], f["w"])
    print(f"C2 precision {precision}: rel L2 phi {e_phi:.2e}, u {e_u:.2e}, max|div| {mx:.2e} "
          f"(oracle {mx_o:.2e}, bound {1e-11 * n:.2e}), relres {relres:.2e} after {iters}")
    assert np.array_equal(f["pold"][1:-1, 1:-1, 1:-1], p0[1:-1, 1:-1, 1:-1])  # the app's pold = p
    if precision == 0:
        assert e_phi <= 1e-12 and e_u <= 1e-12
        assert mx <= 1e-11 * n
    else:
        # FP32 solves refined to 1e-10 in FP64; the Dodd-Ferrante increment of u* is
        # evaluated in FP32 (relative error ~1e-7 of an increment that is a small part of
        # u*), which bounds the error against the oracle (measured: phi 1.2e-8, u 6e-10)
        assert relres <= 1e-10
        assert e_u <= 1e-8 and e_phi <= 5e-8
        # max|div u| = dt/rho0 max|f - A phi|: a 1e-10 relative residual leaves it above
        # 1e-11 U/dx on this grid, below 1e-8 U/dx
        assert mx <= 1e-8 * n


def c3_rhs(shape, seed):
    """Seeded Gaussian random field with a k^-5/3 power spectrum, zero mean, unit
    variance (nz, ny, nx), in a halo-1 array."""
    import torch
    nz, ny, nx = shape
    g = torch.Generator(device="cuda").manual_seed(seed)
    white = torch.randn((nz, ny, nx), generator=g, dtype=torch.float64, device="cuda")
    spec = torch.fft.rfftn(white)
    kz = torch.fft.fftfreq(nz, device="cuda", dtype=torch.float64)[:, None, None] * nz
    ky = torch.fft.fftfreq(ny, device="cuda", dtype=torch.float64)[None, :, None] * ny
    kx = torch.fft.rfftfreq(nx, device="cuda", dtype=torch.float64)[None, None, :] * nx
    k = torch.sqrt(kx * kx + ky * ky + kz * kz)
    k[0, 0, 0] = 1.0
    spec *= k ** (-5.0 / 6.0)
    spec[0, 0, 0] = 0.0
    field = torch.fft.irfftn(spec, s=(nz, ny, nx))
    field -= field.mean()
    field /= field.std()
    out = np.zeros((nz + 2, ny + 2, nx + 2))
    out[1:-1, 1:-1, 1:-1] = field.cpu().numpy()
    return out


def test_c3_stretched_solve_512x512x256(lib, oracle):
    import bench
    n, cbc = [512, 512, 256], "NNPPND"
    dzci, dzfi = bench.zgrid_stretched(n[2], 2.0)
    dli = [512.0, 512.0, 256.0]
    f = c3_rhs((n[2], n[1], n[0]), 7)
    S = oracle.SolverSetup(n, dli, 1, dzci, dzfi, cbc, [0.0] * 6, "ccc")
    ref = f.copy()
    S.solve(ref)
    P = lib.initsolver(n, dli, 1, dzci, dzfi, cbc, [0.0] * 6, "ccc")
    assert np.array_equal(P.a, S.a) and np.array_equal(P.b, S.b) and np.array_equal(P.lambdaxy, S.lambdaxy)
    got = f.copy()
    P.solver(got)
    e = rel_l2(got[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1], remove_mean=singular(cbc))
    print(f"C3 FP64: rel L2 {e:.2e}")
    assert e <= 1e-12
    fnorm = np.linalg.norm(f[1:-1, 1:-1, 1:-1])
    for tol in (1e-6, 1e-10):
        m = f.copy()
        relres, iters = P.solve_mixed(m, tol=tol, max_iter=10)
        r = oracle.residual(n, cbc, dli[0], dli[1], 1, dzci, dzfi, f, m)
        true = np.linalg.norm(r) / fnorm
        err = rel_l2(m[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1])
        print(f"C3 mixed {tol:g}: relres {relres:.2e} (oracle {true:.2e}) after {iters}, rel L2 vs oracle {err:.2e}")
        assert relres <= tol and true <= 1.01 * tol
        # the error follows the residual times the operator's condition (stretched z)
        assert err <= 1e4 * tol
