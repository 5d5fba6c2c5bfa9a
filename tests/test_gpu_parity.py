"""GPU parity tests: the CUDA path through the C ABI against the FP64 oracle.

Tolerances (written here, from the target of the path):
  FP64 solver vs oracle           relative L2 <= 1e-12 (mean-removed where the
                                  problem is singular: x,y in {P,N}, z in N/N or P/P)
  stencils (fillps, correc, ...)  max relative difference <= 1e-14
  projection                      max |div u| <= 1e-11 * U / dx   (U = 1)
  mixed precision                 relative residual <= requested tol; the error
                                  against the FP64 oracle is asserted per case
"""
import numpy as np
import pytest

from conftest import (compatible_rhs, golden_cases, random_velocity, rel_l2, singular,
                      velocity_ghosts, zgrid)

pytestmark = pytest.mark.gpu


def plan_for(lib, n, cbc, gr=0.0, dli=None, bc=None):
    dzci, dzfi, dzc, dzf = zgrid(n[2], gr)
    dli = dli or [n[0] * 1.0, n[1] * 1.0, n[2] * 1.0]
    P = lib.initsolver(n, dli, 1, dzci, dzfi, cbc, bc or [0.0] * 6, "ccc")
    return P, dzci, dzfi, dzc, dzf, dli


@pytest.mark.parametrize("fn", golden_cases(), ids=lambda s: s.split("kat_")[-1][:-4])
def test_gpu_known_answers_fp64(lib, fn):
    d = np.load(fn)
    n = [int(x) for x in d["n"]]
    cbc = str(d["cbc"])
    if cbc[0:2] in ("ND", "DN") and n[0] % 2 or cbc[2:4] in ("ND", "DN") and n[1] % 2:
        pytest.skip("DCT-IV needs even n on the GPU")
    P = lib.initsolver(n, d["dli"], 1, d["dzci"], d["dzfi"], cbc, [0] * 6, "ccc")
    p = np.zeros((n[2] + 2, n[1] + 2, n[0] + 2))
    p[1:-1, 1:-1, 1:-1] = d["f"]
    P.solver(p)
    assert rel_l2(p[1:-1, 1:-1, 1:-1], d["p"], remove_mean=singular(cbc)) <= 1e-12


CASES = [
    ((16, 16, 16), "PPPPNN", 0.0),
    ((32, 32, 24), "PPPPNN", 2.0),
    ((24, 20, 12), "NNPPND", 2.0),
    ((20, 16, 10), "DDNNDD", 1.0),
    ((16, 24, 9), "NDDNNN", 0.0),
    ((48, 16, 8), "PPDDDN", 0.5),
    ((16, 12, 16), "NNNNPP", 0.0),
    ((18, 14, 7), "DNNDNN", 1.0),
    ((128, 128, 12), "PPPPNN", 0.0),   # fused plane path in FP32, cluster path in FP64
    ((256, 64, 6), "NNPPNN", 1.5),     # planes larger than one CTA: cluster path
    ((176, 144, 5), "PPNNDD", 0.0),    # radices 11, 9
    ((32, 24, 40), "PPPPNN", 1.5),     # z sweeps over full 16-level chunks and a partial last one
    ((24, 16, 33), "NNNNDN", 0.0),
    ((32, 24, 16), "PPPPDD", 1.5),     # exactly one chunk
]


@pytest.mark.parametrize("n,cbc,gr", CASES, ids=[f"{c}-{n[0]}x{n[1]}x{n[2]}" for n, c, _ in CASES])
def test_gpu_solver_matches_oracle_fp64(lib, oracle, n, cbc, gr):
    rng = np.random.default_rng(sum(n))
    P, dzci, dzfi, dzc, dzf, dli = plan_for(lib, n, cbc, gr)
    S = oracle.SolverSetup(n, dli, 1, dzci, dzfi, cbc, [0] * 6, "ccc")
    assert np.array_equal(P.lambdaxy, S.lambdaxy) and np.array_equal(P.a, S.a)
    assert np.array_equal(P.b, S.b) and P.normfft == S.normfft
    p = compatible_rhs(rng, n, cbc, dzf)
    ref = p.copy()
    S.solve(ref)
    got = p.copy()
    P.solver(got)
    e = rel_l2(got[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1], remove_mean=singular(cbc))
    assert e <= 1e-12, e
    # halo untouched by the solver (like solver_cpu, which writes p(1:n) only)
    assert np.array_equal(got[0], p[0]) and np.array_equal(got[:, :, -1], p[:, :, -1])


def test_gpu_solver_device_pointers(lib, oracle):
    import torch
    n, cbc = (64, 48, 32), "PPNNNN"
    rng = np.random.default_rng(5)
    P, dzci, dzfi, dzc, dzf, dli = plan_for(lib, n, cbc, 1.5)
    S = oracle.SolverSetup(n, dli, 1, dzci, dzfi, cbc, [0] * 6, "ccc")
    p = compatible_rhs(rng, n, cbc, dzf)
    ref = p.copy()
    S.solve(ref)
    pd = torch.from_numpy(p).cuda()
    P.solver(pd)
    got = pd.cpu().numpy()
    assert rel_l2(got[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1], remove_mean=True) <= 1e-12


def test_gpu_stencils_match_oracle(lib, oracle):
    n = [20, 14, 12]
    rng = np.random.default_rng(11)
    for nh_u in (1, 3):
        dzci, dzfi, dzc, dzf = zgrid(n[2], 1.2, nh_d=nh_u)
        u, v, w = random_velocity(rng, n, nh_u)
        p_ref = np.zeros((n[2] + 2, n[1] + 2, n[0] + 2))
        p_gpu = rng.standard_normal(p_ref.shape)  # halo values must be left alone
        p_ref[...] = p_gpu
        oracle.fillps(n, nh_u, nh_u, 20.0, 14.0, 12.0, dzfi, 1e3, 1.7, u, v, w, p_ref)
        lib.fillps(n, nh_u, nh_u, 20.0, 14.0, 12.0, dzfi, 1e3, 1.7, u, v, w, p_gpu)
        assert np.abs(p_gpu - p_ref).max() <= 1e-14 * np.abs(p_ref).max()
        # correc
        p = rng.standard_normal(p_ref.shape)
        uo, vo, wo = u.copy(), v.copy(), w.copy()
        oracle.correc(n, nh_u, nh_u, 20.0, 14.0, 12.0, dzci, 1e-3, 1.3, p, uo, vo, wo)
        lib.correc(n, nh_u, nh_u, 20.0, 14.0, 12.0, dzci, 1e-3, 1.3, p, u, v, w)
        for a, b in ((u, uo), (v, vo), (w, wo)):
            assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max()
        tot_o, mx_o = oracle.chkdiv(n, 20.0, 14.0, 12.0, nh_u, nh_u, dzfi, u, v, w)
        tot_g, mx_g = lib.chkdiv(n, 20.0, 14.0, 12.0, nh_u, nh_u, dzfi, u, v, w)
        assert mx_g == pytest.approx(mx_o, rel=1e-14)
        assert tot_g == pytest.approx(tot_o, rel=1e-9, abs=1e-9)
    # boundp for every BC type, non-zero BC values
    dzci, dzfi, dzc, dzf = zgrid(n[2], 1.2)
    for cbc in ("PPPPPP", "NNDDND", "DNNDPP", "PPNDDN"):
        bc = [0.3, -0.2, 0.5, 0.1, -0.4, 0.7]
        p = rng.standard_normal((n[2] + 2, n[1] + 2, n[0] + 2))
        po = p.copy()
        oracle.boundp(cbc, n, bc, 1, [1 / 20, 1 / 14, 1 / 12], dzc, dzf, po)
        lib.boundp(cbc, n, bc, 1, [1 / 20, 1 / 14, 1 / 12], dzc, dzf, p)
        assert np.array_equal(p, po), cbc
    # updt_rhs_b with inhomogeneous BCs from initsolver
    cbc = "NNDDND"
    S = oracle.SolverSetup(n, [20.0, 14.0, 12.0], 1, dzci, dzfi, cbc, [0.3, -0.2, 0.5, 0.1, -0.4, 0.7])
    p = rng.standard_normal((n[2] + 2, n[1] + 2, n[0] + 2))
    po = p.copy()
    oracle.updt_rhs_b(n, "ccc", cbc, S.rhsbx, S.rhsby, S.rhsbz, po)
    lib.updt_rhs_b(n, "ccc", cbc, S.rhsbx, S.rhsby, S.rhsbz, p)
    assert np.abs(p - po).max() <= 1e-14 * np.abs(po).max()


def test_gpu_pres_tw_src_matches_oracle(lib, oracle):
    n = [16, 12, 10]
    rng = np.random.default_rng(21)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 0.0)
    u, v, w = random_velocity(rng, n, 1)
    shp = (n[2] + 2, n[1] + 2, n[0] + 2)
    p, pold = rng.standard_normal(shp), rng.standard_normal(shp)
    rho = rng.uniform(1.0, 1000.0, shp)
    uo, vo, wo = u.copy(), v.copy(), w.copy()
    oracle.pres_tw_src(n, 16.0, 12.0, 10.0, 1, 1, dzci, 1.0, 1e-3, 2e-3, p, pold, rho, uo, vo, wo)
    lib.pres_tw_src(n, 16.0, 12.0, 10.0, 1, 1, dzci, 1.0, 1e-3, 2e-3, p, pold, rho, u, v, w)
    for a, b in ((u, uo), (v, vo), (w, wo)):
        assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max()


def _projection_inputs(rng, n, cbc, nh_u=1):
    return velocity_ghosts(*random_velocity(rng, n, nh_u), n, cbc, nh_u)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_gpu_fused_projection(lib, oracle, precision):
    """One fused call == fillps, updt_rhs_b, solver, boundp, correc, p=pold+p, boundp of the oracle."""
    n, cbc = [32, 32, 24], "PPPPNN"
    rng = np.random.default_rng(31)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 0.0)
    dxi, dyi = 32.0, 32.0
    P = lib.initsolver(n, [dxi, dyi, 24.0], 1, dzci, dzfi, cbc, [0] * 6, "ccc")
    S = oracle.SolverSetup(n, [dxi, dyi, 24.0], 1, dzci, dzfi, cbc, [0] * 6, "ccc")
    u, v, w = _projection_inputs(rng, n, cbc)
    pold = rng.standard_normal((n[2] + 2, n[1] + 2, n[0] + 2))
    dt, rho0 = 1e-3, 1.0
    # oracle sequence
    uo, vo, wo = u.copy(), v.copy(), w.copy()
    phi = np.zeros_like(pold)
    oracle.fillps(n, 1, 1, dxi, dyi, 24.0, dzfi, 1 / dt, rho0, uo, vo, wo, phi)
    oracle.updt_rhs_b(n, "ccc", cbc, S.rhsbx, S.rhsby, S.rhsbz, phi)
    S.solve(phi)
    oracle.boundp(cbc, n, [0] * 6, 1, [1 / dxi, 1 / dyi, 1.0], dzc, dzf, phi)
    oracle.correc(n, 1, 1, dxi, dyi, 24.0, dzci, dt, rho0, phi, uo, vo, wo)
    po = pold.copy()
    po[1:-1, 1:-1, 1:-1] += phi[1:-1, 1:-1, 1:-1]
    oracle.boundp(cbc, n, [0] * 6, 1, [1 / dxi, 1 / dyi, 1.0], dzc, dzf, po)
    # GPU
    p = pold.copy()
    P.projection(1, dxi, dyi, dzci, dzfi, [0] * 6, dt, rho0, u, v, w, p, precision=precision, tol=1e-12,
                 max_iter=10)
    tol = 1e-12 if precision == 0 else 1e-9
    for a, b in ((u, uo), (v, vo), (w, wo)):
        assert rel_l2(a, b) <= tol
    assert rel_l2(p[1:-1, 1:-1, 1:-1], po[1:-1, 1:-1, 1:-1], remove_mean=True) <= tol * 100
    velocity_ghosts(u, v, w, n, cbc)
    tot, mx = lib.chkdiv(n, dxi, dyi, 24.0, 1, 1, dzfi, u, v, w)
    assert mx <= 1e-11 * dxi


@pytest.mark.parametrize("n,cbc,gr", [((64, 64, 32), "PPPPNN", 0.0), ((64, 48, 32), "NNPPND", 2.0),
                                      ((48, 80, 16), "DDNNDD", 1.0), ((32, 32, 32), "PPPPPP", 0.0),
                                      ((40, 24, 37), "PPPPNN", 1.0)])  # partial last z chunk
@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_gpu_mixed_precision_refinement(lib, oracle, n, cbc, gr, tol):
    rng = np.random.default_rng(41)
    P, dzci, dzfi, dzc, dzf, dli = plan_for(lib, n, cbc, gr)
    S = oracle.SolverSetup(n, dli, 1, dzci, dzfi, cbc, [0] * 6, "ccc")
    p = compatible_rhs(rng, n, cbc, dzf)
    f = p.copy()
    ref = p.copy()
    S.solve(ref)
    relres, iters = P.solve_mixed(p, tol=tol, max_iter=10)
    assert relres <= tol
    r = oracle.residual(n, cbc, dli[0], dli[1], 1, dzci, dzfi, f, p)
    assert np.linalg.norm(r) / np.linalg.norm(f[1:-1, 1:-1, 1:-1]) <= tol * 1.01
    err = rel_l2(p[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1], remove_mean=singular(cbc))
    assert err <= max(1e3 * tol, 1e-12), err


# z-planes larger than one CTA's shared memory: the FP32 x and y transforms of
# a plane run in a thread-block cluster that exchanges the plane through
# distributed shared memory (xy path 2), 4 to 8 CTAs per cluster here; the FP64
# solver's double-float transforms take separate x and y passes (path 0), which
# measured faster than their cluster form.
LARGE_PLANES = [((256, 256, 4), "PPPPNN", 0.0), ((320, 192, 6), "NNPPDD", 1.0),
                ((256, 128, 5), "DDNNPP", 0.0), ((192, 256, 3), "NDPPNN", 0.5)]


@pytest.mark.parametrize("n,cbc,gr", LARGE_PLANES, ids=[f"{c}-{n[0]}x{n[1]}x{n[2]}" for n, c, _ in LARGE_PLANES])
def test_gpu_cluster_plane_path(lib, oracle, n, cbc, gr, monkeypatch):
    rng = np.random.default_rng(7 + sum(n))
    monkeypatch.setenv("FLUTAS_GB300_XY_PATH", "2")  # the cluster form, not the timed choice
    P, dzci, dzfi, dzc, dzf, dli = plan_for(lib, n, cbc, gr)
    info = P.info()
    assert info["xy_path_fp64"] == 0 and info["xy_path_fp32"] == 2, info
    S = oracle.SolverSetup(n, dli, 1, dzci, dzfi, cbc, [0] * 6, "ccc")
    p = compatible_rhs(rng, n, cbc, dzf)
    f = p.copy()
    ref = p.copy()
    S.solve(ref)
    got = p.copy()
    P.solver(got)
    assert rel_l2(got[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1], remove_mean=singular(cbc)) <= 1e-12
    mixed = p.copy()
    relres, _ = P.solve_mixed(mixed, tol=1e-10, max_iter=10)
    assert relres <= 1e-10
    r = oracle.residual(n, cbc, dli[0], dli[1], 1, dzci, dzfi, f, mixed)
    assert np.linalg.norm(r) / np.linalg.norm(f[1:-1, 1:-1, 1:-1]) <= 1e-10 * 1.01
    # the same solve with separate x and y passes (path 0) agrees to rounding
    monkeypatch.setenv("FLUTAS_GB300_XY_PATH", "0")
    Q = plan_for(lib, n, cbc, gr)[0]
    assert Q.info()["xy_path_fp64"] == 0 and Q.info()["xy_path_fp32"] == 0
    sep = p.copy()
    Q.solver(sep)
    assert rel_l2(got[1:-1, 1:-1, 1:-1], sep[1:-1, 1:-1, 1:-1], remove_mean=singular(cbc)) <= 1e-13
    sep_mixed = p.copy()
    relres_q, _ = Q.solve_mixed(sep_mixed, tol=1e-10, max_iter=10)
    rq = oracle.residual(n, cbc, dli[0], dli[1], 1, dzci, dzfi, f, sep_mixed)
    assert relres_q <= 1e-10 and np.linalg.norm(rq) / np.linalg.norm(f[1:-1, 1:-1, 1:-1]) <= 1e-10 * 1.01


VEL_BCS = ["PPPPDD" * 3, "DDPPDD" * 3, "NNDDND" * 3, "PPNNDD" * 3]


@pytest.mark.parametrize("cbcvel", VEL_BCS)
@pytest.mark.parametrize("nh_u", [1, 3])
@pytest.mark.parametrize("n", [[12, 10, 8], [5, 4, 6]], ids=["one-launch", "pass-by-pass"])
def test_gpu_bounduvw_matches_oracle(lib, oracle, cbcvel, nh_u, n):
    """Bit-identical ghosts.  Grids with fewer than 2*nh_u + 1 cells along an axis
    take the pass-by-pass kernel, the others the single composed launch."""
    rng = np.random.default_rng(nh_u)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 1.3, nh_d=nh_u)
    bcvel = list(rng.uniform(-1, 1, 18))
    u, v, w = random_velocity(rng, n, nh_u)
    uo, vo, wo = u.copy(), v.copy(), w.copy()
    dl = [1 / n[0], 1 / n[1], 1 / n[2]]
    oracle.bounduvw(cbcvel, n, bcvel, nh_u, nh_u, dl, dzc, dzf, uo, vo, wo)
    lib.bounduvw(cbcvel, n, bcvel, nh_u, nh_u, dl, dzc, dzf, u, v, w)
    for a, b in ((u, uo), (v, vo), (w, wo)):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_gpu_two_phase_projection_df(lib, oracle, precision):
    """pres_tw_src + bounduvw + projection of a two-phase field == the oracle sequence."""
    two_phase_case(lib, oracle, precision)


@pytest.mark.parametrize("contraction", ["1e-30", "1.0"], ids=["fused-check-missed", "late-prediction"])
def test_gpu_mixed_projection_final_check(lib, oracle, contraction, monkeypatch):
    """The mixed projection applies correc + p update inside its last check when
    the predicted contraction says the solve has converged.  A prediction of
    1e-30 makes the first check the fused one although it cannot pass: the
    solve goes on and the projection adds the correction of the rest.  A
    prediction of 1 delays the fused check to a later iteration.  Both must
    give the oracle's fields."""
    monkeypatch.setenv("FLUTAS_GB300_CONTRACTION", contraction)
    two_phase_case(lib, oracle, 1)


def test_gpu_projection_df_pinned_host(lib):
    """Page-locked host arrays take the overlapped path (pold copied back while the
    solve runs): the fields equal those of the same call on pageable arrays."""
    torch = pytest.importorskip("torch")
    n, cbc, cbcvel = [32, 24, 16], "PPPPNN", "PPPPDD" * 3
    rng = np.random.default_rng(77)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 0.0)
    dxi, dyi, dt = 32.0, 24.0, 1e-3
    shp = (n[2] + 2, n[1] + 2, n[0] + 2)
    u, v, w = random_velocity(rng, n, 1)
    p, pold = rng.standard_normal(shp), rng.standard_normal(shp)
    lib.boundp(cbc, n, [0] * 6, 1, [1 / dxi, 1 / dyi, 1.0], dzc, dzf, p)
    rho = np.where(rng.uniform(0, 1, shp) > 0.7, 1000.0, 1.0)
    pageable = [a.copy() for a in (rho, pold, u, v, w, p)]
    pinned = []
    for a in (rho, pold, u, v, w, p):
        t = torch.empty(a.shape, dtype=torch.float64).pin_memory()
        t.numpy()[...] = a
        pinned.append(t.numpy())
    outs = []
    for arrs in (pageable, pinned):
        P = lib.initsolver(n, [dxi, dyi, 16.0], 1, dzci, dzfi, cbc, [0] * 6, "ccc")
        P.projection_df(1, dxi, dyi, dzci, dzfi, [0] * 6, dt, dt, 1.0, *arrs, precision=1, tol=1e-11,
                        max_iter=10, cbcvel=cbcvel, bcvel=[0] * 18)
        outs.append([a.copy() for a in arrs[1:]])
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    assert np.array_equal(outs[1][0], p)  # pold on return = p on entry


def two_phase_case(lib, oracle, precision):
    n, cbc, cbcvel = [32, 24, 16], "PPPPNN", "PPPPDD" * 3
    rng = np.random.default_rng(51)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 0.0)
    dxi, dyi, dt = 32.0, 24.0, 1e-3
    P = lib.initsolver(n, [dxi, dyi, 16.0], 1, dzci, dzfi, cbc, [0] * 6, "ccc")
    S = oracle.SolverSetup(n, [dxi, dyi, 16.0], 1, dzci, dzfi, cbc, [0] * 6, "ccc")
    shp = (n[2] + 2, n[1] + 2, n[0] + 2)
    u, v, w = random_velocity(rng, n, 1)
    p, pold = rng.standard_normal(shp), rng.standard_normal(shp)
    oracle.boundp(cbc, n, [0] * 6, 1, [1 / dxi, 1 / dyi, 1.0], dzc, dzf, p)
    oracle.boundp(cbc, n, [0] * 6, 1, [1 / dxi, 1 / dyi, 1.0], dzc, dzf, pold)
    psi = (rng.uniform(0, 1, shp) > 0.7).astype(np.float64)
    rho = oracle.update_property(n, 1000.0, 1.0, psi)
    oracle.boundp(cbc, n, [0] * 6, 1, [1 / dxi, 1 / dyi, 1.0], dzc, dzf, rho)  # as the app does after it
    rho_gpu = np.zeros_like(psi)
    lib.update_property(n, [1000.0, 1.0], psi, rho_gpu)
    lib.boundp(cbc, n, [0] * 6, 1, [1 / dxi, 1 / dyi, 1.0], dzc, dzf, rho_gpu)
    assert np.array_equal(rho_gpu, rho)
    dl = [1 / dxi, 1 / dyi, 0.0]
    uo, vo, wo, po = u.copy(), v.copy(), w.copy(), p.copy()
    oracle.pres_tw_src(n, dxi, dyi, 16.0, 1, 1, dzci, 1.0, dt, dt, po, pold, rho, uo, vo, wo)
    oracle.bounduvw(cbcvel, n, [0] * 18, 1, 1, dl, dzc, dzf, uo, vo, wo)
    phi = np.zeros(shp)
    oracle.fillps(n, 1, 1, dxi, dyi, 16.0, dzfi, 1 / dt, 1.0, uo, vo, wo, phi)
    S.solve(phi)
    oracle.boundp(cbc, n, [0] * 6, 1, dl, dzc, dzf, phi)
    oracle.correc(n, 1, 1, dxi, dyi, 16.0, dzci, dt, 1.0, phi, uo, vo, wo)
    oracle.bounduvw(cbcvel, n, [0] * 18, 1, 1, dl, dzc, dzf, uo, vo, wo)
    po[1:-1, 1:-1, 1:-1] += phi[1:-1, 1:-1, 1:-1]
    oracle.boundp(cbc, n, [0] * 6, 1, dl, dzc, dzf, po)
    p_in, pold_in = p.copy(), pold.copy()
    P.projection_df(1, dxi, dyi, dzci, dzfi, [0] * 6, dt, dt, 1.0, rho, pold, u, v, w, p,
                    precision=precision, tol=1e-11, max_iter=10, cbcvel=cbcvel, bcvel=[0] * 18)
    tol = 1e-12 if precision == 0 else 1e-8
    for a, b in ((u, uo), (v, vo), (w, wo)):
        assert rel_l2(a, b) <= tol
    assert rel_l2(p - pold_in, po - pold_in, remove_mean=True) <= tol * 100
    # the app's pold = p (interior copy, then boundp): p satisfied boundp on entry
    assert np.array_equal(pold, p_in)
    tot, mx = lib.chkdiv(n, dxi, dyi, 16.0, 1, 1, dzfi, u, v, w)
    assert mx <= 1e-11 * dxi


@pytest.mark.parametrize("n,cbc", [((64, 48, 32), "PPPPNN"), ((256, 256, 6), "NNPPDD")])
def test_gpu_mixed_reported_residual(lib, oracle, n, cbc):
    """The residual a mixed solve reports is the residual of the solution it returns.

    An unattainable tolerance walks every branch of the refinement loop: full
    residual passes, a norm-only check predicted to be the last, the transform
    made after that prediction failed, and the final norm-only check at the
    iteration limit."""
    rng = np.random.default_rng(17)
    P, dzci, dzfi, dzc, dzf, dli = plan_for(lib, n, cbc, 1.0)
    f = compatible_rhs(rng, n, cbc, dzf)
    for tol, max_iter in ((1e-6, 8), (1e-10, 8), (1e-15, 4)):
        p = f.copy()
        relres, iters = P.solve_mixed(p, tol=tol, max_iter=max_iter, allow_unconverged=True)
        r = oracle.residual(n, cbc, dli[0], dli[1], 1, dzci, dzfi, f, p)
        true = np.linalg.norm(r) / np.linalg.norm(f[1:-1, 1:-1, 1:-1])
        # FP32 sums of FP32-truncated residuals: ~1e-5 relative; plus the FP64 rounding
        # noise of two different evaluation orders of f - A x near the floor
        assert abs(relres - true) <= 1e-3 * true + 1e-12, (tol, relres, true)
        assert (relres <= tol) == (tol > 1e-14) and iters <= max_iter
        assert relres <= max(tol, 1e-11)


@pytest.mark.parametrize("n,cbc", [((256, 256, 5), "PPPPNN"), ((256, 256, 5), "NNPPDD"), ((256, 256, 5), "PPNNNN"),
                                   ((256, 256, 5), "NNNNPP"), ((512, 512, 3), "NNPPND"), ((512, 512, 3), "PPPPNN")])
def test_gpu_fixed_size_cluster_kernels(lib, oracle, n, cbc, monkeypatch):
    """256^2 and 512^2 planes run the compile-time-sized cluster kernels in the
    mixed path; the result matches the oracle and the run-time-sized kernels."""
    rng = np.random.default_rng(3)
    P, dzci, dzfi, dzc, dzf, dli = plan_for(lib, n, cbc, 0.5)
    f = compatible_rhs(rng, n, cbc, dzf)
    ref = f.copy()
    oracle.SolverSetup(n, dli, 1, dzci, dzfi, cbc, [0] * 6, "ccc").solve(ref)
    out = {}
    for fixed in ("1", "0"):
        monkeypatch.setenv("FLUTAS_GB300_FIXED", fixed)
        p = f.copy()
        relres, _ = P.solve_mixed(p, tol=1e-10, max_iter=8)
        r = oracle.residual(n, cbc, dli[0], dli[1], 1, dzci, dzfi, f, p)
        assert np.linalg.norm(r) / np.linalg.norm(f[1:-1, 1:-1, 1:-1]) <= 1.01e-10
        assert rel_l2(p[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1], remove_mean=singular(cbc)) <= 1e-7
        out[fixed] = p
    assert rel_l2(out["1"][1:-1, 1:-1, 1:-1], out["0"][1:-1, 1:-1, 1:-1], remove_mean=singular(cbc)) <= 1e-7


# The grid shapes and pressure BCs of the reference's example cases
# (examples/*/dns.in: itot jtot ktot and cbcpre); droplet_rb's 1024x1024x512 is
# cut to 4 levels (same 1024^2 planes) so the oracle stays fast.
EXAMPLES = [("abc_triperiodic", (32, 32, 32), "PPPPPP"), ("coarse_two_layer_rb", (128, 64, 128), "PPNNPP"),
            ("dhc", (2, 128, 128), "PPNNNN"), ("droplet_rb", (1024, 1024, 4), "PPPPNN"),
            ("laminar_ldc_2D", (2, 64, 64), "PPNNNN"), ("laminar_channel", (64, 32, 32), "PPPPNN"),
            ("coarse_turb_channel", (256, 128, 72), "PPPPNN"), ("laminar_ldc", (64, 64, 64), "NNNNNN"),
            ("rising_bubble_3d", (32, 32, 64), "NNNNNN")]


@pytest.mark.parametrize("name,n,cbc", EXAMPLES, ids=[e[0] for e in EXAMPLES])
def test_gpu_reference_example_grids(lib, oracle, name, n, cbc):
    rng = np.random.default_rng(len(name))
    P, dzci, dzfi, dzc, dzf, dli = plan_for(lib, n, cbc, 0.0)
    S = oracle.SolverSetup(n, dli, 1, dzci, dzfi, cbc, [0] * 6, "ccc")
    f = compatible_rhs(rng, n, cbc, dzf)
    ref = f.copy()
    S.solve(ref)
    got = f.copy()
    P.solver(got)
    assert rel_l2(got[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1], remove_mean=singular(cbc)) <= 1e-12
    mixed = f.copy()
    relres, _ = P.solve_mixed(mixed, tol=1e-10, max_iter=10)
    r = oracle.residual(n, cbc, dli[0], dli[1], 1, dzci, dzfi, f, mixed)
    assert relres <= 1e-10 and np.linalg.norm(r) / np.linalg.norm(f[1:-1, 1:-1, 1:-1]) <= 1.01e-10


@pytest.mark.parametrize("flags", [[1, 0, 0, 0, 0, 0], [0, 1, 0, 0, 0, 0], [0, 0, 1, 0, 0, 0], [0, 0, 0, 1, 0, 0],
                                   [0, 0, 0, 0, 1, 0], [0, 0, 0, 0, 0, 1], [1] * 6],
                         ids=["x-", "x+", "y-", "y+", "z-", "z+", "all"])
@pytest.mark.parametrize("nh_u", [1, 2])
def test_gpu_bounduvw_outflow(lib, oracle, flags, nh_u):
    """bounduvw with outflow faces (src/bound.f90:649-773): bit-identical to the oracle."""
    n = [14, 10, 8]
    rng = np.random.default_rng(sum(flags) + 10 * nh_u)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 1.5, nh_d=nh_u)
    u, v, w = random_velocity(rng, n, nh_u)
    uo, vo, wo = u.copy(), v.copy(), w.copy()
    dl = [1 / 14, 1 / 10, 0.0]
    oracle.bounduvw("NNDDDD" * 3, n, [0.0] * 18, nh_u, nh_u, dl, dzc, dzf, uo, vo, wo, isoutflow=flags)
    lib.bounduvw("NNDDDD" * 3, n, [0.0] * 18, nh_u, nh_u, dl, dzc, dzf, u, v, w, isoutflow=flags)
    for a, b in ((u, uo), (v, vo), (w, wo)):
        assert np.array_equal(a, b)
