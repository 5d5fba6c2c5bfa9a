"""Failure paths, all made on the host: a NaN or Inf planted in an input, an
iteration limit too small for the tolerance, corrupted requests.

The reference stops the run on invalid input (print + MPI_FINALIZE + exit,
src/sanity.f90:332-353, src/fft.f90:879-883) and carries NaN through its
solver without a word.  Here every entry point returns a status instead:
FLUTAS_ENONFINITE for a non-finite solution, FLUTAS_EITER when the refinement
hits its limit, FLUTAS_EINVAL for a request rejected before admission.  No
kernel traps or faults for any of them.
"""
import numpy as np
import pytest

from conftest import compatible_rhs, random_velocity, velocity_ghosts, zgrid

pytestmark = pytest.mark.gpu


def _plan(lib, n, cbc, gr=0.0):
    dzci, dzfi, dzc, dzf = zgrid(n[2], gr)
    P = lib.initsolver(n, [float(n[0]), float(n[1]), float(n[2])], 1, dzci, dzfi, cbc, [0.0] * 6, "ccc")
    return P, dzci, dzfi, dzf


@pytest.mark.parametrize("bad", [np.nan, np.inf], ids=["nan", "inf"])
@pytest.mark.parametrize("where", ["host", "device"])
def test_solver_nonfinite_rhs(lib, bad, where):
    n, cbc = [32, 24, 16], "PPPPNN"
    P, dzci, dzfi, dzf = _plan(lib, n, cbc, 1.0)
    f = compatible_rhs(np.random.default_rng(1), n, cbc, dzf)
    f[9, 7, 5] = bad
    arr = f
    if where == "device":
        import torch
        arr = torch.from_numpy(f).cuda()
    with pytest.raises(lib.FlutasError) as e:
        P.solver(arr)
    assert e.value.code == lib.FLUTAS_ENONFINITE
    # the plan stays usable: a finite RHS solves again
    g = compatible_rhs(np.random.default_rng(2), n, cbc, dzf)
    P.solver(g)
    assert np.all(np.isfinite(g))


def test_solve_mixed_nonfinite_rhs(lib):
    n, cbc = [40, 32, 24], "NNPPDD"
    P, dzci, dzfi, dzf = _plan(lib, n, cbc)
    f = compatible_rhs(np.random.default_rng(3), n, cbc, dzf)
    f[3, 4, 5] = np.nan
    with pytest.raises(lib.FlutasError) as e:
        P.solve_mixed(f, tol=1e-10, max_iter=8)
    assert e.value.code == lib.FLUTAS_ENONFINITE


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_projection_nonfinite_velocity(lib, precision):
    n, cbc = [32, 32, 16], "PPPPNN"
    P, dzci, dzfi, dzf = _plan(lib, n, cbc)
    u, v, w = velocity_ghosts(*random_velocity(np.random.default_rng(4), n), n, cbc)
    w[8, 8, 8] = np.inf
    p = np.zeros((n[2] + 2, n[1] + 2, n[0] + 2))
    with pytest.raises(lib.FlutasError) as e:
        P.projection(1, 32.0, 32.0, dzci, dzfi, [0.0] * 6, 1e-3, 1.0, u, v, w, p, precision=precision, tol=1e-10,
                     max_iter=8)
    assert e.value.code == lib.FLUTAS_ENONFINITE


@pytest.mark.parametrize("form", ["0", "1"], ids=["passes", "persistent"])
def test_batch_nonfinite_rhs(lib, monkeypatch, form):
    monkeypatch.setenv("FLUTAS_GB300_BATCH_PERSISTENT", form)
    grids, rhs = [], []
    rng = np.random.default_rng(5)
    for n, cbc in (((32, 32, 16), "PPPPNN"), ((48, 32, 16), "NNDDNN")):
        dzci, dzfi, dzc, dzf = zgrid(n[2], 0.0)
        grids.append(dict(n=n, dli=[n[0] * 1.0, n[1] * 1.0, 1.0], dzci=dzci, dzfi=dzfi, cbc=cbc))
        rhs.append(compatible_rhs(rng, n, cbc, dzf))
    rhs[1][4, 4, 4] = np.nan
    B = lib.Batch(grids, autotune=False)
    for g, r in enumerate(rhs):
        B.set(g, r)
    with pytest.raises(lib.FlutasError) as e:
        B.solve(tol=1e-8, max_iter=6)
    assert e.value.code == lib.FLUTAS_ENONFINITE
    B.destroy()


def test_iteration_limit_returns_eiter(lib):
    """A tolerance below what the iteration limit allows: FLUTAS_EITER, not a silent result."""
    n, cbc = [48, 40, 24], "PPPPNN"
    P, dzci, dzfi, dzf = _plan(lib, n, cbc, 1.5)
    f = compatible_rhs(np.random.default_rng(6), n, cbc, dzf)
    with pytest.raises(lib.FlutasError) as e:
        P.solve_mixed(f.copy(), tol=1e-15, max_iter=1)
    assert e.value.code == lib.FLUTAS_EITER and "relative residual" in str(e.value)
    u, v, w = velocity_ghosts(*random_velocity(np.random.default_rng(7), n), n, cbc)
    p = np.zeros_like(f)
    with pytest.raises(lib.FlutasError) as e:
        P.projection(1, 48.0, 40.0, dzci, dzfi, [0.0] * 6, 1e-3, 1.0, u, v, w, p, precision=1, tol=1e-15,
                     max_iter=1)
    assert e.value.code == lib.FLUTAS_EITER
    grids = [dict(n=n, dli=[48.0, 40.0, 24.0], dzci=dzci, dzfi=dzfi, cbc=cbc)]
    import os
    for form in ("0", "1"):  # pass kernels, persistent kernel
        os.environ["FLUTAS_GB300_BATCH_PERSISTENT"] = form
        try:
            B = lib.Batch(grids, autotune=False)
        finally:
            del os.environ["FLUTAS_GB300_BATCH_PERSISTENT"]
        B.set(0, f)
        with pytest.raises(lib.FlutasError) as e:
            B.solve(tol=1e-15, max_iter=1)
        assert e.value.code == lib.FLUTAS_EITER
        B.destroy()


def test_server_rejects_corrupted_requests_before_admission(lib):
    n, cbc = [32, 32, 16], "PPPPNN"
    dzci, dzfi, dzc, dzf = zgrid(n[2], 0.0)
    f = compatible_rhs(np.random.default_rng(8), n, cbc, dzf)
    out = np.zeros_like(f)
    S = lib.Server(hbm_budget_bytes=1 << 30, slots=2)
    bad = [dict(n=[1, 32, 16]), dict(n=[32, 32, 2]), dict(cbc="XPPPNN"), dict(cbc="PNPPNN"),
           dict(tol=float("nan")), dict(dli=[32.0, 0.0, 16.0])]
    for b in bad:
        kw = dict(n=n, dli=[32.0, 32.0, 16.0], cbc=cbc, tol=1e-8)
        kw.update(b)
        with pytest.raises(lib.FlutasError) as e:
            S.submit_solve(kw["n"], kw["dli"], dzci, dzfi, kw["cbc"], f, out, tol=kw["tol"])
        assert e.value.code == lib.FLUTAS_EINVAL, b
    # null arrays, through the raw request structure
    import ctypes as C
    req = lib.Request()
    req.kind = 0
    lib.Server._grid(req, n, [32.0, 32.0, 16.0], 1, dzci, dzfi, cbc, 1e-8, 8)
    req.rhs, req.p = None, out.ctypes.data
    t = C.c_longlong()
    assert lib.load().flutas_gb300_server_submit(S.handle, C.byref(req), C.addressof(t)) == lib.FLUTAS_EINVAL
    # a projection request with a bad velocity BC character or dt = 0
    u, v, w = random_velocity(np.random.default_rng(9), n)
    p = np.zeros_like(f)
    with pytest.raises(lib.FlutasError):
        S.submit_projection(n, [32.0, 32.0, 16.0], dzci, dzfi, cbc, u, v, w, p, dt=1e-3, cbcvel="PPPPQD" * 3)
    with pytest.raises(lib.FlutasError):
        S.submit_projection(n, [32.0, 32.0, 16.0], dzci, dzfi, cbc, u, v, w, p, dt=0.0)
    st = S.stats()
    assert st["completed"] == 0 and st["queued"] == 0 and st["inflight"] == 0
    # the server still serves a valid request, and a NaN one fails with ENONFINITE alone
    g = f.copy()
    g[5, 5, 5] = np.nan
    og = np.zeros_like(f)
    t_bad = S.submit_solve(n, [32.0, 32.0, 16.0], dzci, dzfi, cbc, g, og, tol=1e-8)
    t_ok = S.submit_solve(n, [32.0, 32.0, 16.0], dzci, dzfi, cbc, f, out, tol=1e-8)
    g64 = g.copy()
    o64 = np.zeros_like(f)
    t_bad64 = S.submit_solve(n, [32.0, 32.0, 16.0], dzci, dzfi, cbc, g64, o64, tol=0.0)
    assert S.wait(t_bad)[0] == lib.FLUTAS_ENONFINITE
    assert S.wait(t_bad64)[0] == lib.FLUTAS_ENONFINITE
    rc, rr, it, lat = S.wait(t_ok)
    assert rc == 0 and rr <= 1e-8
    S.close()
