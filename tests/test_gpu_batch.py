"""Batched mixed-precision solves: many grids of uneven sizes and BCs in one
graph-replayed sequence of work-queue pass kernels (the default), or in one
persistent kernel that drains a (pass, grid, tile) queue
(FLUTAS_GB300_BATCH_PERSISTENT=1).  Each grid must reach the requested relative
residual, agree with the FP64 oracle within the error that residual allows, and
give the same answer alone (single-grid mixed solve) as in the batch; the two
batch forms give the same solutions bit for bit."""
import numpy as np
import pytest

from conftest import compatible_rhs, rel_l2, singular, zgrid

pytestmark = pytest.mark.gpu

GRIDS = [
    ((32, 48, 16), "PPPPNN", 0.0),
    ((48, 32, 24), "NNPPNN", 1.5),
    ((64, 64, 32), "DDNNDD", 2.0),
    ((80, 48, 16), "PPDDPP", 0.0),
    ((112, 32, 20), "NNNNND", 1.0),
    ((96, 80, 12), "DDPPDD", 2.5),
    ((32, 32, 32), "PPPPPP", 0.0),
    ((144, 16, 8), "PPNNNN", 1.2),
]


def _batch_inputs():
    rng = np.random.default_rng(123)
    grids, rhs = [], []
    for n, cbc, gr in GRIDS:
        dzci, dzfi, dzc, dzf = zgrid(n[2], gr)
        grids.append(dict(n=n, dli=[n[0] * 1.0, n[1] * 1.1, 1.0], dzci=dzci, dzfi=dzfi, cbc=cbc))
        rhs.append(compatible_rhs(rng, n, cbc, dzf))
    return grids, rhs


@pytest.fixture(params=["passes", "persistent"])
def batch_form(request, monkeypatch):
    monkeypatch.setenv("FLUTAS_GB300_BATCH_PERSISTENT", "1" if request.param == "persistent" else "0")
    return request.param


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_batch_matches_oracle_and_single(lib, oracle, tol, batch_form):
    grids, rhs = _batch_inputs()
    B = lib.Batch(grids, autotune=True)
    for g, r in enumerate(rhs):
        B.set(g, r)
    relres, iters = B.solve(tol=tol, max_iter=8)
    assert np.all(relres <= tol), relres
    assert np.all(iters >= 1)
    for g, (gd, r) in enumerate(zip(grids, rhs)):
        got = B.get(g)
        S = oracle.SolverSetup(gd["n"], gd["dli"], 1, gd["dzci"], gd["dzfi"], gd["cbc"], [0] * 6, "ccc")
        ref = r.copy()
        S.solve(ref)
        sing = singular(gd["cbc"])
        e = rel_l2(got[1:-1, 1:-1, 1:-1], ref[1:-1, 1:-1, 1:-1], remove_mean=sing)
        assert e <= max(1e3 * tol, 1e-12), (g, e)
        # alone: the single-grid mixed solve of the same problem
        P = lib.initsolver(gd["n"], gd["dli"], 1, gd["dzci"], gd["dzfi"], gd["cbc"], [0.0] * 6, "ccc")
        alone = r.copy()
        rr, _ = P.solve_mixed(alone, tol=tol, max_iter=8)
        assert rr <= tol
        d = rel_l2(got[1:-1, 1:-1, 1:-1], alone[1:-1, 1:-1, 1:-1], remove_mean=sing)
        assert d <= max(1e3 * tol, 1e-12), (g, d)
    assert "maxe" in B.report()
    B.destroy()


def test_batch_second_solve_reuses_graph(lib, batch_form):
    grids, rhs = _batch_inputs()
    B = lib.Batch(grids[:3], autotune=False)
    for g in range(3):
        B.set(g, rhs[g])
    r1, _ = B.solve(tol=1e-8)
    sol1 = [B.get(g) for g in range(3)]
    for g in range(3):
        B.set(g, rhs[g])
    r2, _ = B.solve(tol=1e-8)
    for g in range(3):
        assert np.array_equal(sol1[g], B.get(g))
    assert np.array_equal(r1, r2)


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_batch_grid_alone_equals_in_batch(lib, tol):
    """Each grid solved in a batch of one (the same tuned transform plans and tile
    shapes, cached per process) gives the result it gets among the other grids,
    within the requested tolerance (in practice bit for bit)."""
    grids, rhs = _batch_inputs()
    B = lib.Batch(grids, autotune=True)
    for g, r in enumerate(rhs):
        B.set(g, r)
    B.solve(tol=tol, max_iter=8)
    mixed = [B.get(g) for g in range(len(grids))]
    B.destroy()
    for g, (gd, r) in enumerate(zip(grids, rhs)):
        A = lib.Batch([gd], autotune=True)
        A.set(0, r)
        rr, _ = A.solve(tol=tol, max_iter=8)
        alone = A.get(0)
        A.destroy()
        assert rr[0] <= tol
        d = rel_l2(mixed[g][1:-1, 1:-1, 1:-1], alone[1:-1, 1:-1, 1:-1], remove_mean=singular(gd["cbc"]))
        print(f"batch grid {g} in the mix vs alone: {d:.2e}")
        assert d <= tol, (g, d)


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_persistent_kernel_equals_pass_kernels(lib, monkeypatch, tol):
    """The persistent kernel runs the same tiles as the pass kernels: the same
    FP32 solves per grid and the same solutions, bit for bit."""
    grids, rhs = _batch_inputs()
    out = {}
    monkeypatch.setenv("FLUTAS_GB300_BATCH_PLANES", "0")  # row and column tiles in both forms
    for form in ("0", "1"):
        monkeypatch.setenv("FLUTAS_GB300_BATCH_PERSISTENT", form)
        monkeypatch.setenv("FLUTAS_GB300_BATCH_STATS", form)
        B = lib.Batch(grids, autotune=False)
        for g, r in enumerate(rhs):
            B.set(g, r)
        rr, it = B.solve(tol=tol, max_iter=8)
        out[form] = (rr, it, [B.get(g) for g in range(len(grids))], B.report())
        B.destroy()
    assert np.array_equal(out["0"][1], out["1"][1])
    np.testing.assert_allclose(out["0"][0], out["1"][0], rtol=1e-9)  # norms summed in another order
    for a, b in zip(out["0"][2], out["1"][2]):
        assert np.array_equal(a, b)
    q = [ln for ln in out["1"][3].splitlines() if ln.startswith("queue:")]
    assert q and "0 tiles skipped" not in q[0], out["1"][3]


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_whole_plane_items_equal_row_and_column_tiles(lib, oracle, monkeypatch, tol):
    """Grids whose planes fit one CTA take both transforms of a plane per item
    (kb_xyfwd_plane / kb_xyinv_plane); the same batch with row and column tiles
    (FLUTAS_GB300_BATCH_PLANES=0) reaches tol as well, and the two solutions
    agree within it.  A 192x160 grid stays on rows and columns in both."""
    grids, rhs = _batch_inputs()
    rng = np.random.default_rng(9)
    dzci, dzfi, dzc, dzf = zgrid(12, 0.0)
    grids.append(dict(n=(192, 160, 12), dli=[192.0, 176.0, 1.0], dzci=dzci, dzfi=dzfi, cbc="PPNNDD"))
    rhs.append(compatible_rhs(rng, (192, 160, 12), "PPNNDD", dzf))
    sols = {}
    for planes in ("1", "0"):
        monkeypatch.setenv("FLUTAS_GB300_BATCH_PLANES", planes)
        B = lib.Batch(grids, autotune=False)
        for g, r in enumerate(rhs):
            B.set(g, r)
        rr, it = B.solve(tol=tol, max_iter=8)
        assert np.all(rr <= tol), (planes, rr)
        if planes == "1":
            assert "whole planes" in B.report()
        sols[planes] = [B.get(g) for g in range(len(grids))]
        B.destroy()
    for g, gd in enumerate(grids):
        d = rel_l2(sols["1"][g][1:-1, 1:-1, 1:-1], sols["0"][g][1:-1, 1:-1, 1:-1], remove_mean=singular(gd["cbc"]))
        assert d <= max(10 * tol, 1e-12), (g, d)
