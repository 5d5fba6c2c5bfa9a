"""Serving: the continuous-batching request loop.  Requests of different sizes,
BCs and tolerances are admitted while others run (their work overlaps on the
device); each result must be the same as the same request solved alone, within
the tolerance the request asked for.  The HBM budget gates admission."""
import numpy as np
import pytest

from conftest import compatible_rhs, random_velocity, rel_l2, singular, velocity_ghosts, zgrid

pytestmark = pytest.mark.gpu

REQS = [
    ((64, 64, 32), "PPPPNN", 0.0, 1e-6),
    ((96, 48, 40), "NNPPND", 2.0, 1e-10),
    ((32, 128, 24), "DDNNDD", 1.0, 1e-10),
    ((80, 80, 16), "PPPPPP", 0.0, 1e-6),
    ((128, 64, 48), "NNNNNN", 1.5, 1e-10),
    ((48, 48, 48), "PPDDNN", 0.5, 1e-6),
    ((64, 32, 64), "PPPPNN", 2.0, 1e-10),
    ((112, 96, 20), "DDPPNN", 0.0, 1e-10),
]


def _requests(seed=9):
    rng = np.random.default_rng(seed)
    out = []
    for n, cbc, gr, tol in REQS:
        dzci, dzfi, dzc, dzf = zgrid(n[2], gr)
        dli = [n[0] * 1.0, n[1] * 1.0, 1.0]
        out.append(dict(n=n, cbc=cbc, dli=dli, dzci=dzci, dzfi=dzfi, tol=tol, rhs=compatible_rhs(rng, n, cbc, dzf)))
    return out


def test_serving_results_match_alone(lib):
    reqs = _requests()
    S = lib.Server(hbm_budget_bytes=8 << 30, slots=4)
    outs, tickets = [], []
    for r in reqs:
        o = np.zeros_like(r["rhs"])
        outs.append(o)
        tickets.append(S.submit_solve(r["n"], r["dli"], r["dzci"], r["dzfi"], r["cbc"], r["rhs"], o, tol=r["tol"]))
    res, errs = [], []
    for t in tickets:
        res.append(S.wait(t))
        errs.append(lib.last_error() if res[-1][0] else "")
    st = S.stats()
    assert st["completed"] == len(reqs) and st["p99_ms"] >= st["p50_ms"] > 0, [(r[0], e) for r, e in zip(res, errs)]
    # continuous batching, not a queue: requests were on the device at the same time
    # (spans from CUDA events recorded on the workers' streams)
    assert st["max_device_overlap"] >= 2, st
    S.close()
    for r, o, (rc, rr, it, lat) in zip(reqs, outs, res):
        assert rc == 0 and rr <= r["tol"] and it >= 1 and lat > 0
        P = lib.initsolver(r["n"], r["dli"], 1, r["dzci"], r["dzfi"], r["cbc"], [0.0] * 6, "ccc")
        alone = r["rhs"].copy()
        rr2, _ = P.solve_mixed(alone, tol=r["tol"], max_iter=8)
        assert rr2 <= r["tol"]
        # the same plan kinds and kernels run alone and in the mix: the results agree
        # within the request's own tolerance (in practice bit for bit)
        d = rel_l2(o[1:-1, 1:-1, 1:-1], alone[1:-1, 1:-1, 1:-1], remove_mean=singular(r["cbc"]))
        print(f"served vs alone {r['n']} {r['cbc']}: {d:.2e}")
        assert d <= r["tol"], (r["n"], d)


def test_serving_budget_admission(lib):
    reqs = _requests(seed=10)[:4]
    biggest = max(int(np.prod([x + 2 for x in r["n"]])) for r in reqs) * 8
    # room for about one request at a time: everything still completes, one after another
    S = lib.Server(hbm_budget_bytes=6 * biggest, slots=4)
    outs = [np.zeros_like(r["rhs"]) for r in reqs]
    ts = [S.submit_solve(r["n"], r["dli"], r["dzci"], r["dzfi"], r["cbc"], r["rhs"], o, tol=r["tol"])
          for r, o in zip(reqs, outs)]
    assert all(S.wait(t)[0] == 0 for t in ts)
    S.close()
    # a request larger than the whole budget is refused with FLUTAS_ENOMEM, not run out of memory
    S = lib.Server(hbm_budget_bytes=1 << 20, slots=2)
    r = reqs[0]
    o = np.zeros_like(r["rhs"])
    t = S.submit_solve(r["n"], r["dli"], r["dzci"], r["dzfi"], r["cbc"], r["rhs"], o, tol=1e-6)
    assert S.wait(t)[0] == lib.FLUTAS_ENOMEM
    S.close()


def test_serving_two_phase_projection_request(lib):
    n, cbc, cbcvel = [32, 32, 16], "PPPPNN", "PPPPDD" * 3
    rng = np.random.default_rng(4)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 0.0)
    dxi, dyi, dt = 32.0, 32.0, 1e-3
    shp = (n[2] + 2, n[1] + 2, n[0] + 2)
    u, v, w = velocity_ghosts(*random_velocity(rng, n, 1), n, cbc)
    p, pold = rng.standard_normal(shp), rng.standard_normal(shp)
    rho = 1.0 + 999.0 * (rng.uniform(0, 1, shp) > 0.6)
    fields = [a.copy() for a in (u, v, w, p)]
    S = lib.Server(hbm_budget_bytes=4 << 30, slots=2)
    t = S.submit_projection(n, [dxi, dyi, 16.0], dzci, dzfi, cbc, *fields, dt=dt, rho=rho, pold=pold, tol=1e-10,
                            cbcvel=cbcvel)
    rc, rr, it, lat = S.wait(t)
    S.close()
    assert rc == 0 and rr <= 1e-10
    P = lib.initsolver(n, [dxi, dyi, 16.0], 1, dzci, dzfi, cbc, [0.0] * 6, "ccc")
    alone = [a.copy() for a in (u, v, w, p)]
    P.projection_df(1, dxi, dyi, dzci, dzfi, [0.0] * 6, dt, dt, 1.0, rho, pold, *alone, precision=1, tol=1e-10,
                    max_iter=8, cbcvel=cbcvel, bcvel=[0.0] * 18)
    for a, b in zip(fields, alone):
        assert rel_l2(a, b) <= 1e-9


def test_serving_fp64_requests(lib):
    """tol = 0 serves the plain FP64 solver: the result equals the drop-in call's."""
    reqs = _requests(seed=12)[:3]
    S = lib.Server(hbm_budget_bytes=8 << 30, slots=2)
    outs = [np.zeros_like(r["rhs"]) for r in reqs]
    ts = [S.submit_solve(r["n"], r["dli"], r["dzci"], r["dzfi"], r["cbc"], r["rhs"], o, tol=0.0)
          for r, o in zip(reqs, outs)]
    res = [S.wait(t) for t in ts]
    S.close()
    for r, o, (rc, rr, it, lat) in zip(reqs, outs, res):
        assert rc == 0 and it == 0
        P = lib.initsolver(r["n"], r["dli"], 1, r["dzci"], r["dzfi"], r["cbc"], [0.0] * 6, "ccc")
        alone = r["rhs"].copy()
        P.solver(alone)
        assert np.array_equal(o[1:-1, 1:-1, 1:-1], alone[1:-1, 1:-1, 1:-1])


def test_serving_device_resident_fields(lib):
    """Requests whose arrays live on the device are solved in place (no staging
    copies, no field memory charged to the budget): the same result as the host-array
    request, bit for bit, and the RHS array is left as it was."""
    import torch
    reqs = _requests(seed=21)[:4]
    S = lib.Server(hbm_budget_bytes=8 << 30, slots=2)
    host_out = [np.zeros_like(r["rhs"]) for r in reqs]
    dev_rhs = [torch.from_numpy(r["rhs"]).cuda() for r in reqs]
    dev_out = [torch.zeros_like(t) for t in dev_rhs]
    th = [S.submit_solve(r["n"], r["dli"], r["dzci"], r["dzfi"], r["cbc"], r["rhs"], o, tol=r["tol"])
          for r, o in zip(reqs, host_out)]
    td = [S.submit_solve(r["n"], r["dli"], r["dzci"], r["dzfi"], r["cbc"], x, o, tol=r["tol"])
          for r, x, o in zip(reqs, dev_rhs, dev_out)]
    assert all(S.wait(t)[0] == 0 for t in th + td)
    S.close()
    for a, b in zip(host_out, dev_out):
        assert np.array_equal(a, b.cpu().numpy())
    assert all(np.array_equal(r["rhs"], x.cpu().numpy()) for r, x in zip(reqs, dev_rhs))
