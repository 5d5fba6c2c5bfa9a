"""The e2e form of the fused mixed projection on page-locked host arrays copies
w in z-slabs and runs the step's first pass (Dodd-Ferrante terms, bounduvw's
ghost cells, fillps, the forward plane transforms) slab by slab behind the
copies, and corrects u first so that its copy back starts while v, w and p are
corrected.  Its fields must equal, bit for bit, those of the same call with the
slabs switched off (FLUTAS_GB300_SLABS=0) and of the call on device arrays;
z-periodic velocities (ghost planes below the first slab copied from the last
one) keep the one-pass form.  A fused last check that fails (a predicted
contraction of 1e-30) makes the solve go on after u's early copy: u is
corrected again and copied again."""
import numpy as np
import pytest

from conftest import random_velocity, zgrid

pytestmark = pytest.mark.gpu


def _inputs(n, nh_u, cbc, seed):
    rng = np.random.default_rng(seed)
    shp = (n[2] + 2, n[1] + 2, n[0] + 2)
    u, v, w = random_velocity(rng, n, nh_u)
    p, pold = rng.standard_normal(shp), rng.standard_normal(shp)
    rho = np.where(rng.uniform(0, 1, shp) > 0.7, 1000.0, 1.0)
    return dict(rho=rho, pold=pold, u=u, v=v, w=w, p=p)


def _run(lib, n, nh_u, cbc, cbcvel, fields, where, two_phase):
    import torch
    dzci, dzfi, dzc, dzf = zgrid(n[2], 0.0, 1.0, nh_u)
    dxi, dyi, dt = float(n[0]), float(n[1]), 1e-3
    P = lib.initsolver(n, [dxi, dyi, float(n[2])], nh_u, dzci, dzfi, cbc, [0] * 6, "ccc")
    arrs = {}
    for k, a in fields.items():
        if where == "pinned":
            t = torch.empty(a.shape, dtype=torch.float64).pin_memory()
            t.numpy()[...] = a
            arrs[k] = t.numpy()
        else:
            arrs[k] = torch.from_numpy(a.copy()).cuda()
    l0 = lib.launch_count()
    if two_phase:
        P.projection_df(nh_u, dxi, dyi, dzci, dzfi, [0] * 6, dt, dt, 1.0, arrs["rho"], arrs["pold"], arrs["u"],
                        arrs["v"], arrs["w"], arrs["p"], precision=1, tol=1e-10, max_iter=10, cbcvel=cbcvel,
                        bcvel=[0] * 18)
    else:
        P.projection(nh_u, dxi, dyi, dzci, dzfi, [0] * 6, dt, 1.0, arrs["u"], arrs["v"], arrs["w"], arrs["p"],
                     precision=1, tol=1e-10, max_iter=10, cbcvel=cbcvel, bcvel=[0] * 18)
    launches = lib.launch_count() - l0
    rr, it = P.last_solve()
    out = {k: (a.cpu().numpy() if where == "device" else a.copy()) for k, a in arrs.items()}
    P.fftend()
    return out, launches, it


@pytest.mark.parametrize("two_phase,nh_u,cbcvel,slabbed", [
    (True, 1, "PPPPDD" * 3, True),
    (True, 3, "PPPPDD" * 3, True),
    (False, 1, "PPPPDD" * 3, True),
    (True, 1, "PPPPPP" * 3, False),
], ids=["two-phase", "two-phase-halo3", "single-phase", "z-periodic-one-pass"])
def test_slab_projection_equals_one_pass(lib, monkeypatch, two_phase, nh_u, cbcvel, slabbed):
    pytest.importorskip("torch")
    n = [256, 256, 48]  # compile-time plane kernels (256^2, PP), three slabs of 16 planes
    cbc = "PPPPNN" if cbcvel[4] == "D" else "PPPPPP"
    fields = _inputs(n, nh_u, cbc, 11 + nh_u)
    monkeypatch.setenv("FLUTAS_GB300_SLABS", "1")
    a, la, ita = _run(lib, n, nh_u, cbc, cbcvel, fields, "pinned", two_phase)
    monkeypatch.setenv("FLUTAS_GB300_SLABS", "0")
    b, lb, itb = _run(lib, n, nh_u, cbc, cbcvel, fields, "pinned", two_phase)
    c, lc, itc = _run(lib, n, nh_u, cbc, cbcvel, fields, "device", two_phase)
    # the slab form launches the first pass once per slab (the device-array call has
    # no host pold to copy back early, one launch fewer than either host form)
    assert (la > lb) == slabbed and lb >= lc, (la, lb, lc)
    assert ita == itb == itc
    for k in a:
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(a[k], c[k]), k


def test_early_u_copy_redone_when_the_solve_goes_on(lib, monkeypatch):
    pytest.importorskip("torch")
    n = [256, 256, 48]
    cbc, cbcvel = "PPPPNN", "PPPPDD" * 3
    fields = _inputs(n, 1, cbc, 5)
    monkeypatch.setenv("FLUTAS_GB300_CONTRACTION", "1e-30")
    a, la, ita = _run(lib, n, 1, cbc, cbcvel, fields, "pinned", True)
    c, lc, itc = _run(lib, n, 1, cbc, cbcvel, fields, "device", True)
    assert ita == itc and ita >= 2
    for k in a:
        assert np.array_equal(a[k], c[k]), k
