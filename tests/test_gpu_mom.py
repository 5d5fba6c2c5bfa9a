"""Momentum predictor on the GPU (rk, src/rk.f90:26-102, with momad_xyz_tw_cen,
momad_xyz_tw_fll and momad_xyz_sp of src/mom.f90) against the oracle.

Tolerance: the kernels evaluate the reference's FP64 expressions term by term;
the GPU contracts products and sums into fused multiply-adds, the oracle does
not, so results agree to rounding: max |difference| <= 1e-12 of the largest
right-hand side for the rates (dudtrko on return) and of the largest velocity
for the updated velocities.  The halo of u, v, w is left untouched, bit for bit.
"""
import numpy as np
import pytest

from conftest import random_velocity, zgrid

pytestmark = pytest.mark.gpu


def _case(seed, n, nh_u, gr):
    rng = np.random.default_rng(seed)
    dzci, dzfi, dzc, dzf = zgrid(n[2], gr, nh_d=nh_u)
    u, v, w = random_velocity(rng, n, nh_u)
    shp = (n[2] + 2, n[1] + 2, n[0] + 2)
    psi = rng.uniform(0, 1, shp)
    rho = psi * 1000.0 + (1 - psi) * 1.0
    mu = psi * 1e-2 + (1 - psi) * 1e-4
    old = [rng.standard_normal((n[2], n[1], n[0])) for _ in range(3)]
    return dzci, dzfi, [u, v, w], mu, rho, old


@pytest.mark.parametrize("scheme,nh_u", [("cen", 1), ("cen", 2), ("fll", 2), ("fll", 3), ("sp", 1)])
@pytest.mark.parametrize("where", ["host", "device"])
def test_gpu_rk_matches_oracle(lib, oracle, scheme, nh_u, where):
    n = [24, 20, 16]
    dzci, dzfi, vel, mu, rho, old = _case(7 + nh_u, n, nh_u, 1.5)
    dxi, dyi, dzi = 24.0, 20.0, 16.0
    f1, f2 = 1.5e-3, -0.5e-3
    visc = 1e-3 / 1.2
    # oracle
    vo = [a.copy() for a in vel]
    oo = [a.copy() for a in old]
    oracle.rk(scheme, f1, f2, n, dxi, dyi, dzi, nh_u, nh_u, dzci, dzfi, *vo, mu, rho, *oo, visc_sp=visc)
    # GPU
    vg = [a.copy() for a in vel]
    og = [a.copy() for a in old]
    if where == "device":
        import torch
        td = [torch.from_numpy(a).cuda() for a in vg + og + [dzci, dzfi, mu, rho]]
        args_v, args_o, (zci, zfi, mud, rhod) = td[:3], td[3:6], td[6:]
    else:
        args_v, args_o, zci, zfi, mud, rhod = vg, og, dzci, dzfi, mu, rho
    if scheme == "sp":
        lib.rk_sp(f1, f2, n, dxi, dyi, dzi, nh_u, nh_u, zci, zfi, visc, *args_v, *args_o)
    else:
        lib.rk(scheme, f1, f2, n, dxi, dyi, dzi, nh_u, nh_u, zci, zfi, *args_v, mud, rhod, *args_o)
    if where == "device":
        vg = [t.cpu().numpy() for t in args_v]
        og = [t.cpu().numpy() for t in args_o]
    h = nh_u
    for a, b, a0 in zip(vg, vo, vel):
        inner = (slice(h, -h),) * 3
        assert np.abs(a[inner] - b[inner]).max() <= 1e-12 * np.abs(b).max()
        halo = a.copy()
        halo[inner] = 0.0
        ref_halo = a0.copy()
        ref_halo[inner] = 0.0
        assert np.array_equal(halo, ref_halo)  # the halo is the caller's, untouched
    for a, b in zip(og, oo):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max(), scheme


def test_gpu_rk_two_steps_and_checks(lib, oracle):
    """Two AB2 steps in a row (the rates carried over in dudtrko), and the argument
    checks: the flux-limiter stencil needs two halo cells; an unknown scheme is refused."""
    n = [32, 16, 12]
    dzci, dzfi, vel, mu, rho, _ = _case(3, n, 2, 0.0)
    zero = [np.zeros((n[2], n[1], n[0])) for _ in range(3)]
    vo, oo = [a.copy() for a in vel], [a.copy() for a in zero]
    vg, og = [a.copy() for a in vel], [a.copy() for a in zero]
    for istep in (1, 2):
        f1, f2, _ = oracle.cmpt_time_factors("ab2", istep, 1, np.zeros((2, 3)), 1e-3, 1e-3)
        oracle.rk("fll", f1, f2, n, 32.0, 16.0, 12.0, 2, 2, dzci, dzfi, *vo, mu, rho, *oo)
        lib.rk("fll", f1, f2, n, 32.0, 16.0, 12.0, 2, 2, dzci, dzfi, *vg, mu, rho, *og)
    for a, b in zip(vg + og, vo + oo):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    d1 = [np.zeros((n[2] + 2, n[1] + 2, n[0] + 2)) for _ in range(3)]
    with pytest.raises(lib.FlutasError) as e:
        lib.rk("fll", 1e-3, 0.0, n, 32.0, 16.0, 12.0, 1, 1, dzci[1:-1], dzfi[1:-1], *d1, mu, rho, *zero)
    assert e.value.code == lib.FLUTAS_EINVAL and "nh_u" in str(e.value)
    with pytest.raises(lib.FlutasError) as e:
        lib.rk("upw", 1e-3, 0.0, n, 32.0, 16.0, 12.0, 2, 2, dzci, dzfi, *vg, mu, rho, *og)
    assert e.value.code == lib.FLUTAS_EINVAL
