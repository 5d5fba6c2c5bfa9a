"""CPU tests of the single-launch ghost-cell update (ghosts.cuh).

boundp and bounduvw set their ghost cells with set_bc's three passes, x then
y then z.  The library composes the passes per cell (k_ghosts) from maps it
builds on the host; libflutas_emu.so runs the same map builders and the same
per-cell composition on the CPU.  The result must equal the oracle's
pass-by-pass restatement bit for bit, for every BC kind, halo widths 1-3,
non-zero BC values and stretched z spacings.
"""
import ctypes as C

import numpy as np
import pytest

@pytest.fixture(scope="module")
def emu():
    from flutas_gb300 import build as B
    L = C.CDLL(B.build_emu())
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    L.fg_emu_boundp.argtypes = [C.c_char_p, ip, dp, dp, C.c_double, C.c_double, dp]
    L.fg_emu_boundp.restype = C.c_int
    L.fg_emu_bounduvw.argtypes = [C.c_char_p, ip, dp, C.c_int, C.c_int, dp, dp, dp, dp, dp, dp]
    L.fg_emu_bounduvw.restype = C.c_int
    L.fg_emu_bounduvw_slabs.argtypes = [C.c_char_p, ip, dp, C.c_int, C.c_int, dp, dp, dp, dp, dp, dp, C.c_int]
    L.fg_emu_bounduvw_slabs.restype = C.c_int
    return L


def _pairs(rng, count):
    """count (low, high) BC pairs: periodic on both ends, or D/N on each."""
    out = []
    for _ in range(count):
        out += ["P", "P"] if rng.uniform() < 0.3 else list(rng.choice(["D", "N"], 2))
    return "".join(out)


@pytest.mark.parametrize("seed", range(24))
def test_boundp_composed_equals_passes(emu, oracle, seed):
    rng = np.random.default_rng(seed)
    n = [int(x) for x in rng.integers(3, 9, 3)]
    cbc = _pairs(rng, 3)
    bc = rng.uniform(-1, 1, 6)
    dzc, dzf, _, _ = oracle.initgrid(n[2], float(rng.uniform(0, 2)), 1.0)
    dl = np.array([1.0 / n[0], 1.0 / n[1], 1.0])
    p = rng.standard_normal((n[2] + 2, n[1] + 2, n[0] + 2))
    ref = p.copy()
    oracle.boundp(cbc, n, list(bc), 1, list(dl), dzc, dzf, ref)
    got = p.copy()
    rc = emu.fg_emu_boundp(cbc.encode(), np.array(n, np.int32), bc, dl, float(dzc[0]), float(dzc[n[2]]), got)
    assert rc == 0
    assert np.array_equal(got, ref), cbc


@pytest.mark.parametrize("h", [1, 2, 3])
@pytest.mark.parametrize("seed", range(16))
def test_bounduvw_composed_equals_passes(emu, oracle, h, seed):
    rng = np.random.default_rng(100 * h + seed)
    n = [int(x) for x in rng.integers(2 * h + 1, 2 * h + 6, 3)]
    cbc = _pairs(rng, 9)  # 18 characters, Fortran (0:1,1:3,1:3) order: side, direction, component
    bc = rng.uniform(-1, 1, 18)
    dzc, dzf, _, _ = oracle.initgrid(n[2], float(rng.uniform(0, 2)), 1.0, h)
    dl = np.array([1.0 / n[0], 1.0 / n[1], 0.0])
    shp = (n[2] + 2 * h, n[1] + 2 * h, n[0] + 2 * h)
    u, v, w = (rng.standard_normal(shp) for _ in range(3))
    ref = [a.copy() for a in (u, v, w)]
    oracle.bounduvw(cbc, n, list(bc), h, h, list(dl), dzc, dzf, *ref)
    got = [a.copy() for a in (u, v, w)]
    rc = emu.fg_emu_bounduvw(cbc.encode(), np.array(n, np.int32), bc, h, h, dl, dzc, dzf, *got)
    assert rc == 0
    for a, b in zip(got, ref):
        assert np.array_equal(a, b), cbc


def test_small_grids_do_not_compose(emu, oracle):
    """Fewer than 2h + 1 cells along an axis: the maps would read written cells; the
    library keeps the pass-by-pass kernel there (the emulator reports 1)."""
    n = [4, 6, 6]
    h = 2
    dzc, dzf, _, _ = oracle.initgrid(n[2], 0.0, 1.0, h)
    shp = (n[2] + 2 * h, n[1] + 2 * h, n[0] + 2 * h)
    u, v, w = (np.zeros(shp) for _ in range(3))
    rc = emu.fg_emu_bounduvw(("DD" * 9).encode(), np.array(n, np.int32), np.zeros(18), h, h,
                             np.array([0.25, 1 / 6, 0.0]), dzc, dzf, u, v, w)
    assert rc == 1


@pytest.mark.parametrize("h", [1, 2, 3])
@pytest.mark.parametrize("seed", range(6))
def test_bounduvw_by_slabs_equals_one_pass(emu, oracle, h, seed):
    """The slab form of the e2e projection fills the ghost cells of each z-slab
    after its planes arrive (k_ghosts_seg): the slabs' segments cover every
    written cell once, each within its slab's planes, and the values equal
    bounduvw's."""
    rng = np.random.default_rng(1000 * h + seed)
    n = [int(x) for x in rng.integers(2 * h + 1, 2 * h + 6, 2)] + [int(rng.integers(2 * h + 3, 40))]
    K = int(rng.integers(h + 2, max(h + 3, n[2] // 2 + 1)))
    cbc = _pairs(rng, 9)
    bc = rng.uniform(-1, 1, 18)
    dzc, dzf, _, _ = oracle.initgrid(n[2], float(rng.uniform(0, 2)), 1.0, h)
    dl = np.array([1.0 / n[0], 1.0 / n[1], 0.0])
    shp = (n[2] + 2 * h, n[1] + 2 * h, n[0] + 2 * h)
    u, v, w = (rng.standard_normal(shp) for _ in range(3))
    ref = [a.copy() for a in (u, v, w)]
    oracle.bounduvw(cbc, n, list(bc), h, h, list(dl), dzc, dzf, *ref)
    got = [a.copy() for a in (u, v, w)]
    rc = emu.fg_emu_bounduvw_slabs(cbc.encode(), np.array(n, np.int32), bc, h, h, dl, dzc, dzf, *got, K)
    assert rc == 0, (rc, n, K, cbc)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b), cbc
