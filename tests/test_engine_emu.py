"""CPU tests of the GPU transform passes (fft_engine.cuh).

The pre/stage/post passes the kernels run are __host__ __device__ and
barrier-free; libflutas_emu.so runs them on the CPU.  Every BC kind, both
directions, the x-pass (row) and y-pass (column) layouts, FP64 and FP32 are
compared with the oracle's r2r transforms.
"""
import ctypes as C

import numpy as np
import pytest

KINDS = {0: ("R2HC", "HC2R"), 1: ("REDFT10", "REDFT01"), 2: ("RODFT10", "RODFT01"),
         3: ("REDFT11", "REDFT11"), 4: ("RODFT11", "RODFT11")}


@pytest.fixture(scope="module")
def emu():
    from flutas_gb300 import build as B
    L = C.CDLL(B.build_emu())
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    L.fg_emu_lines.argtypes = [C.c_int] * 6 + [dp, dp]
    L.fg_emu_radix_plan.argtypes = [C.c_int, C.POINTER(C.c_int)]
    return L


def test_radix_plans(emu):
    rad = (C.c_int * 16)()
    for N, expect in [(256, [16, 16]), (128, [16, 8]), (512, [8, 8, 8]), (48, [16, 3]),
                      (176, [16, 11]), (1, None)]:
        ns = emu.fg_emu_radix_plan(N, rad)
        if expect is None:
            continue
        assert list(rad[:ns]) == expect
    assert emu.fg_emu_radix_plan(17 * 4, rad) == -1  # prime factor above 13


@pytest.mark.parametrize("dbl", [1, 0, 2], ids=["fp64", "fp32", "df64"])
@pytest.mark.parametrize("pair", [0, 1, 2, 3, 4], ids=["PP", "NN", "DD", "ND", "DN"])
def test_passes_match_oracle(emu, oracle, dbl, pair):
    """Every r2r kind of the engine, FP64, FP32 and double-float (dd.cuh: the FP64
    solver's transforms), against FFTW's definitions in the oracle."""
    rng = np.random.default_rng(pair + 10 * dbl)
    for n in [2, 4, 6, 8, 12, 16, 32, 48, 64, 80, 96, 112, 128, 144, 160, 176, 192, 208, 256, 384,
              512, 9, 15, 21, 25]:
        if pair >= 3 and n % 2:
            continue
        for cols in (0, 1):
            M = 6
            x = rng.standard_normal((M, n))
            for bwd in (0, 1):
                kind = getattr(oracle, KINDS[pair][bwd])
                ref = np.stack([oracle.r2r(kind, x[m]) for m in range(M)])
                xin = np.ascontiguousarray(x if not cols else x.T)
                out = np.zeros_like(xin)
                assert emu.fg_emu_lines(dbl, pair, n, M, bwd, cols, xin, out) == 0
                got = out if not cols else out.T
                tol = {1: 1e-14, 0: 4e-6, 2: 2e-13}[dbl]
                err = np.abs(got - ref).max() / np.abs(ref).max()
                assert err <= tol, (n, cols, bwd, err)


def _trunc_f32(x):
    """FP32 value of x with the mantissa truncated toward zero (numpy reference)."""
    b = x.view(np.uint64) & ~np.uint64((1 << 29) - 1)
    with np.errstate(over="ignore"):
        t = b.view(np.float64).astype(np.float32)
    return np.where(np.abs(x) < 2.0 ** -126, np.copysign(np.float32(0), x).astype(np.float32), t)


def test_bit_conversions(emu):
    """f32_of / f64_of (bits.cuh), the integer-ALU conversions of the FP32 Dodd-Ferrante path."""
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
    emu.fg_emu_f32_of.argtypes = [dp, fp, C.c_long]
    emu.fg_emu_f64_of.argtypes = [fp, dp, C.c_long]
    rng = np.random.default_rng(5)
    edges = [2.0 ** -126, np.nextafter(2.0 ** -126, 0.0), np.nextafter(2.0 ** -126, 1.0), 2.0 ** 127,
             np.nextafter(2.0 ** 128, 0.0), 2.0 ** 128, np.nextafter(2.0 ** -125, 0.0)]  # ends of the fast path
    x = np.concatenate([rng.standard_normal(4000) * 10.0 ** rng.integers(-30, 30, 4000),
                        np.array([0.0, -0.0, 1.0, -1.0, 3.0e38, -3.0e38, 1.5e-38, 2.0 ** -126, 2.0 ** -127]),
                        np.array(edges), -np.array(edges)])
    y = np.empty(len(x), np.float32)
    emu.fg_emu_f32_of(x, y, len(x))
    assert np.array_equal(y.view(np.uint32), _trunc_f32(x).view(np.uint32))
    nrm = (np.abs(x) >= 2.0 ** -126) & (np.abs(x) < np.float64(np.finfo(np.float32).max))
    assert np.all(np.abs(y[nrm] - x[nrm]) <= np.abs(x[nrm]) * 2.0 ** -23)
    # out of range: below 2^-126 -> signed zero, above FP32 max -> inf, NaN stays NaN
    z = np.array([1e-40, -1e-300, 1e39, -1e300, np.inf, -np.inf, np.nan])
    w = np.empty(len(z), np.float32)
    emu.fg_emu_f32_of(z, w, len(z))
    assert w[0] == 0.0 and np.signbit(w[1]) and w[1] == 0.0
    assert w[2] == np.inf and w[3] == -np.inf and w[4] == np.inf and w[5] == -np.inf and np.isnan(w[6])
    tiny = np.array([np.finfo(np.float32).tiny, np.nextafter(np.float32(np.finfo(np.float32).tiny), np.float32(0)),
                     np.finfo(np.float32).max, -np.finfo(np.float32).max], np.float32)
    f = np.concatenate([y[np.isfinite(y)], tiny, np.array([np.inf, -np.inf, np.nan], np.float32)])
    d = np.empty(len(f), np.float64)
    emu.fg_emu_f64_of(np.ascontiguousarray(f), d, len(f))
    normal = (np.abs(f) >= 2.0 ** -126) | (f == 0) | ~np.isfinite(f)
    ok = np.isnan(f) & np.isnan(d) | (f.astype(np.float64) == d)
    assert np.all(ok[normal])


def test_split32_and_diff32(emu):
    """split32: x = h + l exactly in FP32 pieces, |x - h - l| < 2^-46 |x|, h = f32_of(x),
    inside 2^-103 <= |x| < 2^128 and for +-0 (split_ok); diff32: a - b of nearly
    equal values (the cancelling case) to FP32 accuracy, without FP64 arithmetic."""
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    emu.fg_emu_split32.argtypes = [dp, fp, fp, ip, C.c_long]
    emu.fg_emu_diff32.argtypes = [dp, dp, fp, C.c_long]
    emu.fg_emu_f32_of.argtypes = [dp, fp, C.c_long]
    rng = np.random.default_rng(17)
    lo_edge, hi_edge = 2.0 ** -103, 2.0 ** 128
    edges = np.array([lo_edge, np.nextafter(lo_edge, 0.0), np.nextafter(hi_edge, 0.0), hi_edge, 0.0, -0.0,
                      5e-324, np.inf, np.nan, 1.0, np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0)])
    x = np.concatenate([rng.standard_normal(6000) * 10.0 ** rng.integers(-32, 38, 6000), edges, -edges])
    n = len(x)
    h, l, ok = np.empty(n, np.float32), np.empty(n, np.float32), np.empty(n, np.int32)
    emu.fg_emu_split32(x, h, l, ok, n)
    ax = np.abs(x)
    want_ok = ((ax >= lo_edge) & (ax < hi_edge)) | (x == 0)
    assert np.array_equal((ok & 1).astype(bool), want_ok)
    # split_range: the same range without zero; there split32_in / f32_in == split32 / f32_of
    in_range = (ax >= lo_edge) & (ax < hi_edge)
    assert np.array_equal((ok & 6) == 2, in_range) and not np.any(ok & 4)
    t = np.empty(n, np.float32)
    emu.fg_emu_f32_of(x, t, n)
    m = ok.astype(bool) & (x != 0)
    assert np.array_equal(h[m].view(np.uint32), t[m].view(np.uint32))
    s = h.astype(np.float64) + l.astype(np.float64)  # exact: 24 + 23 significant bits
    assert np.all(np.abs(x[m] - s[m]) < ax[m] * 2.0 ** -46)
    z = x == 0
    assert np.all(h[z] == 0) and np.all(l[z] == 0)
    assert np.array_equal(np.signbit(h[z]), np.signbit(x[z]))
    # diff32 on nearby values: error within 2 FP32 roundings of the exact difference
    a = rng.standard_normal(8000) * 10.0 ** rng.integers(-20, 20, 8000)
    rel = 10.0 ** rng.uniform(-12, 0, 8000) * rng.choice([-1.0, 1.0], 8000)
    b = a * (1.0 + rel)
    d = np.empty(len(a), np.float32)
    emu.fg_emu_diff32(a, b, d, len(a))
    exact = a - b  # within 1 FP64 rounding
    err = np.abs(d.astype(np.float64) - exact)
    assert np.all(err <= np.abs(exact) * 2.0 ** -22 + (np.abs(a) + np.abs(b)) * 2.0 ** -45)


@pytest.mark.parametrize("dbl", [0, 1], ids=["f32", "f64"])
@pytest.mark.parametrize("n", [32, 64, 256, 512])
def test_fixed_size_passes_match_engine(emu, dbl, n):
    """fft_fixed.cuh (compile-time N, pre/post folded into the stages) == the run-time engine."""
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    emu.fg_emu_fixed.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, dp, dp]
    rng = np.random.default_rng(n + dbl)
    M = 8
    for pair in (0, 1, 2):
        for bwd in (0, 1):
            x = rng.standard_normal(M * n)
            ref = np.empty_like(x)
            got = np.empty_like(x)
            assert emu.fg_emu_lines(dbl, pair, n, M, bwd, 0, x, ref) == 0
            assert emu.fg_emu_fixed(dbl, pair, n, bwd, x, got) == 0
            tol = 1e-13 if dbl else 2e-6
            assert np.abs(got - ref).max() <= tol * np.abs(ref).max(), (pair, bwd)


@pytest.mark.parametrize("dbl", [0, 1], ids=["f32", "f64"])
@pytest.mark.parametrize("n", [32, 64, 256])
def test_fixed_passes_two_buffer_rotation(emu, dbl, n):
    """The 256^2 plane kernels run each pass with two buffers: the line buffer is the
    second stage's buffer and the forward split lands in the first stage's buffer
    (the inverse writes its lines back over its input).  Run stage by stage, as the
    barriers order them, the rotation gives the separate-buffer results bit for bit."""
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    emu.fg_emu_fixed.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, dp, dp]
    emu.fg_emu_fixed_alias.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, dp, dp]
    rng = np.random.default_rng(7 * n + dbl)
    for pair in (0, 1, 2):
        for bwd in (0, 1):
            x = rng.standard_normal(8 * n)
            ref, got = np.empty_like(x), np.empty_like(x)
            assert emu.fg_emu_fixed(dbl, pair, n, bwd, x, ref) == 0
            assert emu.fg_emu_fixed_alias(dbl, pair, n, bwd, x, got) == 0
            assert np.array_equal(got, ref), (pair, bwd)


EXT_KINDS = {1: "REDFT00", 2: "RODFT00", 3: "RODFT10", 4: "RODFT01", 5: "REDFT11", 6: "RODFT11"}


@pytest.mark.parametrize("kind", sorted(EXT_KINDS), ids=lambda k: EXT_KINDS[k])
@pytest.mark.parametrize("n", [5, 9, 12, 17, 33, 64, 65, 75, 96])
@pytest.mark.parametrize("dbl", [1, 0], ids=["f64", "f32"])
def test_extended_fft_kinds_match_the_oracle(oracle, kind, n, dbl):
    """The face-centred kinds (REDFT00, RODFT00, RODFT10/01 swapped for DN) and the
    odd-length DCT-IV/DST-IV run as one complex DFT of a symmetric extension
    (fft_ext.cuh); executed on the CPU exactly as the kernel runs them, they give
    FFTW's definitions (the oracle's r2r) to rounding.  RODFT00 transforms the first
    n-1 points of a line of n cells and leaves the last one."""
    from flutas_gb300 import build as B
    E = C.CDLL(B.build_emu())
    E.fg_emu_ext.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    E.fg_emu_ext.restype = C.c_int
    rng = np.random.default_rng(n * 10 + kind)
    M = 3
    x = rng.standard_normal((M, n))
    y = np.empty_like(x)
    L = 2 * (n - 1) if kind == 1 else 2 * n
    rc = E.fg_emu_ext(dbl, kind, n, M, x.ctypes.data, y.ctypes.data)
    radix = np.zeros(12, dtype=np.int32)
    if E.fg_emu_radix_plan(L, radix.ctypes.data) < 0:
        assert rc == -2  # a prime factor above 13: refused, not computed
        return
    assert rc == 0
    okind = getattr(oracle, EXT_KINDS[kind])
    for m in range(M):
        if kind == 2:
            ref = np.append(oracle.r2r(okind, x[m, :n - 1]), x[m, n - 1])
        else:
            ref = oracle.r2r(okind, x[m])
        err = np.abs(y[m] - ref).max() / np.abs(ref).max()
        assert err <= (1e-13 if dbl else 2e-6), (n, err)
