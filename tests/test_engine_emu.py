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


@pytest.mark.parametrize("dbl", [1, 0], ids=["fp64", "fp32"])
@pytest.mark.parametrize("pair", [0, 1, 2, 3, 4], ids=["PP", "NN", "DD", "ND", "DN"])
def test_passes_match_oracle(emu, oracle, dbl, pair):
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
                tol = 1e-14 if dbl else 4e-6
                err = np.abs(got - ref).max() / np.abs(ref).max()
                assert err <= tol, (n, cols, bwd, err)
