"""CPU tests of the C-ABI boundary: the library builds for sm_103a, loads, and
exports every symbol include/flutas_gb300.h declares; argument validation
rejects bad input before any device work (no GPU needed for these paths).
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np

from conftest import ROOT


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "flutas_gb300.h")).read()
    return sorted(set(re.findall(r"\b(flutas_gb300_\w+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (flutas_gb300_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    # the Python front end binds every one of them
    assert sorted(lib.EXPORTED) == declared_symbols()


def test_initsolver_rejects_bad_bc_without_touching_the_device(lib):
    L = lib.load()
    n = (C.c_int * 3)(8, 8, 8)
    dli = (C.c_double * 3)(8.0, 8.0, 8.0)
    dz = np.ones(10)
    bc = (C.c_double * 6)()
    lam = np.empty(64)
    abc = [np.empty(8) for _ in range(3)]
    rh = [np.empty(128) for _ in range(3)]
    arr = (C.c_void_p * 4)()
    nf = C.c_double()
    for cbc, code in [(b"PPPPNX", lib.FLUTAS_EINVAL), (b"PNPPNN", lib.FLUTAS_EINVAL)]:
        rc = L.flutas_gb300_initsolver(C.cast(n, C.c_void_p), C.cast(dli, C.c_void_p), 1, dz.ctypes.data,
                                       dz.ctypes.data, cbc, C.cast(bc, C.c_void_p), b"ccc", lam.ctypes.data,
                                       abc[0].ctypes.data, abc[1].ctypes.data, abc[2].ctypes.data,
                                       C.cast(arr, C.c_void_p), C.addressof(nf), rh[0].ctypes.data,
                                       rh[1].ctypes.data, rh[2].ctypes.data)
        assert rc == code
        assert lib.last_error()
    # c_or_f is 'c' (cell-centred) or 'f' (face-centred) per axis; anything else is refused
    rc = L.flutas_gb300_initsolver(C.cast(n, C.c_void_p), C.cast(dli, C.c_void_p), 1, dz.ctypes.data,
                                   dz.ctypes.data, b"PPPPNN", C.cast(bc, C.c_void_p), b"ccx",
                                   lam.ctypes.data, abc[0].ctypes.data, abc[1].ctypes.data,
                                   abc[2].ctypes.data, C.cast(arr, C.c_void_p), C.addressof(nf),
                                   rh[0].ctypes.data, rh[1].ctypes.data, rh[2].ctypes.data)
    assert rc == lib.FLUTAS_EINVAL and "c_or_f" in lib.last_error()


def test_invalid_plan_handles_are_rejected(lib):
    L = lib.load()
    assert L.flutas_gb300_fftend(None) == lib.FLUTAS_EINVAL
    bogus = (C.c_void_p * 4)(None, None, None, None)
    assert L.flutas_gb300_fftend(C.cast(bogus, C.c_void_p)) == lib.FLUTAS_EINVAL
    assert L.flutas_gb300_plan_set_stream(None, None, 1) == lib.FLUTAS_EINVAL
    assert "invalid plan" in lib.last_error()


def test_missing_library_fails_loudly(tmp_path):
    import flutas_gb300 as F
    saved = F._lib
    try:
        F._lib = None
        try:
            F.load(str(tmp_path / "nope.so"))
        except F.FlutasError as e:
            assert "missing" in str(e)
        else:
            raise AssertionError("load() of a missing library must raise")
    finally:
        F._lib = saved


def test_pointer_classification_rejects_another_devices_memory():
    """Arrays are used in place only when they live on the current device (or are
    managed); device memory of another GPU is rejected on the host, because a kernel
    on this device would fault on it.  Checked on the pure decision function the
    library uses, with the attribute values cudaPointerGetAttributes reports."""
    from flutas_gb300 import build as B
    E = C.CDLL(B.build_emu())
    E.fg_emu_classify_ptr.argtypes = [C.c_int] * 4
    E.fg_emu_classify_ptr.restype = C.c_int
    HOST, DEVICE, OTHER = 0, 1, 2
    # (attr_ok, type, ptr_device, current_device) -> kind; type 0 unregistered, 1 host, 2 device, 3 managed
    cases = {(0, 0, -1, 0): HOST, (1, 0, -2, 0): HOST, (1, 1, 0, 0): HOST, (1, 1, 1, 0): HOST,
             (1, 2, 0, 0): DEVICE, (1, 2, 3, 3): DEVICE, (1, 2, 1, 0): OTHER, (1, 2, 0, 1): OTHER,
             (1, 3, 0, 0): DEVICE, (1, 3, 1, 0): DEVICE}
    for args, want in cases.items():
        assert E.fg_emu_classify_ptr(*args) == want, args


def test_initgrid_matches_the_oracle(lib, oracle):
    """flutas_gb300_initgrid (host code, no device work) gives the oracle's restatement
    of src/initgrid.f90 bit for bit: two-end and one-end clustering, uniform, wider halos."""
    for inivel, two_end in (("zer", True), ("poi", True), ("hcl", False), ("hcp", False)):
        for n, gr, nh in ((64, 2.0, 1), (33, 1.3, 2), (16, 0.0, 3), (256, 2.5, 1)):
            got = lib.initgrid(inivel, n, gr, 1.7, nh)
            ref = oracle.initgrid(n, gr, 1.7, nh, two_end=two_end)
            for a, b in zip(got, ref):
                assert np.array_equal(a, b), (inivel, n, gr, nh)
    import pytest
    with pytest.raises(lib.FlutasError):
        lib.initgrid("zer", 4, 1.0, 1.0, 5)  # halo wider than the grid


def test_cmpt_time_factors_matches_the_oracle(lib, oracle):
    """cmpt_time_factors (src/rk.f90:104-135): AB2 (Euler at the first step) and the
    three RK3 substeps with the apps' rkcoeff, bit for bit; a bad scheme is refused."""
    import pytest
    rkcoeff = np.array([[32 / 60, 0.0], [25 / 60, -17 / 60], [45 / 60, -25 / 60]]).T  # rkcoeff(2,3)
    for ts, istep, irk in (("ab2", 1, 1), ("ab2", 7, 1), ("rk3", 3, 1), ("rk3", 3, 2), ("rk3", 3, 3)):
        got = lib.cmpt_time_factors(ts, False, istep, irk, rkcoeff, 1.3e-3, 1.1e-3)
        ref = oracle.cmpt_time_factors(ts, istep, irk, rkcoeff, 1.3e-3, 1.1e-3)
        assert got == tuple(float(x) for x in ref), (ts, istep, irk)
    with pytest.raises(lib.FlutasError) as e:
        lib.cmpt_time_factors("ab3", False, 1, 1, rkcoeff, 1e-3, 1e-3)
    assert e.value.code == lib.FLUTAS_EINVAL
