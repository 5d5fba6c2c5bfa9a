"""Restart-file I/O (src/load.f90) through the C ABI.

Host-array cases run on the CPU; device-array cases are marked gpu.  Files are
raw FP64 values of the global interior, x fastest, no header."""
import numpy as np
import pytest

import flutas_gb300 as F


def _lib_or_skip():
    try:
        F.load()
    except Exception as e:  # library not built
        pytest.skip(f"library not available: {e}")


def test_load_host_round_trip(tmp_path):
    _lib_or_skip()
    rng = np.random.default_rng(3)
    n = (12, 10, 7)
    interior = rng.standard_normal((n[2], n[1], n[0]))
    fn = tmp_path / "fldu.bin"
    interior.tofile(fn)
    for nh in (0, 1, 3):
        fld = np.full((n[2] + 2 * nh, n[1] + 2 * nh, n[0] + 2 * nh), 7.5)
        F.load_field("r", fn, n, fld, nh)
        inner = fld[nh:nh + n[2], nh:nh + n[1], nh:nh + n[0]]
        assert np.array_equal(inner, interior)
        if nh:  # the halo is left alone
            mask = np.ones(fld.shape, bool)
            mask[nh:nh + n[2], nh:nh + n[1], nh:nh + n[0]] = False
            assert np.all(fld[mask] == 7.5)
        out = tmp_path / f"out{nh}.bin"
        F.load_field("w", out, n, fld, nh)
        assert out.read_bytes() == fn.read_bytes()


def test_load_checks_like_the_reference(tmp_path):
    _lib_or_skip()
    n = (8, 8, 8)
    fld = np.zeros((10, 10, 10))
    with pytest.raises(F.FlutasError) as e:
        F.load_field("r", tmp_path / "missing.bin", n, fld)
    assert e.value.code == F.FLUTAS_EINVAL and "does not exist" in str(e.value)
    bad = tmp_path / "short.bin"
    np.zeros(8 * 8 * 8 - 1).tofile(bad)
    with pytest.raises(F.FlutasError) as e:
        F.load_field("r", bad, n, fld)
    assert "incorrect size" in str(e.value) and "4096" in str(e.value) and "4088" in str(e.value)
    with pytest.raises(F.FlutasError):
        F.load_field("x", bad, n, fld)


def test_load_scalar_format(tmp_path):
    _lib_or_skip()
    fn = tmp_path / "scalar.out"
    F.load_scalar("w", fn, 1.234567, 42, -0.001)
    # write(88,'(2E15.7, 1I9.8)') time, dto, istep
    assert fn.read_text() == "  0.1234567E+01 -0.1000000E-02 00000042\n"
    assert F.load_scalar("r", fn) == (1.234567, 42, -0.001)
    F.load_scalar("w", fn, 0.0, 7, 9.99999996)
    assert fn.read_text() == "  0.0000000E+00  0.1000000E+02 00000007\n"
    fn.write_text("1.5D0, 2.5d-3, 17\n")  # list-directed input as Fortran reads it
    assert F.load_scalar("r", fn) == (1.5, 17, 0.0025)


def test_load_ns_round_trip(tmp_path):
    _lib_or_skip()
    rng = np.random.default_rng(4)
    n = (6, 5, 4)
    flds = [rng.standard_normal((n[2] + 2, n[1] + 2, n[0] + 2)) for _ in range(4)]
    fn = tmp_path / "fld.bin"
    F.load_ns("w", fn, n, *flds, time=0.75, istep=1200.0)
    raw = np.fromfile(fn)
    assert raw.size == 4 * np.prod(n) + 2 and raw[-2] == 0.75 and raw[-1] == 1200.0
    back = [np.zeros_like(f) for f in flds]
    t, it = F.load_ns("r", fn, n, *back)
    assert (t, it) == (0.75, 1200.0)
    for a, b in zip(flds, back):
        assert np.array_equal(a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1])


@pytest.mark.gpu
def test_load_device_round_trip(tmp_path):
    import torch
    rng = np.random.default_rng(5)
    n = (40, 24, 33)  # several file chunks are not needed: one per call here
    interior = rng.standard_normal((n[2], n[1], n[0]))
    fn = tmp_path / "fldp.bin"
    interior.tofile(fn)
    dev = torch.full((n[2] + 2, n[1] + 2, n[0] + 2), -1.0, dtype=torch.float64, device="cuda")
    F.load_field("r", fn, n, dev, 1)
    got = dev.cpu().numpy()
    assert np.array_equal(got[1:-1, 1:-1, 1:-1], interior)
    assert np.all(got[0] == -1.0) and np.all(got[:, :, -1] == -1.0)
    out = tmp_path / "out.bin"
    F.load_field("w", out, n, dev, 1)
    assert out.read_bytes() == fn.read_bytes()
    flat = torch.zeros(n[2], n[1], n[0], dtype=torch.float64, device="cuda")
    F.load_field("r", fn, n, flat, 0)
    assert np.array_equal(flat.cpu().numpy(), interior)
