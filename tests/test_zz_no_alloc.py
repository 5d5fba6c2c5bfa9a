"""The allocation-free divergence check (flutas_gb300_chkdiv_noalloc).

Some callers cannot allocate device memory when they call the library: an
application whose own pool owns the whole device, or a diagnostic that runs
after an out-of-memory error.  This entry point keeps its scratch in a fixed
array inside the library instead of calling cudaMalloc.  Its result must match
the regular flutas_gb300_chkdiv, and a second call in a row must give the same
answer (the shared scratch is fully rewritten by every call).  This file is
collected last on purpose and also runs on its own in a fresh process.
"""
import numpy as np
import pytest

from conftest import random_velocity, zgrid

pytestmark = pytest.mark.gpu


def test_chkdiv_noalloc_matches_chkdiv_twice(lib):
    import torch
    n = [40, 24, 20]
    rng = np.random.default_rng(77)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 1.4)
    u, v, w = (torch.from_numpy(a).cuda() for a in random_velocity(rng, n, 1))
    dzfi_d = torch.from_numpy(dzfi).cuda()
    tot_ref, mx_ref = lib.chkdiv(n, 40.0, 24.0, 20.0, 1, 1, dzfi_d, u, v, w)
    for _ in range(2):
        tot, mx = lib.chkdiv_noalloc(n, 40.0, 24.0, 20.0, 1, 1, dzfi_d, u, v, w)
        assert mx == pytest.approx(mx_ref, rel=1e-14)
        assert tot == pytest.approx(tot_ref, rel=1e-10, abs=1e-9 * abs(mx_ref) * np.prod(n))


def test_chkdiv_noalloc_leaves_device_free_memory_unchanged(lib):
    """The property the entry point exists for: once its kernels are loaded on the
    device (one warm-up call), further calls take no device memory.  Free device
    memory (cudaMemGetInfo) is the same before and after several calls."""
    import torch
    n = [64, 48, 40]
    rng = np.random.default_rng(78)
    dzci, dzfi, dzc, dzf = zgrid(n[2], 1.2)
    u, v, w = (torch.from_numpy(a).cuda() for a in random_velocity(rng, n, 1))
    dzfi_d = torch.from_numpy(dzfi).cuda()
    lib.chkdiv_noalloc(n, 64.0, 48.0, 40.0, 1, 1, dzfi_d, u, v, w)  # warm-up: kernels loaded
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    first = lib.chkdiv_noalloc(n, 64.0, 48.0, 40.0, 1, 1, dzfi_d, u, v, w)
    for _ in range(4):
        assert lib.chkdiv_noalloc(n, 64.0, 48.0, 40.0, 1, 1, dzfi_d, u, v, w) == first
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_chkdiv_noalloc_rejects_oversized_and_host_arrays(lib):
    import torch
    n = [8, 300, 300]  # 90000 rows > 65536
    u = torch.zeros((n[2] + 2, n[1] + 2, n[0] + 2), dtype=torch.float64, device="cuda")
    dz = torch.ones(n[2] + 2, dtype=torch.float64, device="cuda")
    with pytest.raises(lib.FlutasError) as e:
        lib.chkdiv_noalloc(n, 1.0, 1.0, 1.0, 1, 1, dz, u, u, u)
    assert e.value.code == lib.FLUTAS_EINVAL and "rows" in str(e.value)
    h = np.zeros((6, 6, 6))
    with pytest.raises(lib.FlutasError) as e:
        lib.chkdiv_noalloc([4, 4, 4], 1.0, 1.0, 1.0, 1, 1, np.ones(6), h, h, h)
    assert e.value.code == lib.FLUTAS_EINVAL
