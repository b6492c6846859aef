"""The allocation-free sweep entry point, ske_sdem_sector_noalloc.

It exists for callers that cannot allocate GPU memory (a fixed memory budget,
another framework's allocator, a path where cudaMalloc is not allowed): its
scratch lives in a static device array inside the library.  This test calls it
through the C ABI on sectors the engine has skewed, twice in a row, and checks
each output against the engine's own total-viewshed operator bit for bit.  The
file sorts last so that a run stopping at the first failure has already run
every other test; it needs nothing from them and also passes on its own.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from skewengine_gb300 import synthetic

pytestmark = pytest.mark.gpu

POVH = np.float32(0.15)


def test_noalloc_sweep_matches_engine(gpu_lib):
    torch = pytest.importorskip("torch")
    import skewengine_gb300 as ske

    x = synthetic.fractal_dem(200, 77, side_y=160)
    with ske.SkewEngine(200, 160) as eng:
        eng.prepare(x)
        for angle in (30, 100):  # two calls in a row on different sectors
            eng.skew(angle)
            eng.kernel(ske.KERNEL_SDEM, POVH)
            _, want = eng.skewed()
            v = eng.sector()
            out = torch.zeros(eng.skew_len, dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            scale2 = np.float32(v.geom.scale * v.geom.scale)
            rc = gpu_lib.ske_sdem_sector_noalloc(0, v.skew_in, C.c_void_p(out.data_ptr()), v.geom.dim_i,
                                                 v.geom.skew_height, v.geom.dim_l, v.first, v.last,
                                                 float(scale2), float(POVH), C.c_void_p(eng.stream))
            assert rc == 0, gpu_lib.ske_last_error().decode()
            got = out.cpu().numpy()
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), angle


def test_noalloc_rejects_oversized_sector(gpu_lib):
    p = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = gpu_lib.ske_sdem_sector_noalloc(0, p, p, 5000, 10, 5000, p, p, 1.0, 0.15, None)
    assert rc == 1
    assert b"4096" in gpu_lib.ske_last_error()


def _call(gpu_lib, skew, first, last, dim_i, h, dim_l, device=0):
    return gpu_lib.ske_sdem_sector_noalloc(device, C.c_void_p(skew.data_ptr()), C.c_void_p(skew.data_ptr()), dim_i,
                                           h, dim_l, C.c_void_p(first.data_ptr()), C.c_void_p(last.data_ptr()),
                                           1.0, float(POVH), None)


def test_noalloc_rejects_rows_outside_the_grid(gpu_lib):
    """A row whose last passes dim_l, or whose first lies far beyond the grid
    with a short length, is refused before any device work; the caller's
    buffers (sized for the valid rows) are never touched."""
    torch = pytest.importorskip("torch")
    dim_i, h, dim_l = 64, 8, 64
    skew = torch.zeros((h - 1) * dim_i + dim_l, dtype=torch.float32, device="cuda")
    first = torch.zeros(h, dtype=torch.int32, device="cuda")
    good = torch.full((h,), dim_l, dtype=torch.int32, device="cuda")
    assert _call(gpu_lib, skew, first, good, dim_i, h, dim_l) == 0, gpu_lib.ske_last_error().decode()
    cases = []
    last = good.clone()
    last[3] = dim_l + 1
    cases.append((first, last))
    far_first = first.clone()
    far_last = good.clone()
    far_first[5] = 1 << 30
    far_last[5] = (1 << 30) + 10
    cases.append((far_first, far_last))
    neg = first.clone()
    neg[0] = -1
    cases.append((neg, good))
    crossed = first.clone()
    crossed[2] = 10
    crossed_last = good.clone()
    crossed_last[2] = 5
    cases.append((crossed, crossed_last))
    for f, l in cases:
        torch.cuda.synchronize()
        assert _call(gpu_lib, skew, f, l, dim_i, h, dim_l) == 1
        assert b"first/last" in gpu_lib.ske_last_error()


def test_noalloc_rejects_too_many_rows_and_items(gpu_lib):
    torch = pytest.importorskip("torch")
    # More skewed rows than the static row arrays hold: refused before reading them.
    p = C.c_void_p(16)  # never dereferenced
    rc = gpu_lib.ske_sdem_sector_noalloc(0, p, p, 64, (1 << 17) + 1, 64, p, p, 1.0, 0.15, None)
    assert rc == 1 and b"131072" in gpu_lib.ske_last_error()
    # 131072 rows of 4096 cells at row stride 1 need 2^22 work items of 128
    # observers (the static item list holds 2^20).  Every row reads cells
    # r + [0, 4096) only, all inside the buffer, had it run.
    h, dim_l = 1 << 17, 4096
    skew = torch.zeros(h - 1 + dim_l, dtype=torch.float32, device="cuda")
    first = torch.zeros(h, dtype=torch.int32, device="cuda")
    last = torch.full((h,), dim_l, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert _call(gpu_lib, skew, first, last, 1, h, dim_l) == 1
    assert b"2^20" in gpu_lib.ske_last_error()


def test_noalloc_rejects_missing_device_and_keeps_current_device(gpu_lib):
    torch = pytest.importorskip("torch")
    p = C.c_void_p(16)  # never dereferenced: the device check comes first
    n = torch.cuda.device_count()
    rc = gpu_lib.ske_sdem_sector_noalloc(n, p, p, 64, 8, 64, p, p, 1.0, 0.15, None)
    assert rc == 3 and b"device" in gpu_lib.ske_last_error()
    # A successful call leaves the calling thread's current device as it was.
    skew = torch.zeros(7 * 64 + 64, dtype=torch.float32, device="cuda:0")
    first = torch.zeros(8, dtype=torch.int32, device="cuda:0")
    last = torch.full((8,), 64, dtype=torch.int32, device="cuda:0")
    before = torch.cuda.current_device()
    torch.cuda.synchronize()
    assert _call(gpu_lib, skew, first, last, 64, 8, 64) == 0
    assert torch.cuda.current_device() == before
