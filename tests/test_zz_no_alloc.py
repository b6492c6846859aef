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
