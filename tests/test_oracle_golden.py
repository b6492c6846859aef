"""The CPU oracle (oracle/skewport.cpp) against the reference's own outputs.

The golden fixtures were produced by the reference's CPU code compiled from its
sources (tests/golden/make_golden.py).  Every comparison here is bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import bits_equal, run_cases
from tests.golden.make_golden import OPS

POVH = np.float32(0.15)


def test_golden_runs(oracle, golden_runs):
    cases = run_cases(golden_runs)
    assert len(cases) >= 15
    for key, op, x, want in cases:
        got = oracle.run(op, x, povh=POVH)
        assert bits_equal(got, want), key


def _sector_cases(golden_sectors):
    out = []
    for k in golden_sectors.files:
        if k.endswith("__iinfo"):
            base = k[: -len("__iinfo")]
            name, kind, shape, seed, a = base.split("__")
            out.append((base, name, "__".join([name, kind, shape, seed]), int(a[1:])))
    return sorted(out)


def test_golden_sectors(oracle, golden_sectors):
    cases = _sector_cases(golden_sectors)
    assert len(cases) >= 20
    for base, name, inkey, angle in cases:
        x = golden_sectors[inkey + "__in"]
        si, so, acc = oracle.sector(OPS[name], x, angle, povh=POVH)
        assert bits_equal(si, golden_sectors[base + "__skew_in"]), base + " skew_in"
        assert bits_equal(so, golden_sectors[base + "__skew_out"]), base + " skew_out"
        assert bits_equal(acc.ravel(), golden_sectors[base + "__acc"]), base + " acc"


def test_golden_geometry(port, golden_geometry):
    shapes = sorted({k.split("__")[0] for k in golden_geometry.files})
    for shp in shapes:
        dx, dy = map(int, shp.split("x"))
        ii, dd = golden_geometry[shp + "__iinfo"], golden_geometry[shp + "__dinfo"]
        offs = {"first": 0, "last": 0, "target": 0, "weight": 0}
        dl = max(dx, dy)
        for a in range(180):
            gi = np.zeros(7, np.int32)
            gd = np.zeros(2, np.float64)
            fi = np.zeros(2 * dl + 1, np.uint16)
            la = np.zeros(2 * dl + 1, np.uint16)
            ta = np.zeros(dl, np.int32)
            we = np.zeros(dl, np.float32)
            assert port.port_geometry(dx, dy, a, gi, gd, fi, la, ta, we) == 0
            assert np.array_equal(gi, ii[a]), (shp, a)
            assert np.array_equal(gd.view(np.uint64), dd[a].view(np.uint64)), (shp, a)
            h, di = int(ii[a, 5]), int(ii[a, 2])
            for name, arr, n in (("first", fi, h), ("last", la, h), ("target", ta, di), ("weight", we, di)):
                ref = golden_geometry[f"{shp}__{name}"][offs[name]:offs[name] + n]
                assert np.array_equal(np.asarray(arr[:n]).view(np.uint8), np.asarray(ref).view(np.uint8)), \
                    (shp, a, name)
                offs[name] += n


def test_counts_scale_to_output(oracle, golden_sectors):
    """cv counts times (float)scale^2 reproduce the reference's skewed output."""
    import math
    x = golden_sectors["sdem__fractal__32x32__11__in"]
    for a in (0, 17, 45, 91, 134, 179):
        cnt = oracle.counts(x, a, povh=POVH)
        so = golden_sectors[f"sdem__fractal__32x32__11__a{a}__skew_out"]
        scale = golden_sectors[f"sdem__fractal__32x32__11__a{a}__dinfo"][0]
        r2 = np.float32(scale * scale)
        assert np.all(cnt == np.round(cnt)), a
        assert bits_equal(cnt * r2, so), a
        assert math.isfinite(float(cnt.sum()))


def test_multithread_matches_reference_semantics(oracle, golden_runs):
    """More threads only change the accumulation order: same values to float
    rounding (the reference's own multi-thread runs differ the same way)."""
    x = golden_runs["sdem__fractal__64x64__12__in"]
    one = oracle.run(0, x, povh=POVH, threads=1)
    many = oracle.run(0, x, povh=POVH, threads=4)
    np.testing.assert_allclose(many, one, rtol=1e-5)


def test_accumulate_folds_like_reduce(oracle, golden_runs):
    """Per-type accumulators folded in type order equal the whole run."""
    x = golden_runs["sdem__fractal__32x32__11__in"]
    acc, used = oracle.accumulate(0, x, list(range(180)), povh=POVH)
    assert used == 15
    from skewengine_gb300.parallel import fold_accumulators
    out = fold_accumulators([acc], [used], 32, 32, is_max=False)
    assert bits_equal(out, golden_runs["sdem__fractal__32x32__11__out"])


@pytest.mark.parametrize("dims", [(500, 500), (2000, 2000)])
def test_los_step_counts(port, dims):
    """Line-of-sight steps of the benchmark grids (the sweep's work units)."""
    steps = port.port_los_steps(dims[0], dims[1], 180)
    expect = {500: 1.918e10, 2000: 1.228e12}[dims[0]]
    assert abs(steps - expect) / expect < 0.01


@pytest.mark.parametrize("op", [0, 1, 2, 4, 5])
def test_ordered_parallel_oracle_equals_single_thread(oracle, op):
    """The all-cores oracle mode reproduces the one-thread accumulation order
    bit for bit (square and non-square grids, a scrambled angle list)."""
    from skewengine_gb300 import synthetic
    rng = np.random.default_rng(op)
    for dx, dy in ((40, 40), (37, 23)):
        x = synthetic.fractal_dem(dx, 5 + op, side_y=dy) if op in (0, 1) else \
            synthetic.blurred_texture(dx, 5 + op, side_y=dy)[0]
        angles = rng.permutation(180)[:70] if op != 5 else rng.permutation(180)[:12]
        want = oracle.run_angles(op, x, angles, povh=0.15, threads=1)
        got = oracle.run_ordered(op, x, angles, povh=0.15, threads=5)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (op, dx, dy)


def _reference_build():
    """The reference's own CPU path compiled from its sources (oracle/_ref), built
    here when the sources are present; None where they are not."""
    import ctypes as C
    import os
    import subprocess
    from tests.conftest import ROOT
    path = os.path.join(ROOT, "oracle", "_ref", "libskewref.so")
    if not os.path.exists(path):
        import __graft_entry__ as entry
        if not os.path.isdir(os.path.join(entry.REFERENCE, "src")):
            return None
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={entry.REFERENCE}"],
                       check=True)
    lib = C.CDLL(path)
    fp = np.ctypeslib.ndpointer(np.float32, flags="C")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C")
    lib.skref_run_angles.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, ip, C.c_int, C.c_float, C.c_int]
    lib.skref_set_local_radon.argtypes = [C.c_int]
    return lib


def test_oracle_equals_reference_build_at_workload_sizes(oracle):
    """The oracle against the reference's own CPU code, run here on the
    benchmark workloads' inputs and sizes (the fixtures above are small grids):
    total viewshed of the 500 x 500 fractal DEM, Radon of the 512 x 512 ellipse
    phantom on all 180 angles, cepstrum and local Radon of the 512 x 512
    motion-blurred texture, on angle subsets that span the four sector types,
    reference single-thread order, bit for bit.  Skipped where the reference's
    sources are absent."""
    from skewengine_gb300 import synthetic
    ref = _reference_build()
    if ref is None:
        pytest.skip("the reference's sources are not on this machine")
    dem = synthetic.fractal_dem(500, 1000, roughness=0.8)
    phantom = synthetic.ellipse_phantom(512, 2024)
    texture, _, _ = synthetic.blurred_texture(512, 2024)
    cases = [(0, dem, [0, 1, 17, 44, 45, 46, 63, 89, 90, 91, 112, 135, 158, 179]),
             (2, phantom, list(range(180))),
             (4, texture, [0, 30, 45, 60, 90, 120, 135, 170]),
             (5, texture, [0, 45, 100, 150])]
    for op, x, angles in cases:
        ref.skref_set_local_radon(1 if op == 5 else 0)
        want = np.zeros_like(x)
        a = np.ascontiguousarray(angles, np.int32)
        assert ref.skref_run_angles(2 if op == 5 else op, np.ascontiguousarray(x), want, x.shape[1], x.shape[0],
                                    a, len(a), POVH, 1) == 0
        ref.skref_set_local_radon(0)
        got = oracle.run_ordered(op, x, angles, povh=POVH)
        assert bits_equal(got, want), op


@pytest.mark.parametrize("dims", [(1, 1), (1, 9), (9, 1), (2, 7), (7, 2), (3, 65), (65, 3)])
def test_oracle_equals_reference_build_on_degenerate_grids(oracle, dims):
    """Single cells, single rows and columns and strongly non-square grids, every
    operator over all 180 angles: the oracle against the reference's own CPU
    code run here, bit for bit (NaNs compared as NaNs).  These are the shapes
    the GPU's tiny-grid tests compare with the oracle.  Skipped where the
    reference's sources are absent."""
    ref = _reference_build()
    if ref is None:
        pytest.skip("the reference's sources are not on this machine")
    dx, dy = dims
    angles = np.arange(180, dtype=np.int32)
    for op in (0, 1, 2, 3, 4, 5):
        rng = np.random.default_rng(dx * 100 + dy + op)
        x = (rng.random((dy, dx)) * 150).astype(np.float32)
        ref.skref_set_local_radon(1 if op == 5 else 0)
        want = np.zeros_like(x)
        assert ref.skref_run_angles(2 if op == 5 else op, x, want, dx, dy, angles, 180, POVH, 1) == 0
        ref.skref_set_local_radon(0)
        got = oracle.run_ordered(op, x, angles, povh=POVH)
        same = (got.view(np.uint32) == want.view(np.uint32)) | (np.isnan(got) & np.isnan(want))
        assert same.all(), (dims, op)
