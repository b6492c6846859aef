"""GPU parity: the sm_103a kernels, called through the C ABI, against the
reference's golden outputs and the CPU oracle.

Bar: bit-exact (float32 bit patterns) for total viewshed, identity and Radon in
reference accumulation order, and for the integer visibility counts; cepstrum is
compared in its output bins (the GPU log may differ from the host libm's in the
last place) and must also match bit for bit on the golden cases.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from skewengine_gb300 import synthetic
from tests.conftest import bits_equal, run_cases

pytestmark = pytest.mark.gpu

POVH = np.float32(0.15)


@pytest.fixture(scope="module")
def ske(gpu_lib):
    import skewengine_gb300 as ske
    return ske


def _run(ske, op, x, **kw):
    dy, dx = x.shape
    with ske.SkewEngine(dx, dy) as eng:
        out = eng.run(op, np.ascontiguousarray(x, np.float32), povh=POVH, **kw)
        assert eng.launch_count() > 0
        return out


def test_golden_runs_bit_exact(ske, golden_runs):
    for key, op, x, want in run_cases(golden_runs):
        got = _run(ske, op, x)
        assert bits_equal(got, want), (key, float(np.abs(got - want).max()))


def test_golden_sectors_per_sector_api(ske, golden_sectors):
    """skew / kernel / deskew of single sectors reproduce the reference's
    intermediate buffers."""
    from tests.golden.make_golden import OPS
    cases = {}
    for k in golden_sectors.files:
        if k.endswith("__iinfo"):
            name, kind, shape, seed, a = k[: -len("__iinfo")].split("__")
            cases.setdefault((name, kind, shape, seed), []).append(int(a[1:]))
    for (name, kind, shape, seed), angles in sorted(cases.items()):
        base = "__".join([name, kind, shape, seed])
        x = golden_sectors[base + "__in"]
        dy, dx = x.shape
        with ske.SkewEngine(dx, dy) as eng:
            for a in sorted(angles):
                eng.prepare(x)
                eng.skew(a)
                eng.kernel(OPS[name], POVH)
                si, so = eng.skewed()
                assert bits_equal(si, golden_sectors[f"{base}__a{a}__skew_in"]), (base, a, "skew_in")
                assert bits_equal(so, golden_sectors[f"{base}__a{a}__skew_out"]), (base, a, "skew_out")
                eng.deskew(1 if OPS[name] == 4 else 0)
                acc = eng.reduce(1 if OPS[name] == 4 else 0)
                assert bits_equal(acc.ravel(), golden_sectors[f"{base}__a{a}__acc"]), (base, a, "acc")


def test_per_sector_after_batched_run(ske, oracle):
    """Batched runs leave the skew buffers' unused cells unwritten; the per-sector
    API on the same engine afterwards still sees the reference's buffers (zeros
    past the sector's rows, a cleared output)."""
    x = synthetic.fractal_dem(64, 13)
    with ske.SkewEngine(64, 64) as eng:
        full = eng.run(0, x, povh=POVH)
        assert bits_equal(full, oracle.run(0, x, povh=POVH))
        for a in (0, 20, 45, 90, 133):
            eng.prepare(x)
            eng.skew(a)
            eng.kernel(0, POVH)
            si, so = eng.skewed()
            want_si, want_so, _ = oracle.sector(0, x, a, povh=POVH)
            assert bits_equal(si, want_si) and bits_equal(so, want_so), a


@pytest.mark.parametrize("side,side_y,seed", [(96, 96, 1), (128, 80, 2), (80, 128, 3), (200, 200, 4),
                                              (257, 257, 5)])
def test_sdem_matches_oracle(ske, oracle, side, side_y, seed):
    x = synthetic.fractal_dem(side, seed, side_y=side_y)
    want = oracle.run(0, x, povh=POVH)
    got = _run(ske, 0, x)
    assert bits_equal(got, want)


def test_sdem_counts_bit_exact(ske, oracle):
    x = synthetic.fractal_dem(150, 9, side_y=130)
    with ske.SkewEngine(150, 130) as eng:
        eng.prepare(x)
        for a in (0, 1, 30, 44, 45, 46, 60, 89, 90, 91, 120, 134, 135, 150, 179):
            got = eng.sdem_counts(a, POVH)
            want = oracle.counts(x, a, povh=POVH)
            assert bits_equal(got, want), a


def test_sector_loop_equals_run(ske):
    """The per-sector drop-in API driven like main.cu:147-164 equals ske_run."""
    x = synthetic.fractal_dem(64, 21)
    with ske.SkewEngine(64, 64) as eng:
        whole = eng.run(0, x, povh=POVH)
        eng.prepare(x)
        for a in range(180):
            eng.skew(a)
            eng.kernel(0, POVH)
            eng.deskew(0)
        loop = eng.reduce(0)
    assert bits_equal(whole, loop)


@pytest.mark.parametrize("op", [1, 2, 3])
def test_identity_radon_match_oracle(ske, oracle, op):
    for side, side_y, seed in ((100, 100, 3), (96, 70, 4)):
        x = synthetic.ellipse_phantom(side, seed, side_y=side_y) if op == 2 else \
            synthetic.fractal_dem(side, seed, side_y=side_y)
        assert bits_equal(_run(ske, op, x), oracle.run(op, x, povh=POVH)), (op, side, side_y)


def test_radon_rows_within_width_non_square(ske, oracle):
    """Radon batches whose sectors' rows stay within their width are deskewed
    from the filtered row values (no back-projection into the skewed output);
    on a non-square grid only the plain (non-transposed) sectors qualify."""
    x = synthetic.ellipse_phantom(96, 12, side_y=70)
    plain = [a for a in range(180) if ske.geometry(96, 70, a)["sector_type"] in (0, 3)]
    plain = plain[:6] + plain[-6:]
    with ske.SkewEngine(96, 70) as eng:
        got = eng.run(2, np.ascontiguousarray(x), povh=POVH, angles=plain)
        kahan = eng.run(2, np.ascontiguousarray(x), povh=POVH, angles=plain, accum="kahan")
    want = oracle.run_angles(2, x, plain, povh=POVH)
    assert bits_equal(got, want)
    assert np.abs(kahan - want).max() <= 1e-5 * np.abs(want).max()


@pytest.mark.parametrize("case", ["wide", "nonfinite"])
def test_radon_special_values_bit_exact(ske, oracle, case):
    """Rows outside the exact integer row sums' conditions (exponent spread
    above 28 binades, magnitude sums at or above 2^53 units, subnormals,
    cancellation to zero) take the sequential binary64 sum; non-finite row sums
    take the transform's exact complex products.  Results equal the oracle's
    (NaNs compared as NaNs)."""
    x = synthetic.ellipse_phantom(64, 21).astype(np.float32)
    if case == "wide":
        x[5, :] = 1e30
        x[5, 1::2] = -1e30
        x[7, 3] = 1e-30
        x[9, :] = 1e-40
        x[12, :20] = 3.0e7
        x[12, 20:24] = 1e-3
        x[15, :] = np.where(np.arange(64) % 2, 1.5, -1.5)
        x[20:40, 50] = 6e-39
    else:
        x[11, 11] = np.inf
        x[30, 2] = np.nan
        x[40, 40] = -np.inf
    got = _run(ske, 2, x)
    want = oracle.run(2, x, povh=POVH)
    same = (got.view(np.uint32) == want.view(np.uint32)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), (case, int((~same).sum()))


def test_radon_long_rows_and_large_transforms(ske, oracle):
    """Rows over 2048 cells take the sequential binary64 row sum; sectors with
    H2 > 8192 transform in global memory instead of shared memory."""
    x = synthetic.ellipse_phantom(2100, 17, side_y=24)
    assert bits_equal(_run(ske, 2, x), oracle.run(2, x, povh=POVH))
    x = synthetic.ellipse_phantom(8300, 18, side_y=4)
    angles = [0, 30, 88, 89, 90, 91, 135]
    assert max(ske.geometry(8300, 4, a)["skew_height"] for a in angles) > 8192
    with ske.SkewEngine(8300, 4) as eng:
        got = eng.run(2, np.ascontiguousarray(x), povh=POVH, angles=angles)
    assert bits_equal(got, oracle.run_angles(2, x, angles, povh=POVH))


@pytest.mark.parametrize("op,accum", [(0, "reference"), (0, "kahan"), (2, "reference"), (4, "reference")])
def test_checkpoint_resume_bit_exact(ske, op, accum, tmp_path):
    """A run interrupted after two chunks of 40 sectors and resumed from its
    checkpoint file gives the bits of an uninterrupted run."""
    if op == 4:
        x = synthetic.blurred_texture(40, 3)[0]
    elif op == 2:
        x = synthetic.ellipse_phantom(40, 3)
    else:
        x = synthetic.fractal_dem(40, 9)
    x = np.ascontiguousarray(x, np.float32)
    path = str(tmp_path / "run.npz")
    with ske.SkewEngine(40, 40) as eng:
        full = eng.run(op, x, povh=POVH, accum=accum)
        assert eng.run_checkpointed(op, x, path, chunk=40, povh=POVH, accum=accum, stop_after=2) is None
        got = eng.run_checkpointed(op, x, path, chunk=40, povh=POVH, accum=accum)
        assert bits_equal(got, full)
        other = 1 if op != 1 else 0
        with pytest.raises(ValueError):
            eng.run_checkpointed(other, x, path, chunk=40, povh=POVH, accum=accum)


def test_allocation_failures_are_clean(ske, oracle):
    """Every device or pinned allocation of engine creation and of a run is made
    to fail in turn (host-side injection): each call returns an error, the
    engine can be destroyed, no device memory is left behind, and once the
    failure point lies past the last allocation the run is bit-exact."""
    import torch
    from skewengine_gb300 import SkeError
    lib = ske.engine.load()
    x = synthetic.fractal_dem(300, 4)
    want = oracle.run(0, x, povh=POVH)
    with ske.SkewEngine(300, 300) as eng:  # device tables and context set up once
        eng.run(0, x, povh=POVH)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failures = 0
    try:
        for k in range(200):
            lib.ske_inject_alloc_failure(k)
            eng = None
            try:
                eng = ske.SkewEngine(300, 300)
                got = eng.run(0, x, povh=POVH)
            except SkeError as exc:
                assert "injected" in str(exc)
                failures += 1
                continue
            finally:
                lib.ske_inject_alloc_failure(-1)
                if eng is not None:
                    eng.close()
            assert bits_equal(got, want)
            break
        else:
            raise AssertionError("the run never got past the injected failures")
    finally:
        lib.ske_inject_alloc_failure(-1)
    assert failures >= 10, failures
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0 - (4 << 20), "device memory leaked"


def test_radon_512_matches_oracle(ske, oracle):
    x = synthetic.ellipse_phantom(512, 7)
    assert bits_equal(_run(ske, 2, x), oracle.run(2, x, povh=POVH))


def test_cepstrum_bins_match_oracle(ske, oracle):
    x, _, _ = synthetic.blurred_texture(72, 11)
    got = _run(ske, 4, x)
    want = oracle.run(4, x, povh=POVH)
    mismatch = np.mean(got != want)
    assert np.all(got == np.round(got)) and np.all(want == np.round(want))
    assert mismatch == 0.0, f"bin mismatch rate {mismatch}"


def test_subset_of_angles(ske, oracle):
    x = synthetic.fractal_dem(90, 31)
    angles = [5, 44, 45, 46, 90, 91, 135, 170]
    with ske.SkewEngine(90, 90) as eng:
        got = eng.run(0, x, povh=POVH, angles=angles)
    assert bits_equal(got, oracle.run_angles(0, x, angles, povh=POVH))


def test_kahan_accumulation_close(ske, oracle):
    x = synthetic.fractal_dem(160, 12)
    got = _run(ske, 0, x, accum="kahan")
    want = oracle.run(0, x, povh=POVH).astype(np.float64)
    rel = np.abs(got - want) / np.maximum(np.abs(want), 1.0)
    assert rel.max() <= 1e-5
    assert abs(got.astype(np.float64).sum() - want.sum()) / want.sum() <= 1e-6


def test_device_pointers(ske, oracle):
    torch = pytest.importorskip("torch")
    x = synthetic.fractal_dem(64, 41)
    xd = torch.from_numpy(x).cuda()
    with ske.SkewEngine(64, 64) as eng:
        out = eng.run(0, xd, povh=POVH)
    assert out.is_cuda
    assert bits_equal(out.cpu().numpy(), oracle.run(0, x, povh=POVH))


@pytest.mark.parametrize("dims", [(1, 1), (2, 1), (1, 7), (7, 1), (3, 2), (5, 17), (17, 5)])
def test_tiny_and_degenerate_grids(ske, oracle, dims):
    dx, dy = dims
    x = (np.random.default_rng(dx * 31 + dy).random((dy, dx)) * 100).astype(np.float32)
    for op in (0, 1, 2):
        assert bits_equal(_run(ske, op, x), oracle.run(op, x, povh=POVH)), (dims, op)


@pytest.mark.parametrize("dx", [4032, 4040])
def test_long_rows_at_fast_path_limit(ske, oracle, dx):
    """Rows of 4032 cells are the longest the sweep's fast path takes; 4040-cell
    rows take the reference-order path.  Both match the oracle bit for bit.
    (Angle 0 only: the transposed sectors of so flat a grid have rows that
    overrun the 3-cell width up to dim_l, about 6.6e10 steps for the oracle.)"""
    x = synthetic.fractal_dem(dx, 21, side_y=3)
    angles = [0]
    with ske.SkewEngine(dx, 3) as eng:
        got = eng.run(0, np.ascontiguousarray(x), povh=POVH, angles=angles)
    assert bits_equal(got, oracle.run_angles(0, x, angles, povh=POVH)), dx


def test_special_values_take_exact_path(ske, oracle):
    """Rows with zeros, huge or non-finite heights use IEEE division and the
    reference's accumulation order; results still match the oracle."""
    x = synthetic.fractal_dem(48, 51)
    x[3, :] = 0.0
    x[10, 10] = 3e30
    x[20, 5] = -1e-30
    x[30, 30] = np.inf
    x[40, 7] = np.nan
    got = _run(ske, 0, x)
    want = oracle.run(0, x, povh=POVH)
    same = (got.view(np.uint32) == want.view(np.uint32)) | (np.isnan(got) & np.isnan(want))
    assert same.all()


def test_constant_and_zero_dem(ske, oracle):
    for v in (0.0, 7.5):
        x = np.full((33, 33), v, np.float32)
        assert bits_equal(_run(ske, 0, x), oracle.run(0, x, povh=POVH)), v


def test_custom_operator_receives_sector(ske):
    """A custom device operator gets the current sector's geometry and buffers;
    a failing operator is reported as an error."""
    seen = {}

    def op(view):
        seen["h"] = view.geom.skew_height
        seen["ptrs"] = (view.skew_in, view.skew_out, view.first)
        return 0

    x = synthetic.fractal_dem(32, 1)
    with ske.SkewEngine(32, 32) as eng:
        eng.prepare(x)
        eng.skew(30)
        eng.kernel_custom(op)
        assert seen["h"] == ske.geometry(32, 32, 30)["skew_height"]
        assert all(seen["ptrs"])
        with pytest.raises(ske.SkeError):
            eng.kernel_custom(lambda v: 7)


def test_state_errors(ske):
    with ske.SkewEngine(16, 16) as eng:
        with pytest.raises(ske.SkeError):
            eng.skew(3)  # before prepare
        eng.prepare(np.zeros((16, 16), np.float32))
        with pytest.raises(ske.SkeError):
            eng.kernel(0)  # before skew
        with pytest.raises(ske.SkeError):
            eng.run(9, np.zeros((16, 16), np.float32))


def test_division_exhaustive(gpu_lib):
    """The sweep's multiply-and-correct division equals IEEE division for every
    float numerator of the fast-path range and every d in [1, 4095]."""
    checked, bad, first = C.c_int64(), C.c_int64(), C.c_uint32()
    assert gpu_lib.ske_selftest_division(0, 4095, C.byref(checked), C.byref(bad), C.byref(first)) == 0
    assert checked.value > 1.3e13
    assert bad.value == 0, f"first mismatching numerator bits {first.value:#010x}"


def test_accumulate_and_fold(ske, oracle):
    from skewengine_gb300.parallel import fold_accumulators
    x = synthetic.fractal_dem(60, 61)
    with ske.SkewEngine(60, 60) as eng:
        a0, u0 = eng.accumulate(0, x, list(range(0, 90)), povh=POVH)
        a1, u1 = eng.accumulate(0, x, list(range(90, 180)), povh=POVH)
    o0, v0 = oracle.accumulate(0, x, list(range(0, 90)), povh=POVH)
    assert bits_equal(a0, o0) and u0 == v0
    got = fold_accumulators([a0, a1], [u0, u1], 60, 60)
    np.testing.assert_allclose(got, oracle.run(0, x, povh=POVH), rtol=1e-5)


def test_run_batch_uneven(ske, oracle):
    grids = [synthetic.fractal_dem(s, 70 + i, roughness=h) for i, (s, h) in
             enumerate([(64, 0.6), (80, 0.9), (40, 0.7), (64, 0.8)])]
    outs = ske.run_batch(0, grids, povh=POVH)
    for g, o in zip(grids, outs):
        assert bits_equal(o, oracle.run(0, g, povh=POVH))


def test_radon_fused_sector_kernel_bit_exact(ske, oracle, gpu_lib):
    """The thread-block-cluster Radon kernel (row sums into the leader CTA's
    shared memory, then the filtered transform) gives the same bits as the
    two-launch path and the oracle, including rows with non-finite values."""
    try:
        assert gpu_lib.ske_radon_select(0) == 0
        for x in (synthetic.ellipse_phantom(512, 2024), synthetic.ellipse_phantom(96, 5, side_y=70)):
            assert bits_equal(_run(ske, 2, x), oracle.run(2, x, povh=POVH))
        x = synthetic.ellipse_phantom(64, 9)
        x[3, 5] = np.inf
        x[40, 7] = np.nan
        fused = _run(ske, 2, x)
        assert gpu_lib.ske_radon_select(1) == 0
        two = _run(ske, 2, x)
        assert bits_equal(fused, two)  # both on the GPU: the same NaN encodings too
        want = oracle.run(2, x, povh=POVH)  # host NaNs may be encoded differently
        assert ((fused.view(np.uint32) == want.view(np.uint32)) | (np.isnan(fused) & np.isnan(want))).all()
    finally:
        gpu_lib.ske_radon_select(1)


@pytest.mark.parametrize("side,side_y", [(640, 480), (1024, 160), (200, 200)])
def test_staged_skew_matches_oracle(ske, oracle, side, side_y):
    """The TMA-staged skew (ske_skew_select(1); sides multiples of 4, >= 129).
    On 1024 x 160 the columns of a 32-wide block shift by more than 64 rows at
    angles 9-25 and 155-171 (those blocks read global memory directly); the
    other angles stage their rows.  Output bit for bit against the oracle, and
    the skewed input of every sector equal to the gather kernel's."""
    x = synthetic.fractal_dem(side, 17, side_y=side_y)
    angles = [0, 5, 9, 12, 20, 33, 45, 80, 90, 100, 135, 160, 170, 179]
    lib = ske.engine.load()
    try:
        assert lib.ske_skew_select(1) == 0
        with ske.SkewEngine(side, side_y) as eng:
            got = eng.run(0, x, povh=synthetic.POVH, angles=angles)
            eng.prepare(x)
            staged = []
            for a in angles:
                eng.skew(a)
                staged.append(eng.skewed()[0])
        assert lib.ske_skew_select(0) == 0
        with ske.SkewEngine(side, side_y) as eng:
            eng.prepare(x)
            for a, si in zip(angles, staged):
                eng.skew(a)
                assert bits_equal(si, eng.skewed()[0]), a
    finally:
        lib.ske_skew_select(0)
    want = oracle.run_ordered(0, x, angles, povh=synthetic.POVH)
    assert bits_equal(got, want)


# Stated float32 Radon bound: max |float32 - binary64| over max |binary64|.
RADON_F32_MAX_REL = 1e-5  # measured: 1.2e-6 at 512 x 512, 3-5e-7 on the small grids


@pytest.mark.parametrize("side,side_y,angles", [(512, 512, list(range(0, 180, 10)) + [45, 90, 135]),
                                                 (128, 80, None), (97, 131, [0, 20, 45, 60, 90, 150])])
def test_radon_float32_mode_error(ske, oracle, side, side_y, angles):
    """SKE_FLAG_RADON_F32 against the binary64 operator (itself bit-equal to the
    oracle): square grids take the gathered-sums path, the non-square ones the
    back-projection path.  The error relative to the output's magnitude is
    printed and bounded by RADON_F32_MAX_REL."""
    x = np.ascontiguousarray(synthetic.ellipse_phantom(side, 31, side_y=side_y), np.float32)
    with ske.SkewEngine(side, side_y) as eng:
        exact = eng.run(ske.KERNEL_RADON, x, povh=POVH, angles=angles)
        fast = eng.run(ske.KERNEL_RADON, x, povh=POVH, angles=angles, flags=ske.FLAG_RADON_F32)
    op = ske.KERNEL_RADON
    want = oracle.run_ordered(op, x, angles, povh=POVH) if angles else oracle.run_ordered(op, x, povh=POVH)
    assert bits_equal(exact, want)
    err = float(np.abs(fast.astype(np.float64) - exact).max() / max(np.abs(exact).max(), 1e-30))
    print(f"float32 Radon {side}x{side_y}: max error {err:.1e} of the output's magnitude")
    assert err <= RADON_F32_MAX_REL, err
