"""Float32 cepstrum mode (SKE_FLAG_CEPSTRUM_F32): fused sector loop on the FP32
pipes for batches of square images.

The reference computes the cepstrum in binary64 (src/kernelBLUR.h:153-228) and
the engine's default operator reproduces it bit for bit (test_config_parity.py).
This mode rounds differently, so an output can fall in another 1000-wide bin
(the max+angle encoding of src/skewEngine.cuh:774-785) where a value sits at a
bin edge.  The rate of outputs that differ from the oracle is stated here and
bounded by MAX_MISMATCH on the benchmark's 512 x 512 motion-blurred textures.
"""
from __future__ import annotations

import numpy as np
import pytest

from skewengine_gb300 import synthetic
from tests.conftest import bits_equal

pytestmark = pytest.mark.gpu

POVH = synthetic.POVH
MAX_MISMATCH = 1e-3  # fraction of output cells whose value differs from the binary64 reference


@pytest.fixture(scope="module")
def ske(gpu_lib):
    import skewengine_gb300 as ske
    return ske


def _f32(ske, x, angles=None):
    with ske.SkewEngine(x.shape[1], x.shape[0]) as eng:
        return eng.run(4, x, povh=POVH, angles=angles, flags=ske.FLAG_CEPSTRUM_F32)


def test_f32_cepstrum_mismatch_rate_512(ske, oracle):
    rates = []
    for seed in (2024, 2026):
        x, _, _ = synthetic.blurred_texture(512, seed)
        got = _f32(ske, x)
        want = oracle.run_ordered(4, x, povh=POVH)
        assert np.all(got == np.round(got))
        diff = got != want
        rate = float(diff.mean())
        # Where they differ the peak search (kernelBLUR.h:88-110) can pick
        # another peak (its first-ascent index moves), so bins may differ by more
        # than one; the rate of differing cells is the stated figure.
        spread = np.abs(np.floor(got[diff] / 1000) - np.floor(want[diff] / 1000))
        rates.append(rate)
        print(f"float32 cepstrum seed {seed}: {int(diff.sum())} of {diff.size} cells differ (rate {rate:.2e}), "
              f"bin difference max {spread.max() if spread.size else 0:.0f}, "
              f"median {np.median(spread) if spread.size else 0:.0f}")
    assert max(rates) <= MAX_MISMATCH, rates


def test_f32_cepstrum_small_grids_and_angle_lists(ske, oracle):
    for side, angles in ((64, None), (97, [0, 44, 45, 46, 90, 135, 179]), (33, list(range(0, 180, 7)))):
        x, _, _ = synthetic.blurred_texture(side, side)
        got = _f32(ske, x, angles)
        want = oracle.run_ordered(4, x, angles, povh=POVH) if angles else oracle.run_ordered(4, x, povh=POVH)
        assert float((got != want).mean()) <= 0.01, side


def test_f32_cepstrum_batch_equals_single_runs(ske, oracle):
    """A batch of equal-size images (one launch sequence) gives each image's
    single-run result; a non-square image in the batch takes the exact path."""
    imgs = [synthetic.blurred_texture(80, 40 + i)[0] for i in range(3)]
    odd, _, _ = synthetic.blurred_texture(48, 7, side_y=30)
    batch = imgs[:2] + [odd] + imgs[2:]
    outs = ske.run_batch(4, batch, povh=POVH, flags=ske.FLAG_CEPSTRUM_F32)
    for img, out in zip(batch, outs):
        if img.shape[0] == img.shape[1]:
            assert bits_equal(out, _f32(ske, img))
        else:
            assert bits_equal(out, oracle.run_ordered(4, img, povh=POVH))
