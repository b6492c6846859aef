"""GPU parity at the benchmark workloads' own sizes, against the oracle.

The small-grid parity tests pin every code path; these pin the sizes the
benchmarks run, where row lengths, level counts, batch capacities and work
lists differ from the small cases:

* total viewshed of the seeded 500 x 500 fractal DEM (roughness 0.8, 0-1500 m,
  10 m cells, observer 1.5 m), all 180 angles (360 directional sectors);
* the 2000 x 2000 headline DEM on an angle subset spanning all four sector
  types and their boundaries, output and integer visibility counts;
* the cepstrum of a 512 x 512 motion-blurred 1/f^2 texture, all 180 angles;
* the local Radon transform of the same texture on an angle subset;
* a batch of six uneven fractal DEMs with sides 256-2000 in compensated (Kahan)
  accumulation, relative error at most 1e-5 per cell against the reference
  order.

The oracle runs its sectors on all host cores and folds them in angle order
(port_run_angles_ordered), which reproduces the reference's single-thread
accumulation bit for bit (checked on the CPU in test_oracle_golden.py).
Reference: src/kernelSDEM.h:168-222, src/kernelBLUR.h:153-228,
src/kernelRADN.h:114-182, src/skewEngine.cuh:756-833.
"""
from __future__ import annotations

import numpy as np
import pytest

from skewengine_gb300 import synthetic
from tests.conftest import bits_equal

pytestmark = pytest.mark.gpu

POVH = synthetic.POVH
# Sector types 0..3 and the angles next to their boundaries (45 and 135 for a
# square grid, 90 between the transposed halves), plus mid-range angles.
HEADLINE_ANGLES = [0, 1, 17, 44, 45, 46, 63, 89, 90, 91, 112, 135, 158, 179]


@pytest.fixture(scope="module")
def ske(gpu_lib):
    import skewengine_gb300 as ske
    return ske


def test_config1_sdem_500_all_angles(ske, oracle):
    x = synthetic.fractal_dem(500, 1000, roughness=0.8)
    with ske.SkewEngine(500, 500) as eng:
        got = eng.run(0, x, povh=POVH)
    want = oracle.run_ordered(0, x, povh=POVH)
    assert bits_equal(got, want)


def test_headline_sdem_2000_angle_subset(ske, oracle):
    x = synthetic.fractal_dem(2000, 1000, roughness=0.8)
    with ske.SkewEngine(2000, 2000) as eng:
        got = eng.run(0, x, povh=POVH, angles=HEADLINE_ANGLES)
        eng.prepare(x)
        counts = [eng.sdem_counts(a, povh=POVH) for a in HEADLINE_ANGLES]
    want = oracle.run_ordered(0, x, HEADLINE_ANGLES, povh=POVH)
    assert bits_equal(got, want)
    for a, c, w in zip(HEADLINE_ANGLES, counts, oracle.counts_many(x, HEADLINE_ANGLES, povh=POVH)):
        assert bits_equal(c, w), f"visibility counts differ at angle {a}"


def test_config4_cepstrum_512_all_angles(ske, oracle):
    x, _, _ = synthetic.blurred_texture(512, 2024)
    with ske.SkewEngine(512, 512) as eng:
        got = eng.run(4, x, povh=POVH)
    want = oracle.run_ordered(4, x, povh=POVH)
    mismatch = int(np.count_nonzero(got != want))
    assert mismatch == 0, f"{mismatch} of {got.size} cells differ"
    assert bits_equal(got, want)


def test_local_radon_512_angle_subset(ske, oracle):
    x, _, _ = synthetic.blurred_texture(512, 2025)
    angles = list(range(0, 180, 8)) + [45, 90, 135]
    with ske.SkewEngine(512, 512) as eng:
        got = eng.run(5, x, povh=POVH, angles=angles)
    want = oracle.run_ordered(5, x, angles, povh=POVH)
    assert bits_equal(got, want)


def test_config3_uneven_batch_kahan(ske, oracle):
    """Six DEMs of the uneven-batch workload's generator (sides 256..2000,
    roughness 0.6-0.9) in one batched call, Kahan mode, 9 angles each."""
    sides = [(256, 0.6), (611, 0.9), (1024, 0.7), (1357, 0.85), (1789, 0.65), (2000, 0.75)]
    grids = [synthetic.fractal_dem(s, 3100 + i, roughness=h) for i, (s, h) in enumerate(sides)]
    angles = list(range(0, 180, 20))
    outs = ske.run_batch(0, grids, povh=POVH, accum="kahan", angles=angles)
    for g, got in zip(grids, outs):
        want = oracle.run_ordered(0, g, angles, povh=POVH).astype(np.float64)
        rel = np.abs(got.astype(np.float64) - want) / np.maximum(np.abs(want), 1.0)
        assert rel.max() <= 1e-5, (g.shape, float(rel.max()))
        assert abs(got.astype(np.float64).sum() - want.sum()) / want.sum() <= 1e-6
