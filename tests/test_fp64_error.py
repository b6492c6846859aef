"""Error of the float pipeline against a binary64 restatement of the same
sector loop (oracle port_run_f64): the stated accuracy of the Radon transform
(filtered back-projection) and of the cepstrum, whose float results are only
defined up to rounding.

Stated bounds (max over the grid, relative to the largest |FP64 value|):
  Radon / FBP   max |err| <= 2e-6, RMS err <= 5e-7
  identity      max |err| <= 2e-6
  cepstrum      the output bins floor(v / 1000) agree on >= 99.9% of cells and
                the encoded angle differs by at most 180 where they agree.
The CPU tests hold the float oracle to these bounds; the GPU tests hold the
sm_103a kernels to the same ones.
"""
from __future__ import annotations

import numpy as np
import pytest

from skewengine_gb300 import synthetic

POVH = np.float32(0.15)
RADON_MAX, RADON_RMS, IDENT_MAX = 2e-6, 5e-7, 2e-6


def _cases():
    return [
        (2, synthetic.ellipse_phantom(128, 3)),
        (2, synthetic.ellipse_phantom(96, 4, side_y=70)),
        (1, synthetic.fractal_dem(96, 2)),
        (3, synthetic.fractal_dem(80, 5, side_y=64)),
    ]


def _check_linear(op, got, ref):
    d = got.astype(np.float64) - ref
    scale = np.abs(ref).max()
    rel_max = np.abs(d).max() / scale
    rel_rms = np.sqrt(np.mean(d * d)) / scale
    if op == 2:
        assert rel_max <= RADON_MAX and rel_rms <= RADON_RMS, (rel_max, rel_rms)
    else:
        assert rel_max <= IDENT_MAX, rel_max


def _check_cepstrum(got, ref):
    gb, rb = np.floor(got / 1000.0), np.floor(ref / 1000.0)
    agree = gb == rb
    assert agree.mean() >= 0.999, agree.mean()
    assert np.abs(got[agree] - ref[agree]).max() <= 180


@pytest.fixture(scope="module")
def f64_refs(oracle):
    refs = [(op, x, oracle.run_f64(op, x, povh=POVH)) for op, x in _cases()]
    xc, _, _ = synthetic.blurred_texture(64, 5)
    refs.append((4, xc, oracle.run_f64(4, xc, povh=POVH)))
    return refs


def test_oracle_within_stated_error(oracle, f64_refs):
    for op, x, ref in f64_refs:
        got = oracle.run(op, x, povh=POVH)
        if op == 4:
            _check_cepstrum(got, ref)
        else:
            _check_linear(op, got, ref)


def test_f64_identity_is_exact_for_zero_drift(oracle):
    """Sanity of the restatement: a 1x1 grid has no drift and no neighbours."""
    x = np.full((1, 1), 3.5, np.float32)
    assert oracle.run_f64(3, x, povh=POVH)[0, 0] == pytest.approx(3.5 * 180)


@pytest.mark.gpu
def test_gpu_within_stated_error(gpu_lib, f64_refs):
    import skewengine_gb300 as ske
    for op, x, ref in f64_refs:
        dy, dx = x.shape
        with ske.SkewEngine(dx, dy) as eng:
            got = eng.run(op, np.ascontiguousarray(x, np.float32), povh=POVH)
        if op == 4:
            _check_cepstrum(got, ref)
        else:
            _check_linear(op, got, ref)
