"""Batched total viewshed over grids of uneven size (ske_run_batch_angles).

Square grids run together: per wave one launch each for the orientations, the
skew, the sweep, the deskew and the fold of every grid and sector, replayed as
a CUDA graph from the second call.  Other grids take the per-grid path.  Every
result must equal the single-grid run bit for bit, in reference order against
the oracle (the reference's single-thread loop, src/main.cu:86-168).
"""
from __future__ import annotations

import numpy as np
import pytest

from skewengine_gb300 import synthetic
from tests.conftest import bits_equal

pytestmark = pytest.mark.gpu

POVH = synthetic.POVH


@pytest.fixture(scope="module")
def ske(gpu_lib):
    import skewengine_gb300 as ske
    return ske


def _grids(spec, base=500):
    return [synthetic.fractal_dem(s, base + i, roughness=h, side_y=sy)
            for i, (s, sy, h) in enumerate(spec)]


def test_batch_reference_order_bit_exact_and_graph_replay(ske, oracle):
    """Uneven square grids (a size repeated), all angles, reference order: each
    output equals the oracle bit for bit, on the first call (plain launches and
    the autotuner) and on two graph replays."""
    spec = [(96, 96, 0.6), (33, 33, 0.9), (150, 150, 0.7), (96, 96, 0.8), (7, 7, 0.75), (121, 121, 0.65)]
    grids = _grids(spec)
    want = [oracle.run_ordered(0, g, povh=POVH) for g in grids]
    with ske.SkewEngine(150, 150) as eng:
        for call in range(3):
            n0 = eng.launch_count()
            outs = ske.run_batch(0, grids, povh=POVH, engine=eng)
            for g, o, w in zip(grids, outs, want):
                assert bits_equal(o, w), (call, g.shape)
            if call > 0:
                assert eng.launch_count() - n0 == 5, "one wave: five launches per call"


def test_batch_device_buffers_angle_list_and_flags(ske, oracle):
    torch = pytest.importorskip("torch")
    spec = [(64, 64, 0.6), (100, 100, 0.8), (45, 45, 0.7)]
    grids = _grids(spec, 600)
    angles = [179, 3, 45, 90, 91, 135, 20]  # any order: accumulated in list order
    want = [oracle.run_ordered(0, g, angles, povh=POVH) for g in grids]
    dev = [torch.from_numpy(g).cuda() for g in grids]
    for flags in (0, ske.FLAG_NO_TUNE | ske.FLAG_NO_GRAPH, ske.FLAG_NO_GRAPH):
        outs = ske.run_batch(0, dev, povh=POVH, angles=angles, flags=flags)
        for o, w in zip(outs, want):
            assert o.is_cuda and bits_equal(o.cpu().numpy(), w), flags


def test_batch_kahan_matches_single_grid_runs(ske, oracle):
    spec = [(80, 80, 0.6), (130, 130, 0.85), (57, 57, 0.7)]
    grids = _grids(spec, 700)
    outs = ske.run_batch(0, grids, povh=POVH, accum="kahan")
    for g, o in zip(grids, outs):
        with ske.SkewEngine(g.shape[1], g.shape[0]) as eng:
            single = eng.run(0, g, povh=POVH, accum="kahan")
        assert bits_equal(o, single)
        want = oracle.run_ordered(0, g, povh=POVH).astype(np.float64)
        assert (np.abs(o - want) / np.maximum(np.abs(want), 1.0)).max() <= 1e-5


def test_batch_mixed_with_non_square_grids(ske, oracle):
    """Non-square grids (some sectors' rows leave their width) run through the
    per-grid path inside the same call; the square ones still batch."""
    spec = [(90, 90, 0.6), (70, 40, 0.8), (60, 60, 0.7), (31, 77, 0.9)]
    grids = _grids(spec, 800)
    outs = ske.run_batch(0, grids, povh=POVH)
    for g, o in zip(grids, outs):
        assert bits_equal(o, oracle.run_ordered(0, g, povh=POVH)), g.shape


def test_batch_shape_change_rebuilds_plan(ske, oracle):
    with ske.SkewEngine(80, 80) as eng:
        a = _grids([(50, 50, 0.6), (80, 80, 0.7)], 900)
        b = _grids([(80, 80, 0.7), (66, 66, 0.8), (12, 12, 0.6)], 910)
        for grids in (a, b, a):
            outs = ske.run_batch(0, grids, povh=POVH, engine=eng)
            for g, o in zip(grids, outs):
                assert bits_equal(o, oracle.run_ordered(0, g, povh=POVH))
        lvl0, lvl1, ctas = eng.sweep_shape()
        assert lvl0 in (16, 32, 64) and lvl1 in (0, 32, 48) and ctas >= 0


def test_autotuned_single_grid_run_is_unchanged(ske, oracle):
    """The autotuner picks a sweep shape on the first large run; every shape
    gives the same bits as the built-in one."""
    x = synthetic.fractal_dem(300, 1234)
    with ske.SkewEngine(300, 300) as eng:
        tuned = eng.run(0, x, povh=POVH)
        fixed = eng.run(0, x, povh=POVH, flags=ske.FLAG_NO_TUNE)
        assert eng.sweep_shape() == (64, 0, 0)
    assert bits_equal(tuned, fixed)
    assert bits_equal(tuned, oracle.run_ordered(0, x, povh=POVH))


def test_batch_stacked_grids_equal_list(ske, oracle):
    """A (N, H, W) stack runs as N grids with computed pointer tables, device and
    host, with the same bits as the list form."""
    torch = pytest.importorskip("torch")
    stack = np.stack([synthetic.fractal_dem(48, 950 + i) for i in range(5)]).astype(np.float32)
    with ske.SkewEngine(48, 48) as eng:
        host = ske.run_batch(0, stack, povh=POVH, engine=eng)
        dev = ske.run_batch(0, torch.from_numpy(stack).cuda(), povh=POVH, engine=eng)
        lst = ske.run_batch(0, [g for g in stack], povh=POVH, engine=eng)
    for i in range(5):
        want = oracle.run_ordered(0, stack[i], povh=POVH)
        assert bits_equal(host[i], want) and bits_equal(dev[i].cpu().numpy(), want) and bits_equal(lst[i], want)


def test_device_inputs_written_late_on_torch_stream(ske, oracle):
    """An engine on its own stream, given CUDA tensors that torch's stream is
    still writing: torch's stream spins on the GPU, then copies the input in.
    The engine's work waits for the copy (first call and graph replays alike)
    instead of reading the buffer early."""
    import torch
    grids = np.stack([synthetic.fractal_dem(64, 700 + i) for i in range(6)])
    want = [oracle.run(0, g, povh=synthetic.POVH) for g in grids]
    src = torch.as_tensor(grids, device="cuda")
    eng = ske.SkewEngine(64, 64)  # its own non-blocking stream
    try:
        for rep in range(4):
            dst = torch.full_like(src, float("nan"))
            torch.cuda._sleep(20_000_000)  # about 10 ms of GPU time queued before the copy
            dst.copy_(src)
            out = ske.run_batch(0, dst, engine=eng)
            single = torch.full_like(src[0], float("nan"))
            torch.cuda._sleep(20_000_000)
            single.copy_(src[rep])
            one = eng.run(0, single)
            torch.cuda.synchronize()
            for g in range(len(grids)):
                assert bits_equal(out[g].cpu().numpy(), want[g]), (rep, g)
            assert bits_equal(one.cpu().numpy(), want[rep]), rep
    finally:
        eng.close()
