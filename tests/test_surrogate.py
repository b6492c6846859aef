"""The learned total-viewshed surrogate: its convolution kernels against a float64
NumPy convolution (forward, data and weight gradients), training, and the
engine-checked tiled inference with fallback."""
from __future__ import annotations

import contextlib

import numpy as np
import pytest

from skewengine_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _conv_ref(x, w, b, relu):
    """NumPy conv3x3 (NHWC, zero padding) in float64; w: (Cout, 9*Cin)."""
    n, h, wd, cin = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    cols = np.stack([xp[:, ky:ky + h, kx:kx + wd, :] for ky in range(3) for kx in range(3)], axis=3)
    cols = cols.reshape(n, h, wd, 9 * cin)
    pre = cols @ w.T + (b if b is not None else 0.0)
    return (np.maximum(pre, 0.0) if relu else pre), pre, cols


def _bf16(a):
    import torch
    return torch.as_tensor(a, dtype=torch.float32).to(torch.bfloat16)


@pytest.fixture(scope="module")
def sur():
    from skewengine_gb300 import build
    build.build()
    from skewengine_gb300 import surrogate
    return surrogate


@pytest.mark.parametrize("n,h,w,cin,cout,relu", [(2, 19, 23, 8, 32, True), (1, 37, 5, 32, 64, False),
                                                  (3, 16, 16, 96, 72, True), (1, 130, 3, 64, 8, True),
                                                  (1, 24, 20, 64, 256, True), (2, 9, 11, 16, 130, False)])
def test_conv_forward_matches_numpy(sur, n, h, w, cin, cout, relu):
    import torch
    rng = np.random.default_rng(cin * 7 + cout)
    xb = _bf16(rng.normal(0, 1, (n, h, w, cin)))
    wb = _bf16(rng.normal(0, 0.2, (cout, 9 * cin)))
    b = torch.as_tensor(rng.normal(0, 0.5, cout), dtype=torch.float32)
    wpad = torch.zeros((cout, sur.kpad(cin)), dtype=torch.bfloat16)
    wpad[:, : 9 * cin] = wb
    y = sur.conv3x3(xb.cuda().contiguous(), wpad.cuda(), b.cuda(), relu)
    sur.conv_check()  # no tensor-core wait ran out
    y = y.float().cpu().numpy()
    ref, _, _ = _conv_ref(xb.double().numpy(), wb.double().numpy(), b.double().numpy(), relu)
    # float32 accumulation of exact bfloat16 products, then one bfloat16 rounding
    assert np.all(np.abs(y - ref) <= 2 ** -7 * np.abs(ref) + 1e-3), np.abs(y - ref).max()


def test_upcat_conv_equals_conv_of_the_concatenation(sur):
    """The fused upsample + concatenate convolution gives the bits of the
    convolution of the materialised concatenation."""
    import torch
    import torch.nn.functional as F
    rng = np.random.default_rng(3)
    low = _bf16(rng.normal(0, 1, (2, 9, 13, 64))).cuda().contiguous()
    skip = _bf16(rng.normal(0, 1, (2, 18, 26, 32))).cuda().contiguous()
    w = torch.zeros((48, sur.kpad(96)), dtype=torch.bfloat16)
    w[:, : 9 * 96] = _bf16(rng.normal(0, 0.1, (48, 9 * 96)))
    w = w.cuda()
    b = torch.as_tensor(rng.normal(0, 0.5, 48), dtype=torch.float32).cuda()
    up = F.interpolate(low.permute(0, 3, 1, 2), scale_factor=2, mode="nearest").permute(0, 2, 3, 1)
    want = sur.conv3x3(torch.cat([up, skip], 3).contiguous(), w, b, True)
    got = sur.conv3x3_upcat(low, skip, w, b, True)
    assert torch.equal(got.view(torch.int16), want.view(torch.int16))


def test_conv_rejects_misaligned_tensors(sur):
    """16-byte copies need 16-byte aligned inputs: a view starting 2 bytes into a
    buffer is refused before anything is launched."""
    import torch
    from skewengine_gb300 import SkeError
    buf = torch.zeros(8 * 8 * 8 + 8, dtype=torch.bfloat16, device="cuda")
    x = buf[1:1 + 8 * 8 * 8].view(1, 8, 8, 8)
    w = torch.zeros((16, sur.kpad(8)), dtype=torch.bfloat16, device="cuda")
    with pytest.raises(SkeError):
        sur.conv3x3(x, w)


def test_conv_gradients_match_numpy(sur):
    """d(sum(g * y))/dx, /dw, /db through the autograd function against NumPy."""
    import torch
    rng = np.random.default_rng(5)
    n, h, w, cin, cout = 2, 21, 18, 32, 64
    xb = _bf16(rng.normal(0, 1, (n, h, w, cin)))
    w32 = torch.zeros((cout, sur.kpad(cin)))
    w32[:, : 9 * cin] = torch.as_tensor(rng.normal(0, 0.1, (cout, 9 * cin)), dtype=torch.float32)
    b32 = torch.as_tensor(rng.normal(0, 0.1, cout), dtype=torch.float32)
    g = _bf16(rng.normal(0, 1, (n, h, w, cout)))
    x = xb.cuda().contiguous().requires_grad_(True)
    wp = w32.cuda().requires_grad_(True)
    bp = b32.cuda().requires_grad_(True)
    y = sur.conv_op(x, wp, bp, True)
    (y.float() * g.cuda().float()).sum().backward()
    wq = w32[:, : 9 * cin].to(torch.bfloat16).double().numpy()
    _, pre, cols = _conv_ref(xb.double().numpy(), wq, b32.double().numpy(), True)
    # the kernel's output is bfloat16: its ReLU mask is that of the rounded output
    ybf = _bf16(np.maximum(pre, 0)).double().numpy()
    dpre = _bf16(g.double().numpy() * (ybf > 0)).double().numpy()
    dw_ref = dpre.reshape(-1, cout).T @ cols.reshape(-1, 9 * cin)
    db_ref = dpre.reshape(-1, cout).sum(0)
    dcols = (dpre @ wq).reshape(n, h, w, 9, cin)
    dxp = np.zeros((n, h + 2, w + 2, cin))
    for t in range(9):
        ky, kx = divmod(t, 3)
        dxp[:, ky:ky + h, kx:kx + w, :] += dcols[:, :, :, t, :]
    dx_ref = dxp[:, 1:-1, 1:-1, :]
    dw = wp.grad[:, : 9 * cin].cpu().double().numpy()
    if wp.grad.shape[1] > 9 * cin:  # padding columns of the reduction get no gradient
        assert wp.grad[:, 9 * cin:].abs().max().item() == 0
    assert np.abs(dw - dw_ref).max() <= 1e-3 * np.abs(dw_ref).max()
    assert np.abs(bp.grad.cpu().double().numpy() - db_ref).max() <= 1e-3 * np.abs(db_ref).max()
    dx = x.grad.float().cpu().double().numpy()
    assert np.all(np.abs(dx - dx_ref) <= 2 ** -7 * np.abs(dx_ref) + 2e-2 * np.abs(dx_ref).max() / 64)


def test_training_reduces_loss(sur):
    """A few hundred Adam steps on engine-labelled tiles reduce the loss several-fold."""
    tiles = sur.make_tiles(24, 11)
    x = sur.encode_tiles(tiles)
    y = sur.label_tiles(tiles)
    net = sur.make_net(seed=1)
    losses = sur.train(net, x, y, steps=150, batch=8, lr=2e-3)
    first, last = np.mean(losses[:10]), np.mean(losses[-10:])
    assert last < first / 3, (first, last)


def test_inference_falls_back_to_the_engine(sur):
    """Tiles whose checked error exceeds the bound are replaced by the engine's
    result (errors injected on the host); the others keep the network's."""
    import torch
    dem = synthetic.fractal_dem(520, 3, side_y=600)
    net = sur.make_net(seed=2)
    area, st = sur.infer_dem(net, dem, check_fraction=0.25, bound=0.02,
                             force_error={t: 0.5 for t in range(9)})
    assert st["tiles"] == 9 and len(st["checked"]) == 2
    assert sorted(st["fell_back"]) == sorted(st["checked"])  # untrained net and injected errors
    # a fallen-back tile equals the engine's own result for that tile
    t = st["checked"][0]
    ty, tx = divmod(t, 3)
    tile = np.pad(dem, ((0, 768 - 600), (0, 768 - 520)), mode="edge")[ty * 256:(ty + 1) * 256, tx * 256:(tx + 1) * 256]
    from skewengine_gb300 import SkewEngine
    with SkewEngine(256, 256) as eng:
        want = eng.run(0, np.ascontiguousarray(tile, np.float32))
    got = np.pad(area, ((0, 768 - 600), (0, 768 - 520)))[ty * 256:(ty + 1) * 256, tx * 256:(tx + 1) * 256]
    h, w = min(256, 600 - ty * 256), min(256, 520 - tx * 256)
    want_log = torch.log1p(torch.as_tensor(want)).numpy()
    np.testing.assert_allclose(got[:h, :w], np.expm1(want_log)[:h, :w], rtol=1e-5, atol=1e-3)


def test_trained_network_beats_the_untrained_method(sur):
    """On held-out tiles the committed, trained network's total-area error is far
    below that of the method without it: a constant per-cell log area (the
    training labels' mean) and an untrained network of the same shape."""
    import torch
    net = sur.load_net()
    tiles = sur.make_tiles(48, 99)
    x = sur.encode_tiles(tiles)
    y = sur.label_tiles(tiles)
    with torch.no_grad():
        pred = torch.cat([net(x[i:i + 16]) for i in range(0, len(tiles), 16)])
        raw = torch.cat([sur.make_net(seed=5)(x[i:i + 16]) for i in range(0, len(tiles), 16)])
    err = sur.tile_area_error(pred, y)
    trained = np.median(err)
    constant = np.median(sur.tile_area_error(torch.full_like(y, float(y.mean())), y))
    untrained = np.median(sur.tile_area_error(raw, y))
    print(f"held-out tile-area error: trained median {trained:.4f} p90 {np.quantile(err, 0.9):.4f}, "
          f"constant {constant:.4f}, untrained {untrained:.4f}")
    assert trained < 0.5 * constant and trained < 0.5 * untrained, (trained, constant, untrained)
    # The stated bound: median tile-area error within 2% on these held-out tiles
    # (measured 1.89%, 5.9% at the 90th percentile; the tiles are seeded and the
    # forward pass and the engine's labels are deterministic, so the value repeats).
    assert trained <= 0.02, trained


@contextlib.contextmanager
def _conv_path(path):
    """Forward-convolution kernel choice (ske_conv_select) for the block."""
    from skewengine_gb300 import _lib
    lib = _lib.load()
    assert lib.ske_conv_select(path) == 0
    try:
        yield
    finally:
        lib.ske_conv_select(0)


# 0: warp-specialised persistent kernel, 2: halo-staged kernel (both stage the
# input once per 16-channel group; odd widths give an odd row pitch).
@pytest.mark.parametrize("path", [0, 2])
@pytest.mark.parametrize("n,h,w,cin,cout,relu", [(1, 8, 128, 32, 32, True), (2, 4, 256, 16, 48, False),
                                                  (1, 8, 256, 64, 128, True), (1, 4, 128, 192, 64, True),
                                                  (1, 760, 45, 16, 32, True), (3, 33, 30, 48, 16, False)])
def test_halo_conv_forward_matches_numpy(sur, path, n, h, w, cin, cout, relu):
    """The staged kernels against float64 NumPy.  760 x 45 (row pitch 47) has a
    tile whose first slot sits in the last column of its row, so the last
    output slot's tap (2, 2) reads the last staged plane slot."""
    import torch
    rng = np.random.default_rng(cin * 5 + cout + w)
    xb = _bf16(rng.normal(0, 1, (n, h, w, cin)))
    wb = _bf16(rng.normal(0, 0.2, (cout, 9 * cin)))
    b = torch.as_tensor(rng.normal(0, 0.5, cout), dtype=torch.float32)
    wpad = torch.zeros((cout, sur.kpad(cin)), dtype=torch.bfloat16)
    wpad[:, : 9 * cin] = wb
    with _conv_path(path):
        y = sur.conv3x3(xb.cuda().contiguous(), wpad.cuda(), b.cuda(), relu)
        sur.conv_check()
    y = y.float().cpu().numpy()
    ref, _, _ = _conv_ref(xb.double().numpy(), wb.double().numpy(), b.double().numpy(), relu)
    assert np.all(np.abs(y - ref) <= 2 ** -7 * np.abs(ref) + 1e-3), np.abs(y - ref).max()


def test_ws_upcat_many_tiles_equals_halo_bits(sur):
    """The fused upsample + concatenate convolution with several tiles per CTA:
    the warp-specialised kernel gives the halo-staged kernel's bits."""
    import torch
    rng = np.random.default_rng(12)
    for (n, r, c1, c2, cout) in ((32, 256, 64, 32, 32), (32, 64, 256, 128, 128)):
        low = _bf16(rng.normal(0, 1, (n, r // 2, r // 2, c1))).cuda().contiguous()
        skip = _bf16(rng.normal(0, 1, (n, r, r, c2))).cuda().contiguous()
        w = torch.zeros((cout, sur.kpad(c1 + c2)), dtype=torch.bfloat16)
        w[:, : 9 * (c1 + c2)] = _bf16(rng.normal(0, 0.05, (cout, 9 * (c1 + c2))))
        w = w.cuda()
        b = torch.as_tensor(rng.normal(0, 0.5, cout), dtype=torch.float32).cuda()
        with _conv_path(2):
            want = sur.conv3x3_upcat(low, skip, w, b, True)
        with _conv_path(0):
            got = sur.conv3x3_upcat(low, skip, w, b, True)
            sur.conv_check()
        assert torch.equal(got.view(torch.int16), want.view(torch.int16)), (n, r, c1, c2, cout)


@pytest.mark.parametrize("path", [0, 2])
def test_halo_upcat_equals_halo_conv_of_the_concatenation(sur, path):
    import torch
    import torch.nn.functional as F
    rng = np.random.default_rng(4)
    low = _bf16(rng.normal(0, 1, (2, 4, 64, 64))).cuda().contiguous()
    skip = _bf16(rng.normal(0, 1, (2, 8, 128, 32))).cuda().contiguous()
    w = torch.zeros((32, sur.kpad(96)), dtype=torch.bfloat16)
    w[:, : 9 * 96] = _bf16(rng.normal(0, 0.1, (32, 9 * 96)))
    w = w.cuda()
    b = torch.as_tensor(rng.normal(0, 0.5, 32), dtype=torch.float32).cuda()
    up = F.interpolate(low.permute(0, 3, 1, 2), scale_factor=2, mode="nearest").permute(0, 2, 3, 1)
    with _conv_path(path):
        want = sur.conv3x3(torch.cat([up, skip], 3).contiguous(), w, b, True)
        got = sur.conv3x3_upcat(low, skip, w, b, True)
        sur.conv_check()
    assert torch.equal(got.view(torch.int16), want.view(torch.int16))


@pytest.mark.parametrize("path", [0, 2])
def test_network_forward_halo_and_im2col_kernels_agree(sur, path):
    """The whole U-Net forward with a staged kernel (where it applies) and with
    the im2col kernel only: same function, float32 accumulation in different
    orders, so equal to bfloat16 rounding."""
    import torch
    net = sur.make_net(seed=5)
    x = sur.encode_tiles(np.stack([synthetic.fractal_dem(256, 80 + i) for i in range(2)]))
    with torch.no_grad():
        with _conv_path(1):
            ref = net(x)
        with _conv_path(path):
            got = net(x)
            sur.conv_check()
    err = (got - ref).abs().max().item()
    assert err <= 0.05 * ref.abs().max().item(), err


def test_ws_conv_equals_halo_conv_bits(sur):
    """The warp-specialised and halo-staged kernels issue the same MMAs in the
    same order per output (taps within a group, groups in order), so their
    outputs are the same bits.  The larger cases give every persistent CTA
    several tiles (2112, 1056 and 544 tiles on 152 SMs), so both tensor-memory
    accumulators and every pipeline stage are reused."""
    import torch
    rng = np.random.default_rng(11)
    for (n, h, w, cin, cout) in ((2, 16, 256, 32, 32), (1, 20, 64, 128, 128), (2, 9, 128, 64, 64),
                                 (32, 256, 256, 32, 32), (32, 128, 128, 64, 64), (32, 64, 64, 128, 128)):
        x = _bf16(rng.normal(0, 1, (n, h, w, cin))).cuda().contiguous()
        wt = torch.zeros((cout, sur.kpad(cin)), dtype=torch.bfloat16)
        wt[:, : 9 * cin] = _bf16(rng.normal(0, 0.1, (cout, 9 * cin)))
        wt = wt.cuda()
        b = torch.as_tensor(rng.normal(0, 0.5, cout), dtype=torch.float32).cuda()
        with _conv_path(2):
            want = sur.conv3x3(x, wt, b, True)
        with _conv_path(0):
            got = sur.conv3x3(x, wt, b, True)
            sur.conv_check()
        assert torch.equal(got.view(torch.int16), want.view(torch.int16)), (n, h, w, cin, cout)


def test_conv_head_equals_conv_then_1x1(sur):
    """The fused last convolution + 1x1 head against the two steps: bfloat16
    activations, then their float32 dot product with the head weights (orders
    of the float32 sums differ, so equal to float32 rounding).  16 tiles of
    64 x 256 give every persistent CTA two tiles."""
    import torch
    rng = np.random.default_rng(21)
    n, h, w, cin, cout = 16, 64, 256, 96, 32
    x = _bf16(rng.normal(0, 1, (n, h, w, cin))).cuda().contiguous()
    wt = torch.zeros((cout, sur.kpad(cin)), dtype=torch.bfloat16)
    wt[:, : 9 * cin] = _bf16(rng.normal(0, 0.05, (cout, 9 * cin)))
    wt = wt.cuda()
    b = torch.as_tensor(rng.normal(0, 0.5, cout), dtype=torch.float32).cuda()
    hw = torch.as_tensor(rng.normal(0, 0.3, (cout, 1)), dtype=torch.float32).cuda()
    hb = torch.tensor([8.0], device="cuda")
    got = sur.conv3x3_head(x, wt, b, hw, hb, True)
    sur.conv_check()
    assert got is not None and got.shape == (n, h, w)
    want = (sur.conv3x3(x, wt, b, True).float() @ hw)[..., 0] + hb
    err = (got - want).abs().max().item()
    assert err <= 1e-5 * want.abs().max().item(), err


def test_maxpool2_equals_torch_amax_bits(sur):
    import torch
    rng = np.random.default_rng(22)
    x = _bf16(rng.normal(0, 1, (3, 34, 18, 48))).cuda().contiguous()
    x.view(-1)[::977] = float("nan")
    want = x.view(3, 17, 2, 9, 2, 48).amax((2, 4))
    got = sur.maxpool2(x)
    assert torch.equal(torch.isnan(got), torch.isnan(want))
    assert torch.equal(got.nan_to_num(0).view(torch.int16), want.nan_to_num(0).view(torch.int16))


def test_encode_kernel_equals_tensor_expressions(sur):
    """The input-encoding kernel writes the bits of the element-wise tensor
    expressions it replaces (coarse areas repeated over their 4 x 4 cells)."""
    import torch
    tiles = torch.as_tensor(np.stack([synthetic.fractal_dem(256, 90 + i) for i in range(3)] +
                                     [np.full((256, 256), 7.0, np.float32)]), device="cuda")
    coarse = sur.coarse_area(tiles)
    assert coarse.shape == (4, 64, 64)
    got = sur.encode_tiles(tiles, coarse)
    t = tiles
    mean = t.mean((1, 2), keepdim=True)
    rng = t.amax((1, 2), keepdim=True) - t.amin((1, 2), keepdim=True)
    want = torch.zeros(t.shape + (8,), dtype=torch.bfloat16, device="cuda")
    want[..., 0] = ((t - mean) / torch.where(rng > 0, rng, torch.ones_like(rng))).to(torch.bfloat16)
    want[..., 1] = torch.log1p(rng).expand_as(t).to(torch.bfloat16)
    full = coarse.repeat_interleave(4, 1).repeat_interleave(4, 2)
    want[..., 2] = (torch.log1p(full) / sur.COARSE_SCALE).to(torch.bfloat16)
    assert torch.equal(got.view(torch.int16), want.view(torch.int16))


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 21, 18, 8, 16), (2, 64, 256, 32, 32), (1, 32, 64, 96, 64),
                                            (2, 16, 32, 64, 256), (3, 23, 45, 16, 40)])
def test_wgrad_tcgen05_matches_numpy(sur, n, h, w, cin, cout):
    """The tcgen05 weight gradient (ske_conv_wgrad_select(0): MN-major operands
    read in place from staged planes) and the default mma.sync kernel against
    float64 NumPy on the same bfloat16 inputs: 16- and 32-channel N blocks,
    several N and M blocks, 32-column segments with several tiles per CTA, an
    odd width."""
    import torch
    from skewengine_gb300 import _lib
    rng = np.random.default_rng(cin * 3 + cout + w)
    xb = _bf16(rng.normal(0, 1, (n, h, w, cin)))
    dyb = _bf16(rng.normal(0, 1, (n, h, w, cout)))
    xp = np.pad(xb.double().numpy(), ((0, 0), (1, 1), (1, 1), (0, 0)))
    cols = np.stack([xp[:, ky:ky + h, kx:kx + w, :] for ky in range(3) for kx in range(3)], axis=3)
    ref = dyb.double().numpy().reshape(-1, cout).T @ cols.reshape(-1, 9 * cin)
    x, dy = xb.cuda().contiguous(), dyb.cuda().contiguous()
    lib = _lib.load()
    try:
        assert lib.ske_conv_wgrad_select(0) == 0
        got = sur.conv3x3_wgrad(x, dy, cout)
    finally:
        assert lib.ske_conv_wgrad_select(1) == 0
    dflt = sur.conv3x3_wgrad(x, dy, cout)
    sur.conv_check()
    scale = np.abs(ref).max()
    for name, t in (("tcgen05", got), ("mma.sync", dflt)):
        v = t.cpu().double().numpy()
        assert np.all(v[:, 9 * cin:] == 0)
        err = np.abs(v[:, : 9 * cin] - ref).max() / scale
        print(f"wgrad {n}x{h}x{w} {cin}->{cout} {name}: {err:.1e} of max |dW|")
        assert err <= 1e-5, (name, err)
