"""Host-side parts of the learned surrogate, on the CPU: the weight transform of
the data gradient, the tiling of a DEM and its reassembly, the tile-area error
and the network's convolution work count."""
from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from skewengine_gb300 import surrogate as sur  # noqa: E402


def _conv(x, w, cin):
    """3x3 convolution, zero padding 1, NHWC float64; w: (Cout, >= 9*cin), entry
    [co][(ky*3 + kx)*cin + ci]."""
    n, h, wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    cols = np.stack([xp[:, ky:ky + h, kx:kx + wd, :] for ky in range(3) for kx in range(3)], axis=3)
    return cols.reshape(n, h, wd, 9 * cin) @ w[:, : 9 * cin].T


@pytest.mark.parametrize("cin,cout", [(8, 16), (32, 24)])
def test_flip_transpose_gives_the_data_gradient(cin, cout):
    """d(sum(g * conv(x, W)))/dx equals conv(g, flip_transpose(W)): the backward
    pass runs the forward kernel on these weights."""
    rng = np.random.default_rng(cin + cout)
    n, h, wd = 2, 7, 9
    x = rng.normal(0, 1, (n, h, wd, cin))
    w = np.zeros((cout, sur.kpad(cin)))
    w[:, : 9 * cin] = rng.normal(0, 1, (cout, 9 * cin))
    g = rng.normal(0, 1, (n, h, wd, cout))
    # adjoint of the im2col gather
    dcols = (g @ w[:, : 9 * cin]).reshape(n, h, wd, 9, cin)
    dxp = np.zeros((n, h + 2, wd + 2, cin))
    for t in range(9):
        ky, kx = divmod(t, 3)
        dxp[:, ky:ky + h, kx:kx + wd, :] += dcols[:, :, :, t, :]
    want = dxp[:, 1:-1, 1:-1, :]
    wt = sur.flip_transpose(torch.as_tensor(w), cin, cout)
    assert tuple(wt.shape) == (cin, sur.kpad(cout))
    if wt.shape[1] > 9 * cout:  # padding columns of the reduction stay zero
        assert wt[:, 9 * cout:].abs().max().item() == 0
    got = _conv(g, wt.numpy(), cout)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-10)


def test_kpad_is_the_reduction_rounded_to_32():
    assert [sur.kpad(c) for c in (8, 32, 96, 384)] == [96, 288, 864, 3456]
    assert all(sur.kpad(c) % 32 == 0 and sur.kpad(c) >= 9 * c for c in range(8, 520, 8))


@pytest.mark.parametrize("shape", [(256, 256), (300, 520), (600, 257), (5, 700)])
def test_tiling_covers_the_dem_and_reassembles(shape):
    rng = np.random.default_rng(shape[0])
    dem = rng.normal(0, 10, shape).astype(np.float32)
    tiles, (ty, tx) = sur.cut_tiles(dem)
    assert tiles.shape == (ty * tx, sur.TILE, sur.TILE)
    assert ty * sur.TILE >= shape[0] > (ty - 1) * sur.TILE and tx * sur.TILE >= shape[1] > (tx - 1) * sur.TILE
    back = tiles.reshape(ty, tx, sur.TILE, sur.TILE).transpose(0, 2, 1, 3).reshape(ty * sur.TILE, tx * sur.TILE)
    assert np.array_equal(back[: shape[0], : shape[1]], dem)
    # padding replicates the last row and column
    assert np.array_equal(back[shape[0]:, : shape[1]], np.broadcast_to(dem[-1], back[shape[0]:, : shape[1]].shape))
    assert np.array_equal(back[: shape[0], shape[1]:],
                          np.broadcast_to(dem[:, -1:], back[: shape[0], shape[1]:].shape))
    # the device-side cut (here on a CPU tensor) gives the same tiles
    dev, grid = sur._cut_tiles_dev(torch.as_tensor(dem))
    assert grid == (ty, tx) and np.array_equal(dev.numpy(), tiles)


def test_tile_area_error():
    true = torch.log1p(torch.full((2, 4, 4), 99.0))  # 16 cells of area 99 per tile
    pred = true.clone()
    pred[1] = torch.log1p(torch.full((4, 4), 108.9))  # tile 1: 10% high
    err = sur.tile_area_error(pred, true)
    assert err[0] == 0 and abs(err[1] - 0.1) < 1e-5


def test_convolution_work_count():
    """2 * 9 * Cin * Cout per output pixel, summed over the U-Net's convolutions
    at their resolutions: 21.44 GFLOP per 256 x 256 tile."""
    res = {"e1": 256, "e2": 128, "e3": 64, "b4": 32, "d3": 64, "d2": 128, "d1": 256}
    want = sum(18 * cin * cout * res[name[:2]] ** 2 for name, cin, cout in sur.LAYERS)
    assert sur.conv_flops_per_tile() == want
    assert abs(want / 1e9 - 21.44) < 0.01
    # the decoder's inputs are the upsampled level below and the skip connection
    chans = {name: (cin, cout) for name, cin, cout in sur.LAYERS}
    assert chans["d3a"][0] == chans["b4b"][1] + chans["e3b"][1]
    assert chans["d2a"][0] == chans["d3b"][1] + chans["e2b"][1]
    assert chans["d1a"][0] == chans["d2b"][1] + chans["e1b"][1]


def test_kernel_wrappers_refuse_host_tensors_and_wrong_types():
    """The convolution, pooling and weight-gradient wrappers hand raw device
    pointers to kernels that size every access from the shape arguments, so
    each refuses a host tensor (or a non-tensor) before any kernel is called.
    The element-type, contiguity and shape checks come after this one and
    need CUDA tensors to reach."""
    bf = torch.bfloat16
    x = torch.zeros((1, 8, 8, 8), dtype=bf)
    w = torch.zeros((16, sur.kpad(8)), dtype=bf)
    with pytest.raises(TypeError, match="CUDA"):
        sur.conv3x3(x, w)
    with pytest.raises(TypeError, match="CUDA"):
        sur.conv3x3_upcat(torch.zeros((1, 4, 4, 8), dtype=bf), x, torch.zeros((16, sur.kpad(16)), dtype=bf))
    with pytest.raises(TypeError, match="CUDA"):
        sur.conv3x3_head(x, w, None, torch.zeros(16), torch.zeros(1))
    with pytest.raises(TypeError, match="CUDA"):
        sur.maxpool2(x)
    with pytest.raises(TypeError, match="CUDA"):
        sur.conv3x3_wgrad(x, torch.zeros((1, 8, 8, 16), dtype=bf), 16)
    with pytest.raises(TypeError, match="CUDA"):
        sur.conv3x3(None, w)
