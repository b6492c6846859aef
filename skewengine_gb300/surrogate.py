"""Learned total-viewshed surrogate.

A 4-level U-Net (32 base channels, 3x3 convolutions, bfloat16 weights and
activations, float32 accumulation) maps a 256 x 256 DEM tile to the log of the
visible area of each cell that the engine computes for that tile (kernelSDEM,
180 angles = 360 directional sectors).  The reference has no such model: it is
trained on the engine's own outputs, and at inference the engine itself checks
a sample of tiles and recomputes every tile whose error exceeds the bound.

The convolutions are the engine's hand-written implicit-GEMM kernels
(``ske_conv3x3_bf16`` forward and data gradient on tcgen05 with the accumulator
in tensor memory, ``ske_conv3x3_wgrad_bf16`` weight gradient on mma.sync, both
with bfloat16 operands and float32 accumulation).  At inference the decoder's
upsampling and concatenation are read in place by the convolution
(``ske_conv3x3_upcat_bf16``), the last convolution and the 1x1 output layer are
one kernel (``ske_conv3x3_head_bf16``) and pooling is a kernel of its own
(``ske_maxpool2_bf16``); in training those, the loss and the optimiser are
PyTorch operations around the convolutions.

Tensors are NHWC.  Input channels: 0 = the tile's heights minus their mean,
divided by the tile's height range (or 1 for a flat tile), 1 = log(1 + range)
(the relief amplitude, which visibility depends on), 2 = the engine's own total
viewshed of the tile at 1/4 resolution (4 x 4 cell means, 40 m cells) from every
4th angle, scaled by 4 (about 1/256 of the full-resolution run's work), as
log(1 + area per cell in tile cells) / 16, 3-7 = 0 (the kernels need a multiple
of 8 channels).  The tile-context head
predicts a correction to the log of the coarse run's total area.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import threading

import numpy as np

from . import synthetic
from ._lib import SkeError, check, load

TILE = 256
IN_CH = 8
BASE = 32
CTX = 64  # width of the tile-context MLP
COARSE = 4  # the coarse engine run's cell is COARSE x COARSE tile cells
COARSE_SCALE = 16.0  # input channel 2 = log(1 + coarse area per cell) / COARSE_SCALE
COARSE_ANGLE_STEP = 4  # the coarse run takes every 4th of the 180 angles
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "surrogate_unet32.npz")


def kpad(cin: int) -> int:
    """Padded reduction length of a 3x3 convolution with cin input channels."""
    return (9 * cin + 31) // 32 * 32


def _stream(t):
    import torch
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _need(t, name: str, dtype, shape=None, device=None) -> None:
    """Raise unless ``t`` is a contiguous CUDA tensor of ``dtype`` (and
    ``shape``, on ``device``).  The kernels take raw device pointers and size
    every read and write from the shape arguments, so a host tensor, another
    element type or a smaller tensor would be read or written out of place."""
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    if device is not None and t.device != device:
        raise ValueError(f"{name} is on {t.device}, the other operands on {device}")


def conv3x3(x, w, bias=None, relu: bool = False):
    """y = relu?(conv3x3(x, w) + bias); x (N, H, W, Cin) bf16, w (Cout, kpad(Cin)) bf16."""
    import torch
    _need(x, "x", torch.bfloat16)
    n, h, wd, cin = x.shape
    cout = w.shape[0]
    _need(w, "w", torch.bfloat16, (cout, kpad(cin)), x.device)
    if bias is not None:
        _need(bias, "bias", torch.float32, (cout,), x.device)
    y = torch.empty((n, h, wd, cout), dtype=torch.bfloat16, device=x.device)
    check(load().ske_conv3x3_bf16(C.c_void_p(x.data_ptr()), C.c_void_p(w.data_ptr()),
                                  C.c_void_p(bias.data_ptr()) if bias is not None else None,
                                  C.c_void_p(y.data_ptr()), n, h, wd, cin, cout, int(relu), _stream(x)))
    return y


def conv3x3_upcat(xlow, skip, w, bias=None, relu: bool = False):
    """conv3x3(cat([nearest-upsampled xlow, skip], channels)) without building the
    concatenation; the same values as conv3x3 on it."""
    import torch
    _need(skip, "skip", torch.bfloat16)
    n, h, wd, c2 = skip.shape
    _need(xlow, "xlow", torch.bfloat16, None, skip.device)
    c1 = xlow.shape[3]
    _need(xlow, "xlow", torch.bfloat16, (n, h // 2, wd // 2, c1))
    cout = w.shape[0]
    _need(w, "w", torch.bfloat16, (cout, kpad(c1 + c2)), skip.device)
    if bias is not None:
        _need(bias, "bias", torch.float32, (cout,), skip.device)
    y = torch.empty((n, h, wd, cout), dtype=torch.bfloat16, device=skip.device)
    check(load().ske_conv3x3_upcat_bf16(C.c_void_p(xlow.data_ptr()), C.c_void_p(skip.data_ptr()),
                                        C.c_void_p(w.data_ptr()),
                                        C.c_void_p(bias.data_ptr()) if bias is not None else None,
                                        C.c_void_p(y.data_ptr()), n, h, wd, c1, c2, cout, int(relu), _stream(skip)))
    return y


def conv3x3_head(x, w, bias, head_w, head_b, relu: bool = True):
    """head_b + sum_c bf16(relu?(conv3x3(x, w) + bias))[..., c] * head_w[c]: the
    3x3 convolution and a 1x1 convolution to one channel in one kernel
    (ske_conv3x3_head_bf16), float32 (N, H, W); the activations are not stored.
    None where that kernel does not apply."""
    import torch
    _need(x, "x", torch.bfloat16)
    n, h, wd, cin = x.shape
    cout = w.shape[0]
    _need(w, "w", torch.bfloat16, (cout, kpad(cin)), x.device)
    if bias is not None:
        _need(bias, "bias", torch.float32, (cout,), x.device)
    hw = head_w.reshape(-1).float().contiguous()
    hb = head_b.reshape(-1).float().contiguous()
    _need(hw, "head_w", torch.float32, (cout,), x.device)
    _need(hb, "head_b", torch.float32, (1,), x.device)
    y = torch.empty((n, h, wd), dtype=torch.float32, device=x.device)
    rc = load().ske_conv3x3_head_bf16(C.c_void_p(x.data_ptr()), C.c_void_p(w.data_ptr()),
                                      C.c_void_p(bias.data_ptr()) if bias is not None else None,
                                      C.c_void_p(hw.data_ptr()), C.c_void_p(hb.data_ptr()), C.c_void_p(y.data_ptr()),
                                      n, h, wd, cin, cout, int(relu), _stream(x))
    if rc == 5:  # SKE_ERR_UNSUPPORTED
        return None
    check(rc)
    return y


def maxpool2(x):
    """2 x 2 max pooling of a contiguous NHWC bfloat16 tensor (ske_maxpool2_bf16)."""
    import torch
    _need(x, "x", torch.bfloat16)
    n, h, wd, c = x.shape
    y = torch.empty((n, h // 2, wd // 2, c), dtype=torch.bfloat16, device=x.device)
    check(load().ske_maxpool2_bf16(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), n, h, wd, c, _stream(x)))
    return y


def conv_check(device=None) -> None:
    """Synchronise the current stream and raise SkeError if a forward convolution
    since the previous check gave up waiting for its tensor-core operations."""
    import torch
    failed = C.c_int(0)
    check(load().ske_conv_status(C.byref(failed), C.c_void_p(torch.cuda.current_stream(device).cuda_stream)))
    if failed.value:
        raise SkeError(6, "a tensor-core convolution gave up waiting for its MMAs; its output is not valid")


def conv3x3_wgrad(x, dy, cout: int):
    """dW (Cout, kpad(Cin)) float32 of conv3x3 for input x and output gradient dy."""
    import torch
    _need(x, "x", torch.bfloat16)
    n, h, wd, cin = x.shape
    _need(dy, "dy", torch.bfloat16, (n, h, wd, cout), x.device)
    dw = torch.zeros((cout, kpad(cin)), dtype=torch.float32, device=x.device)
    check(load().ske_conv3x3_wgrad_bf16(C.c_void_p(x.data_ptr()), C.c_void_p(dy.data_ptr()),
                                        C.c_void_p(dw.data_ptr()), n, h, wd, cin, cout, _stream(x)))
    return dw


def flip_transpose(w, cin: int, cout: int):
    """Weights of the data gradient: W'[ci][(ky*3+kx)*cout + co] = W[co][((2-ky)*3 + 2-kx)*cin + ci]."""
    import torch
    w9 = w[:, : 9 * cin].reshape(cout, 9, cin).flip(1).permute(2, 1, 0).reshape(cin, 9 * cout)
    out = torch.zeros((cin, kpad(cout)), dtype=w.dtype, device=w.device)
    out[:, : 9 * cout] = w9
    return out


def _conv_fn():
    import torch

    class Conv3x3(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, w32, b, relu):
            w = w32.to(torch.bfloat16)
            y = conv3x3(x, w, b, relu)
            ctx.save_for_backward(x, w, y)
            ctx.relu = relu
            return y

        @staticmethod
        def backward(ctx, dy):
            x, w, y = ctx.saved_tensors
            if ctx.relu:
                dy = dy * (y > 0)
            dy = dy.to(torch.bfloat16).contiguous()
            cin, cout = x.shape[3], w.shape[0]
            dx = conv3x3(dy, flip_transpose(w, cin, cout)) if ctx.needs_input_grad[0] else None
            dw = conv3x3_wgrad(x, dy, cout)
            db = dy.float().sum((0, 1, 2))
            return dx, dw, db, None

    return Conv3x3


_CONV = None


def conv_op(x, w32, b, relu=True):
    global _CONV
    if _CONV is None:
        _CONV = _conv_fn()
    return _CONV.apply(x, w32, b, relu)


# Channel plan: (name, cin, cout).
LAYERS = [("e1a", IN_CH, BASE), ("e1b", BASE, BASE),
          ("e2a", BASE, 2 * BASE), ("e2b", 2 * BASE, 2 * BASE),
          ("e3a", 2 * BASE, 4 * BASE), ("e3b", 4 * BASE, 4 * BASE),
          ("b4a", 4 * BASE, 8 * BASE), ("b4b", 8 * BASE, 8 * BASE),
          ("d3a", 12 * BASE, 4 * BASE), ("d3b", 4 * BASE, 4 * BASE),
          ("d2a", 6 * BASE, 2 * BASE), ("d2b", 2 * BASE, 2 * BASE),
          ("d1a", 3 * BASE, BASE), ("d1b", BASE, BASE)]


def conv_flops_per_tile(size: int = TILE) -> float:
    """2 * 9 * Cin * Cout * H * W summed over the network's 3x3 convolutions."""
    res = {"e1": size, "e2": size // 2, "e3": size // 4, "b4": size // 8, "d3": size // 4, "d2": size // 2,
           "d1": size}
    return float(sum(2 * 9 * cin * cout * res[name[:2]] ** 2 for name, cin, cout in LAYERS))


def make_net(seed: int = 0, device="cuda"):
    import torch

    class UNet(torch.nn.Module):
        def __init__(self):
            super().__init__()
            g = torch.Generator().manual_seed(seed)
            self.w = torch.nn.ParameterDict()
            self.b = torch.nn.ParameterDict()
            for name, cin, cout in LAYERS:
                w = torch.zeros(cout, kpad(cin))
                w[:, : 9 * cin] = torch.randn(cout, 9 * cin, generator=g) * math.sqrt(2.0 / (9 * cin))
                self.w[name] = torch.nn.Parameter(w)
                self.b[name] = torch.nn.Parameter(torch.zeros(cout))
            self.head_w = torch.nn.Parameter(torch.randn(BASE, 1, generator=g) * math.sqrt(1.0 / BASE))
            self.head_b = torch.nn.Parameter(torch.full((1,), 8.0))
            # Tile context: the bottleneck's channel means (and maxima) -> MLP
            # -> the log of the tile's total visible area, which calibrates the
            # per-cell map (visibility is a property of whole lines of sight).
            cin = 2 * 8 * BASE + 1
            self.ctx1_w = torch.nn.Parameter(torch.randn(cin, CTX, generator=g) * math.sqrt(2.0 / cin))
            self.ctx1_b = torch.nn.Parameter(torch.zeros(CTX))
            self.ctx2_w = torch.nn.Parameter(torch.randn(CTX, 1, generator=g) * math.sqrt(1.0 / CTX) * 0.1)
            self.ctx2_b = torch.nn.Parameter(torch.zeros(1))
            self._wb = {}

        def c(self, x, name):
            if not torch.is_grad_enabled():
                return conv3x3(x, self.wb(name), self.b[name], True)
            return conv_op(x, self.w[name], self.b[name], True)

        def wb(self, name):
            # bfloat16 copy of a layer's weights for inference, made again only
            # when the float32 parameter has changed (its version counter).
            p = self.w[name]
            hit = self._wb.get(name)
            if hit is None or hit[0] != p._version or hit[1].device != p.device:
                hit = (p._version, p.detach().to(torch.bfloat16).contiguous())
                self._wb[name] = hit
            return hit[1]

        @staticmethod
        def pool(x):
            # 2 x 2 max pooling of an NHWC tensor in place of layout (no NCHW round
            # trip); without gradients one kernel (the same values).
            n, h, w, c = x.shape
            if not torch.is_grad_enabled() and x.is_contiguous() and h % 2 == 0 and w % 2 == 0 and c % 8 == 0:
                return maxpool2(x)
            return x.view(n, h // 2, 2, w // 2, 2, c).amax((2, 4))

        @staticmethod
        def up(x):
            import torch.nn.functional as F
            return F.interpolate(x.permute(0, 3, 1, 2), scale_factor=2, mode="nearest").permute(0, 2, 3, 1)

        def upcat(self, low, skip, name):
            # Without gradients the decoder reads the upsampled low-resolution
            # input and the skip connection in place (same values).
            if not torch.is_grad_enabled():
                return conv3x3_upcat(low, skip, self.wb(name), self.b[name], True)
            return self.c(torch.cat([self.up(low), skip], 3).contiguous(), name)

        def forward(self, x):
            e1 = self.c(self.c(x, "e1a"), "e1b")
            e2 = self.c(self.c(self.pool(e1), "e2a"), "e2b")
            e3 = self.c(self.c(self.pool(e2), "e3a"), "e3b")
            b4 = self.c(self.c(self.pool(e3), "b4a"), "b4b")
            d3 = self.c(self.upcat(b4, e3, "d3a"), "d3b")
            d2 = self.c(self.upcat(d3, e2, "d2a"), "d2b")
            d1a = self.upcat(d2, e1, "d1a")
            cells = None
            if not torch.is_grad_enabled():  # the last convolution and the 1x1 head in one kernel
                cells = conv3x3_head(d1a, self.wb("d1b"), self.b["d1b"], self.head_w, self.head_b, True)
            if cells is None:
                d1 = self.c(d1a, "d1b")
                cells = (d1.float() @ self.head_w)[..., 0] + self.head_b  # (N, H, W) log(1 + area)
            # log total area of the coarse engine run (input channel 2)
            lct = torch.log(torch.expm1(x[..., 2].float() * COARSE_SCALE).clamp_min(0).sum((1, 2)).clamp_min(1.0))
            # the bottleneck's channel means (float32 sums) and maxima
            pooled = torch.cat([b4.mean((1, 2), dtype=torch.float32), b4.amax((1, 2)).float(),
                                (lct / 20.0)[:, None]], 1)
            t = lct + (torch.relu(pooled @ self.ctx1_w + self.ctx1_b) @ self.ctx2_w)[:, 0] + self.ctx2_b
            return calibrate(cells, t)

    import torch  # noqa: F811  (used inside forward)
    return UNet().to(device)


def calibrate(cells, log_total):
    """Scale the per-cell areas of each tile (cells: log(1 + area)) so that they
    sum to exp(log_total); returns log(1 + scaled area)."""
    import torch
    area = torch.expm1(cells).clamp_min(0.0)
    tot = area.sum((1, 2)).clamp_min(1e-6)
    scale = torch.exp(log_total - torch.log(tot))
    return torch.log1p(area * scale[:, None, None])


_COARSE_ENGINES = {}


def coarse_area(tiles, engine=None, chunk: int = 4096):
    """The engine's total viewshed of each tile at 1/COARSE resolution from
    every COARSE_ANGLE_STEP-th of the 180 angles (scaled by the step), per
    coarse cell in tile-cell units: (N, 256/COARSE, 256/COARSE) float32 (CUDA);
    every tile cell takes its coarse cell's value.  The coarse grid averages
    COARSE x COARSE cells; its heights, observer height and areas are rescaled
    to its COARSE-times larger cells."""
    import torch
    from .engine import SkewEngine, run_batch
    t = torch.as_tensor(tiles, dtype=torch.float32, device="cuda")
    n, side = t.shape[0], TILE // COARSE
    c = (t.reshape(n, side, COARSE, side, COARSE).mean((2, 4)) / COARSE).contiguous()
    out = torch.empty_like(c)
    if engine is None:  # one engine per device for the process: it keeps the batch plan
        dev = torch.cuda.current_device()
        if dev not in _COARSE_ENGINES:
            _COARSE_ENGINES[dev] = SkewEngine(side, side, device=dev)
        engine = _COARSE_ENGINES[dev]
    povh = float(synthetic.POVH) / COARSE
    angles = list(range(0, 180, COARSE_ANGLE_STEP))
    for i in range(0, n, chunk):
        run_batch(0, c[i:i + chunk], povh=povh, engine=engine, outs=out[i:i + chunk], angles=angles)
    return out * float(COARSE * COARSE * COARSE_ANGLE_STEP)


def encode_tiles(tiles, coarse=None):
    """(N, 256, 256) float32 heights (NumPy or CUDA tensor) -> (N, 256, 256, 8)
    bfloat16 network input (CUDA), written by one kernel
    (ske_surrogate_encode_bf16).  coarse: coarse_area(tiles), computed here
    when not given."""
    import torch
    t = torch.as_tensor(tiles, dtype=torch.float32, device="cuda").contiguous()
    if t.dim() != 3 or t.shape[1] != t.shape[2]:
        raise ValueError(f"tiles must be (N, side, side), got {tuple(t.shape)}")
    n, side = t.shape[0], t.shape[1]
    mean = t.mean((1, 2)).contiguous()
    rng = (t.amax((1, 2)) - t.amin((1, 2))).contiguous()
    if coarse is None:
        coarse = coarse_area(t)
    coarse = coarse.contiguous()
    # The kernel reads N coarse grids of (side / factor)^2 cells, the factor
    # taken from the coarse grid's side, which must divide the tile's.
    c = int(coarse.shape[-1]) if coarse.dim() == 3 else 0
    if c < 1 or side % c:
        raise ValueError(f"coarse must be (N, c, c) with c dividing {side}, got {tuple(coarse.shape)}")
    _need(coarse, "coarse", torch.float32, (n, c, c), t.device)
    x = torch.empty(t.shape + (IN_CH,), dtype=torch.bfloat16, device="cuda")
    check(load().ske_surrogate_encode_bf16(C.c_void_p(t.data_ptr()), C.c_void_p(mean.data_ptr()),
                                           C.c_void_p(rng.data_ptr()), C.c_void_p(coarse.data_ptr()),
                                           side // c, COARSE_SCALE, C.c_void_p(x.data_ptr()), n, side,
                                           _stream(t)))
    return x


def label_tiles(tiles: np.ndarray, engine=None, chunk: int = 512):
    """The engine's total visible area of every cell of each tile (180 angles),
    as log(1 + area): batched engine calls of `chunk` tiles each."""
    import torch
    from .engine import SkewEngine, run_batch
    eng = engine or SkewEngine(tiles.shape[2], tiles.shape[1])
    out = torch.empty(tiles.shape, dtype=torch.float32, device="cuda")
    for i in range(0, len(tiles), chunk):
        x = torch.as_tensor(np.ascontiguousarray(tiles[i:i + chunk], np.float32), device="cuda")
        run_batch(0, x, engine=eng, outs=out[i:i + len(x)])
    torch.cuda.synchronize()
    if engine is None:
        eng.close()
    return torch.log1p(out)


SOURCE_SIDES = (256, 512, 1024, 2048, 4096)


def _dem_tiles(args):
    side, seed, h = args
    return cut_tiles(synthetic.fractal_dem(side, seed, roughness=h))[0]


def make_tiles(count: int, seed: int, workers: int | None = None) -> np.ndarray:
    """Seeded fractal DEM tiles: the 256 x 256 tiles of diamond-square DEMs of
    sides 256 to 4096 (roughness 0.6-0.9, 0-1500 m relief, 10 m cells), an equal
    share of the tiles from each side, shuffled.  A tile of a larger DEM has less
    relief than a whole small DEM, as the tiles of a large DEM at inference do.
    Large counts are generated by a pool of spawned processes (spawned, so that
    no CUDA context is forked)."""
    rng = np.random.default_rng(seed)
    share = [count // len(SOURCE_SIDES) + (i < count % len(SOURCE_SIDES)) for i in range(len(SOURCE_SIDES))]
    spec, cls = [], []
    for c, side in enumerate(SOURCE_SIDES):
        per_dem = (side // TILE) ** 2
        for _ in range(-(-share[c] // per_dem)):
            spec.append((side, int(rng.integers(1 << 30)), float(rng.uniform(0.6, 0.9))))
            cls.append(c)
    if count < 256:
        parts = [_dem_tiles(a) for a in spec]
    else:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(workers or os.cpu_count()) as pool:
            parts = pool.map(_dem_tiles, spec, chunksize=1)
    picked = []
    for c in range(len(SOURCE_SIDES)):
        pool_c = np.concatenate([p for p, k in zip(parts, cls) if k == c]) if share[c] else np.zeros((0, TILE, TILE))
        picked.append(pool_c[rng.permutation(len(pool_c))[: share[c]]])
    tiles = np.concatenate(picked).astype(np.float32)
    return tiles[rng.permutation(len(tiles))]


def _log_total(logarea):
    """log of a tile's total visible area from per-cell log(1 + area)."""
    import torch
    return torch.log(torch.expm1(logarea.float()).clamp_min(0.0).sum((1, 2)).clamp_min(1e-6))


def train(net, x, y, steps: int, batch: int = 16, lr: float = 2e-3, seed: int = 0, log=None,
          tile_weight: float = 1.0):
    """Adam on the mean squared error of per-cell log area plus `tile_weight`
    times the squared error of the log of each tile's total area (per-cell log
    errors alone leave tile totals biased low: the totals are dominated by the
    few cells that see far).  The learning rate warms up linearly over the first
    5% of the steps and then follows a cosine to zero; gradients are clipped to
    norm 1 (without both, runs at this rate could diverge part-way).  Returns
    the per-step losses."""
    import torch
    opt = torch.optim.Adam(net.parameters(), lr=lr)
    warm = max(1, steps // 20)
    sched = torch.optim.lr_scheduler.LambdaLR(
        opt, lambda s: min(1.0, (s + 1) / warm) * 0.5 * (1.0 + math.cos(math.pi * min(s, steps) / max(steps, 1))))
    g = torch.Generator(device="cpu").manual_seed(seed)
    losses = []
    for step in range(steps):
        idx = torch.randint(0, x.shape[0], (batch,), generator=g).to(x.device)
        pred = net(x[idx])
        yt = y[idx]
        loss = torch.mean((pred - yt) ** 2) + tile_weight * torch.mean((_log_total(pred) - _log_total(yt)) ** 2)
        opt.zero_grad(set_to_none=True)
        loss.backward()
        torch.nn.utils.clip_grad_norm_(net.parameters(), 1.0)
        opt.step()
        sched.step()
        losses.append(float(loss.detach()))
        if step % 200 == 0 or step == steps - 1:
            conv_check()
        if log and (step % 200 == 0 or step == steps - 1):
            log(f"step {step} loss {losses[-1]:.4f}")
    return losses


def save(net, path: str = WEIGHTS) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    arrs = {k: v.detach().float().cpu().numpy() for k, v in net.state_dict().items()}
    np.savez_compressed(path, **arrs)


def load_net(path: str = WEIGHTS, device="cuda"):
    import torch
    net = make_net(device=device)
    z = np.load(path)
    net.load_state_dict({k: torch.as_tensor(z[k]) for k in z.files})
    return net


def tile_area_error(pred_log, true_log):
    """Per tile: |sum(pred area) - sum(true area)| / sum(true area)."""
    import torch
    pa = torch.expm1(pred_log.float()).clamp_min(0).sum((1, 2))
    ta = torch.expm1(true_log.float()).sum((1, 2))
    return ((pa - ta).abs() / ta.clamp_min(1e-6)).cpu().numpy()


def cut_tiles(dem: np.ndarray):
    """256 x 256 tiles of a DEM in row-major tile order (edge tiles padded by
    replicating the last row / column) and the tile grid's shape."""
    H, W = dem.shape
    ty, tx = -(-H // TILE), -(-W // TILE)
    padded = np.pad(dem, ((0, ty * TILE - H), (0, tx * TILE - W)), mode="edge")
    return padded.reshape(ty, TILE, tx, TILE).transpose(0, 2, 1, 3).reshape(ty * tx, TILE, TILE), (ty, tx)


def _cut_tiles_dev(dem):
    """cut_tiles on a CUDA tensor, on the device."""
    import torch.nn.functional as F
    H, W = dem.shape
    ty, tx = -(-H // TILE), -(-W // TILE)
    padded = F.pad(dem[None, None], (0, tx * TILE - W, 0, ty * TILE - H), mode="replicate")[0, 0]
    return padded.reshape(ty, TILE, tx, TILE).permute(0, 2, 1, 3).reshape(ty * tx, TILE, TILE).contiguous(), (ty, tx)


def infer_dem(net, dem, engine=None, check_fraction: float = 0.05, bound: float = 0.02,
              batch: int = 256, seed: int = 0, force_error=None):
    """Per-tile total viewshed of a large DEM cut into 256 x 256 tiles (edge tiles
    padded by replicating the last row / column).  The network predicts every
    tile; the engine recomputes a random check_fraction of them, and any checked
    tile whose total visible area is off by more than `bound` (relative) is
    replaced by the engine's result.  `force_error` (tile index -> error) injects
    errors on the host to exercise the fallback.

    `dem` is a NumPy array or a CUDA tensor; the area map comes back the same way
    (a CUDA tensor stays on the device throughout).  Returns (area map, stats)."""
    import torch
    from .engine import SkewEngine, run_batch
    on_host = not torch.is_tensor(dem)
    d = torch.as_tensor(np.ascontiguousarray(dem, np.float32) if on_host else dem, dtype=torch.float32,
                        device="cuda")
    H, W = d.shape
    tiles, (ty, tx) = _cut_tiles_dev(d)
    rng = np.random.default_rng(seed)
    n_check = max(1, int(round(check_fraction * len(tiles))))
    checked = np.sort(rng.choice(len(tiles), n_check, replace=False))
    eng = engine or SkewEngine(TILE, TILE)
    truth = torch.empty((n_check, TILE, TILE), dtype=torch.float32, device="cuda")
    sel = tiles[torch.as_tensor(checked, device="cuda")].contiguous()
    # The checked tiles do not depend on the network: their batched engine call
    # (ske_run_batch on the engine's own stream, a CUDA graph replay after the
    # first call) runs from a host thread while this thread computes the coarse
    # channel and the network on torch's stream.
    # The engine's stream waits here for the gather of `sel` (torch's stream of
    # this thread); the worker makes the engine's stream its current one, so it
    # adds no wait on other work.
    eng._after_torch(sel, truth)
    failure = []

    def checks():
        try:
            with torch.cuda.stream(eng._ext):
                run_batch(0, sel, engine=eng, outs=truth)
        except BaseException as exc:  # re-raised below
            failure.append(exc)

    worker = threading.Thread(target=checks)
    worker.start()
    try:
        x = encode_tiles(tiles)
        out = torch.empty((len(tiles), TILE, TILE), dtype=torch.float32, device="cuda")
        with torch.no_grad():
            for i in range(0, len(tiles), batch):
                out[i:i + batch] = net(x[i:i + batch])
        conv_check()
    finally:
        worker.join()
    if failure:
        raise failure[0]
    truth = torch.log1p(truth)
    errs = tile_area_error(out[torch.as_tensor(checked, device="cuda")], truth)
    if force_error:
        for j, t in enumerate(checked):
            if int(t) in force_error:
                errs[j] = force_error[int(t)]
    fell_back = [int(t) for t, e in zip(checked, errs) if e > bound]
    for j, t in enumerate(checked):
        if errs[j] > bound:
            out[int(t)] = truth[j]
    if engine is None:
        eng.close()
    area = torch.expm1(out).clamp_min_(0)
    area = area.reshape(ty, tx, TILE, TILE).permute(0, 2, 1, 3).reshape(ty * TILE, tx * TILE)[:H, :W]
    stats = {"tiles": int(len(tiles)), "checked": [int(t) for t in checked], "errors": [float(e) for e in errs],
             "fell_back": fell_back}
    return (area.cpu().numpy() if on_host else area), stats


def main(argv=None) -> int:
    """Train the surrogate on engine-labelled tiles and save its weights:
    python -m skewengine_gb300.surrogate --tiles 20000 --steps 4000."""
    import argparse
    import json
    import time
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--tiles", type=int, default=20000)
    ap.add_argument("--val", type=int, default=256)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--tile-weight", type=float, default=4.0)
    ap.add_argument("--out", default=WEIGHTS)
    a = ap.parse_args(argv)
    t0 = time.time()
    tiles = make_tiles(a.tiles, 1)
    val = make_tiles(a.val, 2)
    t1 = time.time()
    x, y = encode_tiles(tiles), label_tiles(tiles)
    xv, yv = encode_tiles(val), label_tiles(val)
    torch.cuda.synchronize()
    t2 = time.time()
    net = make_net(seed=0)
    losses = train(net, x, y, a.steps, a.batch, a.lr, log=lambda m: print(m, flush=True),
                   tile_weight=a.tile_weight)
    torch.cuda.synchronize()
    t3 = time.time()
    with torch.no_grad():
        pv = torch.cat([net(xv[i:i + 16]) for i in range(0, len(xv), 16)])
    err = tile_area_error(pv, yv)
    base = tile_area_error(torch.full_like(yv, float(y.mean())), yv)
    save(net, a.out)
    print(json.dumps({"tiles": a.tiles, "steps": a.steps, "batch": a.batch, "gen_s": t1 - t0, "label_s": t2 - t1,
                      "train_s": t3 - t2, "final_loss": float(np.mean(losses[-50:])),
                      "val_rms_log": float(torch.sqrt(torch.mean((pv - yv) ** 2))),
                      "val_tile_area_err_median": float(np.median(err)), "val_tile_area_err_p90": float(np.quantile(err, 0.9)),
                      "val_within_2pct": float(np.mean(err <= 0.02)),
                      "baseline_tile_area_err_median": float(np.median(base)),
                      "baseline_within_2pct": float(np.mean(base <= 0.02))}), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
