"""Seeded synthetic inputs standing in for the reference's data files.

The reference reads a 2000x2000 int16 ``.bil`` DEM and a PNG image from a
hard-coded input folder (``src/main.h:23-58``, ``src/kernelSDEM.h:31-55``); neither
file ships with it.  These generators produce inputs with the shapes, units and
value distributions the workloads are quoted on:

* ``fractal_dem``: diamond-square terrain, heights in metres rescaled to cell units
  (divided by the 10 m cell size, as ``readBilData`` does at ``kernelSDEM.h:47``);
* ``ellipse_phantom``: sum of random ellipses on [-1, 1]^2 (Radon / back-projection);
* ``blurred_texture``: 1/f^2 spectral noise blurred by a linear motion kernel plus
  Gaussian noise (cepstrum blur estimation).

All randomness comes from ``numpy.random.default_rng(seed)`` so inputs are
reproducible.
"""
from __future__ import annotations

import numpy as np

CELL_SIZE_M = 10.0  # kernelSDEM.h:11 (STEP)
OBSERVER_HEIGHT_M = 1.5  # kernelSDEM.h:12 (OBS_H)
POVH = np.float32(OBSERVER_HEIGHT_M / CELL_SIZE_M)  # kernelSDEM.h:159


def _diamond_square(levels: int, roughness: float, rng: np.random.Generator) -> np.ndarray:
    size = (1 << levels) + 1
    g = np.zeros((size, size), dtype=np.float64)
    g[0, 0], g[0, -1], g[-1, 0], g[-1, -1] = rng.standard_normal(4)
    step = size - 1
    amp = 1.0
    decay = 2.0 ** (-roughness)
    while step > 1:
        half = step // 2
        # diamond step: centres of squares
        c = (g[0:-1:step, 0:-1:step] + g[0:-1:step, step::step] + g[step::step, 0:-1:step]
             + g[step::step, step::step]) * 0.25
        g[half::step, half::step] = c + amp * rng.standard_normal(c.shape)
        # square step: edge midpoints, averaging the in-grid neighbours
        for r0, c0 in ((0, half), (half, 0)):
            rows = np.arange(r0, size, step)
            cols = np.arange(c0, size, step)
            rr, cc = np.meshgrid(rows, cols, indexing="ij")
            acc = np.zeros(rr.shape)
            cnt = np.zeros(rr.shape)
            for dr, dc in ((-half, 0), (half, 0), (0, -half), (0, half)):
                r2, c2 = rr + dr, cc + dc
                ok = (r2 >= 0) & (r2 < size) & (c2 >= 0) & (c2 < size)
                acc[ok] += g[r2[ok], c2[ok]]
                cnt[ok] += 1
            g[rr, cc] = acc / cnt + amp * rng.standard_normal(rr.shape)
        step = half
        amp *= decay
    return g


def fractal_dem(side: int, seed: int, roughness: float = 0.8, max_height_m: float = 1500.0,
                cell_size_m: float = CELL_SIZE_M, side_y: int | None = None) -> np.ndarray:
    """Diamond-square DEM of ``side_y`` x ``side`` cells, heights in cell units.

    Generated on the next 2^k+1 grid and cropped top-left; heights are rescaled to
    [0, max_height_m] metres and divided by the cell size.
    """
    side_y = side if side_y is None else side_y
    need = max(side, side_y, 2)
    levels = int(np.ceil(np.log2(need - 1))) if need > 2 else 1
    rng = np.random.default_rng(seed)
    g = _diamond_square(levels, roughness, rng)[:side_y, :side]
    lo, hi = g.min(), g.max()
    span = hi - lo if hi > lo else 1.0
    metres = (g - lo) / span * max_height_m
    return (metres / cell_size_m).astype(np.float32)


def ellipse_phantom(side: int, seed: int, n_ellipses: int = 10, side_y: int | None = None) -> np.ndarray:
    """Sum of ``n_ellipses`` random filled ellipses rasterised on [-1, 1]^2.

    Centres uniform in the unit disk, semi-axes uniform in [0.05, 0.4], rotation
    uniform in [0, pi), intensities uniform in [-0.5, 1.0].
    """
    side_y = side if side_y is None else side_y
    rng = np.random.default_rng(seed)
    xs = (np.arange(side) + 0.5) / side * 2.0 - 1.0
    ys = (np.arange(side_y) + 0.5) / side_y * 2.0 - 1.0
    X, Y = np.meshgrid(xs, ys)
    img = np.zeros((side_y, side), dtype=np.float64)
    for _ in range(n_ellipses):
        r = np.sqrt(rng.random())
        phi = rng.random() * 2 * np.pi
        cx, cy = r * np.cos(phi), r * np.sin(phi)
        a, b = rng.uniform(0.05, 0.4, size=2)
        rot = rng.random() * np.pi
        val = rng.uniform(-0.5, 1.0)
        ca, sa = np.cos(rot), np.sin(rot)
        u = (X - cx) * ca + (Y - cy) * sa
        v = -(X - cx) * sa + (Y - cy) * ca
        img[(u / a) ** 2 + (v / b) ** 2 <= 1.0] += val
    return img.astype(np.float32)


def motion_kernel(length: float, angle_deg: float) -> np.ndarray:
    """Normalised linear motion-blur point spread function."""
    half = int(np.ceil(length / 2.0)) + 1
    size = 2 * half + 1
    k = np.zeros((size, size), dtype=np.float64)
    t = np.linspace(-length / 2.0, length / 2.0, max(int(np.ceil(length)) * 4, 2))
    ca, sa = np.cos(np.deg2rad(angle_deg)), np.sin(np.deg2rad(angle_deg))
    xi = np.clip(np.rint(half + t * ca).astype(int), 0, size - 1)
    yi = np.clip(np.rint(half - t * sa).astype(int), 0, size - 1)
    np.add.at(k, (yi, xi), 1.0)
    return k / k.sum()


def blurred_texture(side: int, seed: int, noise_sigma: float = 0.01, side_y: int | None = None,
                    length: float | None = None, angle_deg: float | None = None):
    """1/f^2 spectral-noise texture blurred by a linear motion kernel plus noise.

    Returns ``(image, length_px, angle_deg)``.  The blur length is uniform in
    [5, 40] px and the angle uniform in [0, 180) degrees unless given.
    """
    side_y = side if side_y is None else side_y
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((side_y, side))
    fy = np.fft.fftfreq(side_y)[:, None]
    fx = np.fft.fftfreq(side)[None, :]
    f = np.sqrt(fx * fx + fy * fy)
    f[0, 0] = 1.0
    spec = np.fft.fft2(white) / f  # amplitude 1/f -> power 1/f^2
    spec[0, 0] = 0.0
    tex = np.real(np.fft.ifft2(spec))
    tex = (tex - tex.min()) / max(tex.max() - tex.min(), 1e-12)
    if length is None:
        length = float(rng.uniform(5.0, 40.0))
    if angle_deg is None:
        angle_deg = float(rng.uniform(0.0, 180.0))
    k = motion_kernel(length, angle_deg)
    kp = np.zeros((side_y, side))
    kh, kw = k.shape
    ky, kx = np.meshgrid(np.arange(kh) - kh // 2, np.arange(kw) - kw // 2, indexing="ij")
    np.add.at(kp, (ky % side_y, kx % side), k)  # centred, wrapped (circular convolution)
    blurred = np.real(np.fft.ifft2(np.fft.fft2(tex) * np.fft.fft2(kp)))
    blurred += noise_sigma * rng.standard_normal(blurred.shape)
    return blurred.astype(np.float32), length, angle_deg


def uneven_dem_batch(count: int, base_seed: int, lo: int = 256, hi: int = 2000):
    """Sides uniform in [lo, hi] and roughness uniform in [0.6, 0.9], seed base+i."""
    rng = np.random.default_rng(base_seed)
    sides = rng.integers(lo, hi + 1, size=count)
    rough = rng.uniform(0.6, 0.9, size=count)
    return [(int(s), float(h), base_seed + i) for i, (s, h) in enumerate(zip(sides, rough))]
