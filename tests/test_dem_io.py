"""DEM file input and output of run(argc, argv) and ske_read_grid: the ESRI .bil
int16 grid with its .hdr and crop (readBilData / parse_hdr / check_dem,
src/kernelSDEM.h:31-142) and the raw float32 .flt result dump (showResultsSDEM,
src/kernelSDEM.h:433-439).

The reference reads a .bil as little-endian int16 metres, row after row, and
divides each value by 10 in binary64 before storing it as float (cell units of
a 10 m grid, kernelSDEM.h:43-50).  Without a header the grid is square with the
side taken from the file size (check_dem, :132-135).  The GPU tests write such
files, run the total viewshed through run(), and compare the .flt bit for bit
with the oracle on the same divided grid.
"""
from __future__ import annotations

import numpy as np
import pytest

from skewengine_gb300 import synthetic


def _bil_grid(raw: np.ndarray) -> np.ndarray:
    """The float grid readBilData makes of int16 metres: (float)((float)v / 10.0)."""
    return (raw.astype(np.float32).astype(np.float64) / 10.0).astype(np.float32)


def _fractal_int16(side_x: int, side_y: int, seed: int) -> np.ndarray:
    # Heights in metres (0-1500 m, the fractal DEM of the benchmark configs).
    m = synthetic.fractal_dem(side_x, seed, side_y=side_y) * np.float32(synthetic.CELL_SIZE_M)
    return np.round(m).astype("<i2")


def _write_hdr(path, ncols, nrows):
    path.write_text(f"BYTEORDER      I\nLAYOUT         BIL\nNROWS         {nrows}\nNCOLS         {ncols}\n"
                    f"NBANDS        1\nNBITS         16\nCELLSIZE      10\nXLLCORNER     310000\n"
                    f"YLLCORNER     4070000\n")


def test_bil_reader_rejects_short_files(tmp_path):
    """A .bil with fewer bytes than its header's grid is refused before any
    device work (so this runs without a GPU)."""
    from skewengine_gb300 import cli_run
    raw = np.zeros((10, 12), "<i2")
    (tmp_path / "dem.bil").write_bytes(raw.tobytes())
    _write_hdr(tmp_path / "dem.hdr", 40, 40)
    assert cli_run(["sdem", str(tmp_path / "dem.bil"), 0, 0, str(tmp_path / "out.flt")]) == 1


def test_read_grid_bil_header_and_crop(tmp_path):
    """ske_read_grid reads a .bil as readBilData does (int16 metres / 10 in
    binary64), its size from the .hdr, and crops the top-left window at the
    file's row pitch (readBilData's crop_x/crop_y, src/kernelSDEM.h:31-52).
    Host only."""
    from skewengine_gb300 import read_grid
    raw = _fractal_int16(80, 56, 401)
    (tmp_path / "dem.bil").write_bytes(raw.tobytes())
    _write_hdr(tmp_path / "dem.hdr", 80, 56)
    want = _bil_grid(raw)
    got = read_grid(tmp_path / "dem.bil")
    assert got.shape == (56, 80) and np.array_equal(got.view(np.uint32), want.view(np.uint32))
    got = read_grid(tmp_path / "dem.bil", crop_x=7, crop_y=5)
    assert got.shape == (51, 73) and np.array_equal(got.view(np.uint32), want[:51, :73].view(np.uint32))
    # Explicit dims override the header; the crop applies to them.
    got = read_grid(tmp_path / "dem.bil", 80, 40, crop_x=30)
    assert np.array_equal(got.view(np.uint32), want[:40, :50].view(np.uint32))
    # The window's rows alone need be present, as readBilData reads them.
    cut = raw.tobytes()[: (50 * 80 + 73) * 2]
    (tmp_path / "cut.bil").write_bytes(cut)
    got = read_grid(tmp_path / "cut.bil", 80, 56, crop_x=7, crop_y=5)
    assert np.array_equal(got.view(np.uint32), want[:51, :73].view(np.uint32))


def test_read_grid_matches_reference_reader(tmp_path):
    """ske_read_grid against the reference's own readBilData run on the same
    files (tests/golden/dem_io.npz, made by make_dem_golden.py from the
    reference's sources): full reads and crops in x, y and both, int16 extremes
    and negative heights, bit for bit."""
    import os
    from skewengine_gb300 import read_grid
    from tests.conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, "dem_io.npz"))
    cases = sorted(int(k[5:]) for k in z.files if k.startswith("meta_"))
    assert len(cases) >= 5
    for k in cases:
        fdx, fdy, cx, cy = (int(v) for v in z[f"meta_{k}"])
        (tmp_path / f"d{k}.bil").write_bytes(z[f"bil_{k}"].astype("<i2").tobytes())
        got = read_grid(tmp_path / f"d{k}.bil", fdx, fdy, crop_x=cx, crop_y=cy)
        want = z[f"grid_{k}"]
        assert got.shape == want.shape and np.array_equal(got.view(np.uint32), want.view(np.uint32)), k


def test_read_grid_raw_square_png_and_refusals(tmp_path):
    import skewengine_gb300 as ske
    from skewengine_gb300 import SkeError
    x = synthetic.fractal_dem(33, 402)
    x.tofile(tmp_path / "g.raw")
    got = ske.read_grid(tmp_path / "g.raw")  # square from the file size
    assert np.array_equal(got.view(np.uint32), x.view(np.uint32))
    got = ske.read_grid(tmp_path / "g.raw", 33, 33, crop_x=1, crop_y=32)
    assert np.array_equal(got.view(np.uint32), x[:1, :32].view(np.uint32))
    px = (np.arange(20 * 14 * 3) % 251).astype(np.uint8).reshape(14, 20, 3)
    ske.write_png(tmp_path / "i.png", px)
    img = ske.read_image(tmp_path / "i.png")
    got = ske.read_grid(tmp_path / "i.png", crop_x=3, crop_y=2)
    assert np.array_equal(got, img[:12, :17])
    for args in [dict(crop_x=33), dict(crop_y=40), dict(crop_x=-1), dict(dimx=40, dimy=40)]:
        with pytest.raises(SkeError):
            ske.read_grid(tmp_path / "g.raw", **args)
    with pytest.raises(SkeError, match="need"):  # the reason reaches ske_last_error
        ske.read_grid(tmp_path / "g.raw", 40, 40)
    with pytest.raises(SkeError, match="cannot open"):
        ske.read_grid(tmp_path / "missing.bil")
    with pytest.raises(SkeError):
        ske.read_grid(tmp_path / "i.png", 21, 14)  # not the image's size


@pytest.mark.gpu
def test_bil_square_without_header(gpu_lib, oracle, tmp_path):
    """No .hdr: the side comes from the file size, as check_dem does."""
    from skewengine_gb300 import cli_run
    raw = _fractal_int16(96, 96, 311)
    (tmp_path / "dem.bil").write_bytes(raw.tobytes())
    assert cli_run(["sdem", str(tmp_path / "dem.bil"), 0, 0, str(tmp_path / "out.flt")]) == 0
    got = np.fromfile(tmp_path / "out.flt", "<f4").reshape(96, 96)
    want = oracle.run(0, _bil_grid(raw), povh=synthetic.POVH)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.gpu
def test_bil_with_esri_header_non_square(gpu_lib, oracle, tmp_path):
    """An ESRI header's NCOLS/NROWS give a non-square grid (dimx/dimy 0)."""
    from skewengine_gb300 import cli_run
    raw = _fractal_int16(80, 56, 312)  # 56 rows of 80 columns
    (tmp_path / "dem.bil").write_bytes(raw.tobytes())
    _write_hdr(tmp_path / "dem.hdr", 80, 56)
    assert cli_run(["sdem", str(tmp_path / "dem.bil"), 0, 0, str(tmp_path / "out.flt"), 180, 0.15]) == 0
    got = np.fromfile(tmp_path / "out.flt", "<f4")
    assert got.size == 80 * 56
    want = oracle.run(0, _bil_grid(raw), povh=np.float32(0.15))
    assert np.array_equal(got.reshape(56, 80).view(np.uint32), want.view(np.uint32))


@pytest.mark.gpu
def test_bil_explicit_dims_and_angle_count(gpu_lib, oracle, tmp_path):
    """Explicit dimx/dimy take precedence over the header; max_sector limits the
    angles 0..max_sector-1; the division by 10 reaches negative and large values."""
    from skewengine_gb300 import cli_run
    rng = np.random.default_rng(313)
    raw = rng.integers(-400, 8000, size=(48, 64)).astype("<i2")
    (tmp_path / "dem.bil").write_bytes(raw.tobytes())
    _write_hdr(tmp_path / "dem.hdr", 10, 10)  # ignored: dims given
    assert cli_run(["sdem", str(tmp_path / "dem.bil"), 64, 48, str(tmp_path / "out.flt"), 45]) == 0
    got = np.fromfile(tmp_path / "out.flt", "<f4").reshape(48, 64)
    want = oracle.run(0, _bil_grid(raw), nsect=45, povh=np.float32(0.15))
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
