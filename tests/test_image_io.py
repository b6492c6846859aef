"""Image input/output (host only): PNG decoding against the reference's PNG
library, PNG writing, HSVtoRGB and the result colourings against the
reference's own code (fixtures from tests/golden/make_image_golden.py)."""
from __future__ import annotations

import os

import numpy as np
import pytest

from tests.conftest import GOLDEN, ROOT


@pytest.fixture(scope="module")
def ske():
    from skewengine_gb300 import build
    build.build()
    import skewengine_gb300 as m
    return m


@pytest.fixture(scope="module")
def images():
    return np.load(os.path.join(GOLDEN, "images.npz"))


def test_hsv_to_rgb_matches_reference(ske, images):
    import ctypes as C
    lib = ske.engine.load()
    rgb = (C.c_ubyte * 3)()
    got = np.zeros_like(images["hsv_out"])
    for i, (h, s, v) in enumerate(images["hsv_in"]):
        lib.ske_hsv_to_rgb(C.c_float(h), C.c_float(s), C.c_float(v), rgb)
        got[i] = list(rgb)
    assert np.array_equal(got, images["hsv_out"])


def test_png_decode_matches_reference_library(ske, images, tmp_path):
    meta = images["png_meta"]
    kinds = set()
    for k, (ct, bd, il, w, h) in enumerate(meta):
        path = tmp_path / f"{k}.png"
        path.write_bytes(images[f"png_{k}"].tobytes())
        assert ske.png_size(path) == (w, h)
        assert np.array_equal(ske.read_png_rgba(path), images[f"rgba_{k}"]), (ct, bd, il, w, h)
        kinds.add((int(ct), int(bd), int(il)))
    # every colour type / depth the library writes, plain and interlaced
    assert {(6, 8, 1), (6, 16, 0), (2, 16, 1), (4, 16, 0), (0, 1, 1), (0, 2, 0), (0, 4, 1), (0, 16, 1)} <= kinds


def test_read_image_is_rgb_sum(ske, images, tmp_path):
    k = 3
    path = tmp_path / "img.png"
    path.write_bytes(images[f"png_{k}"].tobytes())
    rgba = images[f"rgba_{k}"].astype(np.int32)
    assert np.array_equal(ske.read_image(path), (rgba[..., 0] + rgba[..., 1] + rgba[..., 2]).astype(np.float32))


@pytest.mark.parametrize("shape", [(1, 1), (5, 9), (300, 257)])
def test_png_write_round_trip(ske, tmp_path, shape):
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    grey = rng.integers(0, 256, shape, dtype=np.uint8)
    rgb = rng.integers(0, 256, shape + (3,), dtype=np.uint8)
    ske.write_png(tmp_path / "g.png", grey)
    ske.write_png(tmp_path / "c.png", rgb)
    g = ske.read_png_rgba(tmp_path / "g.png")
    c = ske.read_png_rgba(tmp_path / "c.png")
    assert np.array_equal(g[..., 0], grey) and np.array_equal(g[..., 2], grey) and (g[..., 3] == 255).all()
    assert np.array_equal(c[..., :3], rgb) and (c[..., 3] == 255).all()


def test_png_rejects_damaged_files(ske, images, tmp_path):
    from skewengine_gb300 import SkeError
    good = images["png_5"].tobytes()
    bad_crc = bytearray(good)
    bad_crc[20] ^= 1  # inside IHDR: its CRC no longer matches
    cases = {"sig": b"\x00" + good[1:], "crc": bytes(bad_crc), "cut": good[: len(good) // 2], "empty": b""}
    for name, data in cases.items():
        p = tmp_path / f"{name}.png"
        p.write_bytes(data)
        with pytest.raises(SkeError, match="not a readable PNG file"):  # the reason reaches ske_last_error
            ske.read_png_rgba(p)
    with pytest.raises(SkeError, match="missing.png"):
        ske.read_png_rgba(tmp_path / "missing.png")


def test_png_decompression_is_bounded_by_the_header(ske, tmp_path):
    """An IDAT that inflates to far more than the header's image needs is refused
    (decompression stops at the expected size)."""
    import struct
    import zlib
    from skewengine_gb300 import SkeError

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xffffffff)

    ihdr = struct.pack(">IIBBBBB", 4, 4, 8, 0, 0, 0, 0)  # 4 x 4 grey: 20 bytes of scanlines
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(b"\0" * 20_000_000)) + \
        chunk(b"IEND", b"")
    (tmp_path / "bomb.png").write_bytes(png)
    with pytest.raises(SkeError):
        ske.read_png_rgba(tmp_path / "bomb.png")
    good = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(b"\0\x07\x07\x07\x07" * 4)) + \
        chunk(b"IEND", b"")
    (tmp_path / "ok.png").write_bytes(good)
    assert (ske.read_png_rgba(tmp_path / "ok.png")[..., 0] == 7).all()


def test_min_max_of_renderer_matches_reference(ske, images):
    """The Radon colouring's scale comes from getMinMax; an all-negative grid
    reports FLT_MIN as its maximum in the reference."""
    for g, n, (lo, hi) in zip(images["minmax_in"], images["minmax_len"], images["minmax_out"]):
        x = g[:n].reshape(1, n)
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):  # all-zero grid: 0 * inf, byte 0 as on x86-64
            esc = np.float32(255) / (np.float32(hi) - np.float32(lo))
            want = ((x - np.float32(lo)).astype(np.int32).astype(np.float32) * esc).astype(np.int32).astype(np.uint8)
        got = ske.render(2, x)
        assert np.array_equal(got[..., 0], want) and np.array_equal(got[..., 1], want)


def test_render_matches_reference_colourings(ske):
    """ske_render against the reference's own result writers run on the same
    outputs (tests/golden/render.npz from make_render_golden.py): the Radon
    grey scale with its automatic range (an all-negative grid included), the
    image identity's 1/540, and the HSV colourings of the cepstrum and the DEM
    identity, pixel for pixel."""
    z = np.load(os.path.join(GOLDEN, "render.npz"))
    n = len([k for k in z.files if k.startswith("alg_")])
    assert n >= 6
    for k in range(n):
        grid, alg = z[f"out_{k}"], int(z[f"alg_{k}"])
        with np.errstate(all="ignore"):
            got = ske.render(alg, grid)
        assert np.array_equal(got, z[f"rgb_{k}"]), (k, alg)


def test_render_colourings(ske, images):
    rng = np.random.default_rng(5)
    out = rng.uniform(0, 2e6, (9, 11)).astype(np.float32)
    # image identity: (int)out * (1/540), truncated to a byte
    ident = ske.render(3, out)
    want = (out.astype(np.int32).astype(np.float32) * np.float32(1.0 / 540)).astype(np.int32).astype(np.uint8)
    assert np.array_equal(ident[..., 0], want)
    # cepstrum: HSV with hue = int(out) mod 360, value min(100, out / 540000)
    import ctypes as C
    lib = ske.engine.load()
    ceps = ske.render(4, out)
    rgb = (C.c_ubyte * 3)()
    for (i, j), v in np.ndenumerate(out):
        val = np.float32(v) / np.float32(540000.0)
        lib.ske_hsv_to_rgb(C.c_float(float(int(v) % 360)), C.c_float(100.0), C.c_float(min(float(val), 100.0)), rgb)
        assert list(ceps[i, j]) == list(rgb)
    from skewengine_gb300 import SkeError
    with pytest.raises(SkeError):
        ske.render(0, out)  # the reference writes no image of a viewshed
    grey = ske.render_input(np.array([[0, 3, 765, 382]], np.float32))
    assert list(grey[0]) == [0, 1, 255, 127]


def _chunks(png: bytes):
    import struct
    i, out = 8, []
    while i + 8 <= len(png):
        n = struct.unpack(">I", png[i:i + 4])[0]
        out.append([png[i + 4:i + 8], bytearray(png[i + 8:i + 8 + n])])
        i += 12 + n
    return out


def _mutated_pngs(images, count: int, seed: int) -> list[bytes]:
    """Seeded damaged variants of the reference-encoded fixtures (every colour
    type and bit depth, plain and interlaced): byte changes inside chunk data
    with the CRC recomputed, so that the damage gets past the checksums to the
    header checks, the inflater and the scanline filters; IHDR fields set to
    extreme values; chunks cut short, dropped or repeated; bytes flipped with
    the CRC left stale."""
    import struct
    import zlib
    rng = np.random.default_rng(seed)
    seeds = [images[f"png_{i}"].tobytes() for i in range(int(images["png_meta"].shape[0]))]
    big = [0, 1, 7, 65535, 1 << 20, 0x7FFFFFFF, 0xFFFFFFFF]
    out = []
    for _ in range(count):
        cs = _chunks(seeds[rng.integers(len(seeds))])
        for _ in range(int(rng.integers(1, 4))):
            kind = int(rng.integers(6))
            c = cs[int(rng.integers(len(cs)))] if cs else None
            if kind == 0 and c is not None and c[1]:
                for _ in range(int(rng.integers(1, 4))):
                    c[1][int(rng.integers(len(c[1])))] = int(rng.integers(256))
            elif kind == 1 and cs and len(cs[0][1]) == 13:
                f = int(rng.integers(7))
                if f < 2:
                    cs[0][1][4 * f:4 * f + 4] = struct.pack(">I", big[int(rng.integers(len(big)))])
                else:
                    cs[0][1][6 + f] = int(rng.choice([0, 1, 2, 3, 4, 6, 8, 16, 255]))
            elif kind == 2 and c is not None:
                c[1] = c[1][: int(rng.integers(len(c[1]) + 1))]
            elif kind == 3 and cs:
                j = int(rng.integers(len(cs)))
                cs.insert(j, [cs[j][0], bytearray(cs[j][1])]) if rng.random() < 0.5 else cs.pop(j)
            elif kind == 4 and c is not None:
                c[1] += rng.integers(0, 256, int(rng.integers(1, 600)), dtype=np.uint8).tobytes()
        data = bytearray(b"\x89PNG\r\n\x1a\n" + b"".join(
            struct.pack(">I", len(d)) + t + bytes(d) + struct.pack(">I", zlib.crc32(t + bytes(d)) & 0xFFFFFFFF)
            for t, d in cs))
        if rng.random() < 0.2:
            for _ in range(int(rng.integers(1, 4))):
                data[int(rng.integers(len(data)))] = int(rng.integers(256))
        out.append(bytes(data))
    return out


def test_png_decoder_survives_mutated_files(ske, images, tmp_path):
    """Two thousand damaged files go through the decoder in a child process (a
    crash fails the test instead of ending the run): each is either refused
    with an error or decoded to exactly the size its header declares, never
    written past its buffer."""
    import subprocess
    import sys
    files = _mutated_pngs(images, 2000, 77)
    for i, data in enumerate(files):
        (tmp_path / f"m{i:04d}.png").write_bytes(data)
    script = (
        "import sys, glob\n"
        "import skewengine_gb300 as s\n"
        "acc = rej = 0\n"
        "for f in sorted(glob.glob(sys.argv[1] + '/m*.png')):\n"
        "    try:\n"
        "        w, h = s.png_size(f)\n"
        "        if w * h > 1 << 24:\n"
        "            rej += 1\n"
        "            continue\n"
        "        px = s.read_png_rgba(f)\n"
        "        img = s.read_image(f)\n"
        "        assert px.shape == (h, w, 4) and img.shape == (h, w)\n"
        "        acc += 1\n"
        "    except s.SkeError:\n"
        "        rej += 1\n"
        "print(acc, rej)\n")
    r = subprocess.run([sys.executable, "-c", script, str(tmp_path)], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    acc, rej = (int(v) for v in r.stdout.split())
    print(f"{acc} decoded, {rej} refused")
    assert acc + rej == len(files) and acc > 0 and rej > 0, (acc, rej)


def test_png_header_alone_sizes_nothing(ske, tmp_path):
    """A file whose header claims a huge image is refused by png_size beyond
    the decoder's 2^31-pixel limit, and below it the CLI decodes before it
    allocates the grid: a damaged 1.6e9-pixel claim with a few bytes of data
    is refused without the gigabytes its header asks for."""
    import struct
    import subprocess
    import sys
    import zlib
    from skewengine_gb300 import SkeError

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xffffffff)

    def png(w, h):
        return b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 0, 0, 0, 0)) + \
            chunk(b"IDAT", zlib.compress(b"\0" * 64)) + chunk(b"IEND", b"")

    (tmp_path / "huge.png").write_bytes(png(65536, 65536))
    with pytest.raises(SkeError):
        ske.png_size(tmp_path / "huge.png")
    (tmp_path / "claim.png").write_bytes(png(40000, 40000))
    assert ske.png_size(tmp_path / "claim.png") == (40000, 40000)
    script = ("import resource, sys\n"
              "import skewengine_gb300 as s\n"
              "rc = s.cli_run(['radon', sys.argv[1], 0, 0, sys.argv[2]])\n"
              "print(rc, resource.getrusage(resource.RUSAGE_SELF).ru_maxrss)\n")
    r = subprocess.run([sys.executable, "-c", script, str(tmp_path / "claim.png"), str(tmp_path / "o.png")],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    rc, peak_kb = (int(v) for v in r.stdout.split()[-2:])
    assert rc == 1 and peak_kb < 2 << 20, (rc, peak_kb)  # refused, under 2 GB at its peak


@pytest.mark.gpu
def test_cli_png_in_png_out(ske, tmp_path):
    """run(argc, argv) with an image input and an image output: the engine runs on
    the R + G + B grid, the result is written coloured, the input in grey."""
    from skewengine_gb300 import synthetic
    x = synthetic.ellipse_phantom(64, 3)
    px = np.clip((x - x.min()) / (x.max() - x.min()) * 255, 0, 255).astype(np.uint8)
    ske.write_png(tmp_path / "in.png", np.stack([px, px, px], axis=2))
    img = ske.read_image(tmp_path / "in.png")
    assert ske.cli_run(["radon", str(tmp_path / "in.png"), 0, 0, str(tmp_path / "out.png")]) == 0
    with ske.SkewEngine(64, 64) as eng:
        want = eng.run(2, img)
    assert np.array_equal(ske.read_png_rgba(tmp_path / "out.png")[..., :3], ske.render(2, want))
    assert np.array_equal(ske.read_png_rgba(tmp_path / "out_input.png")[..., 0], ske.render_input(img))
