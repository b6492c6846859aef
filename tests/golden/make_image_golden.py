"""Generate the image input/output fixtures from the reference's own code.

Run where the reference sources are present (it builds ``oracle/_ref`` from them
through ``oracle/Makefile``)::

    python tests/golden/make_image_golden.py --ref /path/to/skewEngine

Output ``images.npz`` in this folder:

* ``hsv_in`` (k x 3 float32 H, S, V) and ``hsv_out`` (k x 3 uint8): the
  reference's HSVtoRGB (src/color.cpp:80-115) over a grid of hues, saturations
  and values, including out-of-range ones;
* ``minmax_in`` / ``minmax_out``: helper::getMinMax (src/helper.h:190-201) of a
  few grids, including an all-negative one;
* ``png_<i>`` (uint8 file bytes), ``rgba_<i>`` (uint8 RGBA) and ``png_meta``
  (colour type, bit depth, interlace, width, height per file): small images
  encoded by the reference's vendored PNG library (src/third-party/Lodepng.cpp)
  in every colour type and bit depth it writes, plain and Adam7-interlaced, and
  the RGBA that library decodes from each file, which is what read_png
  (src/helper.h:167-184) starts from.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def build_ref(ref: str) -> C.CDLL:
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref}"], check=True,
                   stdout=subprocess.DEVNULL)
    return C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libskewref.so"))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="reference project root")
    args = ap.parse_args()
    lib = build_ref(args.ref)
    rng = np.random.default_rng(20240)
    out: dict[str, np.ndarray] = {}

    hues = np.concatenate([np.arange(-2, 363, 0.5), rng.uniform(-5, 365, 600)]).astype(np.float32)
    sv = [(100, 100), (100, 50), (50, 80), (100, 0.37), (100, 1e-3), (0, 50), (100, 120), (-1, 50), (100, 100.5)]
    hsv_in = np.array([(h, s, v) for h in hues for s, v in sv], np.float32)
    hsv_out = np.zeros((len(hsv_in), 3), np.uint8)
    rgb = (C.c_ubyte * 3)()
    for i, (h, s, v) in enumerate(hsv_in):
        lib.skref_hsv_to_rgb(C.c_float(h), C.c_float(s), C.c_float(v), rgb)
        hsv_out[i] = list(rgb)
    out["hsv_in"], out["hsv_out"] = hsv_in, hsv_out

    grids = [rng.normal(0, 50, 97).astype(np.float32), -rng.uniform(1, 9, 40).astype(np.float32),
             np.zeros(5, np.float32), rng.uniform(0, 1e6, 64).astype(np.float32)]
    mm_in = np.zeros((len(grids), 97), np.float32)
    mm_len = np.array([len(g) for g in grids], np.int32)
    mm_out = np.zeros((len(grids), 2), np.float32)
    for i, g in enumerate(grids):
        mm_in[i, :len(g)] = g
        lo, hi = C.c_float(), C.c_float()
        lib.skref_min_max(g.ctypes.data_as(C.c_void_p), len(g), C.byref(lo), C.byref(hi))
        mm_out[i] = (lo.value, hi.value)
    out["minmax_in"], out["minmax_len"], out["minmax_out"] = mm_in, mm_len, mm_out

    meta = []
    tmp = tempfile.mkdtemp()
    path = os.path.join(tmp, "img.png")
    k = 0
    for h, w in [(1, 1), (7, 13), (21, 17)]:
        rgba = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
        grey = np.repeat(rng.integers(0, 256, (h, w, 1), dtype=np.uint8), 4, axis=2)
        grey[..., 3] = 255
        cases = [(6, 8, rgba), (6, 16, rgba), (2, 8, rgba), (2, 16, rgba), (4, 8, grey), (4, 16, grey),
                 (0, 8, grey), (0, 16, grey), (0, 1, grey), (0, 2, grey), (0, 4, grey)]
        few = rng.integers(0, 256, (5, 4), dtype=np.uint8)
        cases.append((-1, 0, few[rng.integers(0, 5, (h, w))]))  # the library's choice: a palette
        for ct, bd, img in cases:
            for il in (0, 1):
                im = img.copy()
                if ct == 0 and bd < 8:  # values the low bit depth holds exactly
                    q = im[..., 0] >> (8 - bd)
                    im[..., 0] = im[..., 1] = im[..., 2] = (q * 255 // ((1 << bd) - 1)).astype(np.uint8)
                im = np.ascontiguousarray(im)
                ptr = im.ctypes.data_as(C.c_void_p)
                if ct >= 0:
                    rc = lib.skref_png_encode(path.encode(), ptr, w, h, ct, bd, il)
                else:
                    rc = lib.skref_png_encode_auto(path.encode(), ptr, w, h, il)
                if rc:
                    raise RuntimeError(f"encode failed: {rc} {(h, w, ct, bd, il)}")
                dec = np.zeros(h * w * 4, np.uint8)
                W, H = C.c_uint(), C.c_uint()
                if lib.skref_png_decode(path.encode(), dec.ctypes.data_as(C.c_void_p), dec.size, C.byref(W),
                                        C.byref(H)):
                    raise RuntimeError("decode failed")
                with open(path, "rb") as f:
                    out[f"png_{k}"] = np.frombuffer(f.read(), np.uint8)
                out[f"rgba_{k}"] = dec.reshape(h, w, 4)
                meta.append((ct, bd, il, w, h))
                k += 1
    out["png_meta"] = np.array(meta, np.int32)
    np.savez_compressed(os.path.join(HERE, "images.npz"), **out)
    print(f"wrote images.npz: {len(hsv_in)} HSV cases, {k} PNG files")


if __name__ == "__main__":
    main()
