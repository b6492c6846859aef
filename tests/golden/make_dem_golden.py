"""Generate the DEM-reader fixtures from the reference's own code.

Run where the reference sources are present (it builds ``oracle/_ref`` from them
through ``oracle/Makefile``)::

    python tests/golden/make_dem_golden.py --ref /path/to/skewEngine

Output ``dem_io.npz`` in this folder: for each case ``<k>``, the int16 cells of
a .bil file (``bil_<k>``, file_dx x file_dy, little-endian), the file's size
and crop (``meta_<k>`` = file_dx, file_dy, crop_x, crop_y) and the float grid
the reference's readBilData (src/kernelSDEM.h:31-52) builds from it with that
crop (``grid_<k>``).
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

CASES = [(37, 29, 0, 0), (37, 29, 5, 0), (37, 29, 0, 7), (40, 32, 11, 3), (16, 48, 15, 47)]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="reference project root")
    args = ap.parse_args()
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.ref}"], check=True,
                   stdout=subprocess.DEVNULL)
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libskewref.so"))
    lib.skref_read_bil.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                   np.ctypeslib.ndpointer(np.float32, flags="C")]
    rng = np.random.default_rng(4242)
    out: dict[str, np.ndarray] = {}
    with tempfile.TemporaryDirectory() as tmp:
        for k, (fdx, fdy, cx, cy) in enumerate(CASES):
            # Metres of relief, negative heights and the int16 extremes.
            cells = rng.integers(-500, 9000, size=(fdy, fdx)).astype("<i2")
            cells.flat[::97] = 32767
            cells.flat[5::131] = -32768
            path = os.path.join(tmp, f"dem{k}.bil")
            cells.tofile(path)
            grid = np.zeros((fdy - cy, fdx - cx), np.float32)
            assert lib.skref_read_bil(path.encode(), fdx, fdy, cx, cy, grid) == 0
            out[f"bil_{k}"] = cells
            out[f"meta_{k}"] = np.array([fdx, fdy, cx, cy], np.int32)
            out[f"grid_{k}"] = grid
    np.savez_compressed(os.path.join(HERE, "dem_io.npz"), **out)
    print("wrote", os.path.join(HERE, "dem_io.npz"))


if __name__ == "__main__":
    main()
