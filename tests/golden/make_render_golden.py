"""Generate the result-colouring fixtures from the reference's own code.

Run where the reference sources are present (it builds ``oracle/_ref`` from them
through ``oracle/Makefile``)::

    python tests/golden/make_render_golden.py --ref /path/to/skewEngine

Output ``render.npz`` in this folder: for each case ``<k>`` an operator output
grid (``out_<k>``, float32), its operator id (``alg_<k>``) and the RGB image
the reference writes for it (``rgb_<k>``): showResultsRADN with the scale and
shift showResults picks (src/kernelRADN.h:384-400, src/main.h:124-141) for the
Radon operator (2) and the image identity (3), showResultsCEPS
(src/kernelBLUR.h:396-410) for the DEM identity (1) and the cepstrum (4),
decoded from the salida2.png it writes (oracle/ref_harness.cu, skref_render).
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


def cases(rng):
    yield 2, rng.normal(0, 50, (13, 17))
    yield 2, -rng.uniform(1, 9, (9, 31))  # all negative: getMinMax reports FLT_MIN as the maximum
    yield 3, rng.uniform(0, 2e6, (13, 17))
    yield 4, rng.integers(0, 180, (13, 17)) + 1000.0 * rng.integers(0, 900, (13, 17))
    yield 4, rng.integers(0, 180, (9, 31)) + 1000.0 * rng.integers(0, 40, (9, 31))
    yield 1, rng.uniform(0, 4e5, (13, 17))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="reference project root")
    args = ap.parse_args()
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.ref}"], check=True,
                   stdout=subprocess.DEVNULL)
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libskewref.so"))
    lib.skref_render.argtypes = [C.c_int, np.ctypeslib.ndpointer(np.float32, flags="C"), C.c_int, C.c_int,
                                 C.c_char_p, np.ctypeslib.ndpointer(np.uint8, flags="C")]
    out: dict[str, np.ndarray] = {}
    for k, (alg, grid) in enumerate(cases(np.random.default_rng(777))):
        grid = np.ascontiguousarray(grid, np.float32)
        rgb = np.zeros(grid.shape + (3,), np.uint8)
        with tempfile.TemporaryDirectory() as d:
            assert lib.skref_render(alg, grid, grid.shape[1], grid.shape[0], d.encode(), rgb) == 0
        out[f"out_{k}"], out[f"alg_{k}"], out[f"rgb_{k}"] = grid, np.array(alg, np.int32), rgb
    np.savez_compressed(os.path.join(HERE, "render.npz"), **out)
    print("wrote", os.path.join(HERE, "render.npz"))


if __name__ == "__main__":
    main()
