"""Generate the golden fixtures from the reference's own CPU code.

Run where the reference sources are present (it builds ``oracle/_ref`` from them
through ``oracle/Makefile``)::

    python tests/golden/make_golden.py --ref /path/to/skewEngine

Outputs, all in this folder:

* ``runs.npz``      whole-run inputs/outputs (single thread, 180 sectors) for every
                    operator on small square and non-square grids;
* ``sectors.npz``   per-sector intermediates (geometry, skewed input, operator
                    output, deskewed contribution) for selected angles;
* ``geometry.npz``  full per-angle geometry tables for small grids;
* ``geometry_digest.json``  SHA-256 of the per-angle geometry of the benchmark
                    grid sizes (too large to store whole).
"""
from __future__ import annotations

import argparse
import ctypes as C
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from skewengine_gb300 import synthetic  # noqa: E402

OPS = {"sdem": 0, "identitydem": 1, "radon": 2, "identityimg": 3, "cepstrum": 4, "localradon": 5}
# The reference has no operator id for the local Radon transform: it is its Radon
# operator (2) with the LRT switch set (kernelRADN.h:212-220).
LOCAL_RADON = 5
POVH = float(synthetic.POVH)


def load_ref(ref_root: str):
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref_root}"], check=True)
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libskewref.so"))
    fp = np.ctypeslib.ndpointer(np.float32, flags="C")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C")
    dp = np.ctypeslib.ndpointer(np.float64, flags="C")
    up = np.ctypeslib.ndpointer(np.uint16, flags="C")
    lib.skref_run.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int]
    lib.skref_sector.argtypes = [C.c_int, fp, C.c_int, C.c_int, C.c_int, C.c_float, ip, dp, fp, fp,
                                 up, up, ip, fp, fp]
    lib.skref_set_local_radon.argtypes = [C.c_int]
    return lib


def ref_op(lib, op: int) -> int:
    """Reference operator id for `op`, setting the LRT switch for the local Radon."""
    lib.skref_set_local_radon(1 if op == LOCAL_RADON else 0)
    return 2 if op == LOCAL_RADON else op


def input_for(kind: str, dx: int, dy: int, seed: int) -> np.ndarray:
    if kind == "fractal":
        return synthetic.fractal_dem(dx, seed, side_y=dy)
    if kind == "phantom":
        return synthetic.ellipse_phantom(dx, seed, side_y=dy)
    if kind == "texture":
        return synthetic.blurred_texture(dx, seed, side_y=dy)[0]
    if kind == "uniform":
        return (np.random.default_rng(seed).random((dy, dx)) * 150).astype(np.float32)
    raise ValueError(kind)


# (operator, input kind, dimx, dimy, seed)
RUN_CASES = [
    ("sdem", "fractal", 32, 32, 11), ("sdem", "fractal", 64, 64, 12), ("sdem", "fractal", 33, 33, 13),
    ("sdem", "uniform", 16, 16, 14), ("sdem", "fractal", 48, 32, 15), ("sdem", "fractal", 32, 48, 16),
    ("sdem", "uniform", 1, 1, 17), ("sdem", "uniform", 3, 2, 18), ("sdem", "fractal", 7, 7, 19),
    ("identitydem", "fractal", 32, 32, 21), ("identitydem", "uniform", 48, 32, 22),
    ("identitydem", "uniform", 5, 17, 23),
    ("identityimg", "texture", 40, 40, 31),
    ("radon", "phantom", 64, 64, 41), ("radon", "phantom", 64, 48, 42), ("radon", "phantom", 33, 33, 43),
    ("radon", "uniform", 2, 2, 44),
    ("cepstrum", "texture", 32, 32, 51), ("cepstrum", "texture", 40, 24, 52),
    ("cepstrum", "texture", 24, 40, 53),
    ("localradon", "phantom", 32, 32, 61), ("localradon", "phantom", 40, 24, 62),
    ("localradon", "texture", 24, 36, 63),
]

SECTOR_CASES = [
    ("sdem", "fractal", 32, 32, 11, [0, 1, 17, 44, 45, 46, 89, 90, 91, 120, 134, 135, 179]),
    ("identitydem", "uniform", 48, 32, 22, [0, 20, 33, 34, 60, 90, 100, 146, 147, 170]),
    ("radon", "phantom", 64, 64, 41, [0, 30, 45, 90, 135]),
    ("cepstrum", "texture", 32, 32, 51, [0, 45, 100]),
    ("localradon", "phantom", 32, 32, 61, [0, 45, 100, 160]),
]

GEOMETRY_SMALL = [(32, 32), (48, 32), (32, 48), (7, 5), (1, 1), (3, 2)]
GEOMETRY_DIGEST = [(500, 500), (512, 512), (2000, 2000), (256, 256), (1000, 700), (64, 64)]


def sector_dump(lib, op: int, x: np.ndarray, angle: int):
    dy, dx = x.shape
    n, dl = dx * dy, max(dx, dy)
    ii = np.zeros(7, np.int32)
    dd = np.zeros(2, np.float64)
    si = np.zeros(2 * n + dl, np.float32)
    so = np.zeros(2 * n + dl, np.float32)
    fi = np.zeros(2 * dl + 1, np.uint16)
    la = np.zeros(2 * dl + 1, np.uint16)
    ta = np.zeros(dl, np.int32)
    we = np.zeros(dl, np.float32)
    acc = np.zeros(n, np.float32)
    assert lib.skref_sector(ref_op(lib, op), np.ascontiguousarray(x), dx, dy, angle, POVH, ii, dd, si, so, fi,
                            la, ta, we, acc) == 0
    h = int(ii[5])
    return ii, dd, si, so, fi[:h].copy(), la[:h].copy(), ta, we, acc


def geometry_digest(lib, dx: int, dy: int) -> list[str]:
    x = np.zeros((dy, dx), np.float32)
    out = []
    for a in range(180):
        ii, dd, _, _, fi, la, ta, we, _ = sector_dump(lib, 1, x, a)
        di = int(ii[2])
        h = hashlib.sha256()
        for arr in (ii, dd, fi, la, ta[:di], we[:di]):
            h.update(np.ascontiguousarray(arr).tobytes())
        out.append(h.hexdigest())
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="reference project root")
    args = ap.parse_args()
    lib = load_ref(args.ref)

    runs = {}
    for name, kind, dx, dy, seed in RUN_CASES:
        x = input_for(kind, dx, dy, seed)
        y = np.zeros_like(x)
        assert lib.skref_run(ref_op(lib, OPS[name]), x, y, dx, dy, 180, POVH, 1) == 0
        key = f"{name}__{kind}__{dx}x{dy}__{seed}"
        runs[key + "__in"] = x
        runs[key + "__out"] = y
        print("run", key, float(y.min()), float(y.max()))
    np.savez_compressed(os.path.join(HERE, "runs.npz"), **runs)

    sectors = {}
    for name, kind, dx, dy, seed, angles in SECTOR_CASES:
        x = input_for(kind, dx, dy, seed)
        base = f"{name}__{kind}__{dx}x{dy}__{seed}"
        sectors[base + "__in"] = x
        for a in angles:
            ii, dd, si, so, fi, la, ta, we, acc = sector_dump(lib, OPS[name], x, a)
            k = f"{base}__a{a}"
            for suffix, arr in (("iinfo", ii), ("dinfo", dd), ("skew_in", si), ("skew_out", so),
                                ("first", fi), ("last", la), ("target", ta), ("weight", we), ("acc", acc)):
                sectors[f"{k}__{suffix}"] = arr
        print("sectors", base, angles)
    np.savez_compressed(os.path.join(HERE, "sectors.npz"), **sectors)

    # Per grid: iinfo [180,7], dinfo [180,2]; first/last concatenated over angles
    # (skewHeight entries each), target/weight concatenated (dim_i entries each).
    geo = {}
    for dx, dy in GEOMETRY_SMALL:
        x = np.zeros((dy, dx), np.float32)
        parts = {"iinfo": [], "dinfo": [], "first": [], "last": [], "target": [], "weight": []}
        for a in range(180):
            ii, dd, _, _, fi, la, ta, we, _ = sector_dump(lib, 1, x, a)
            di = int(ii[2])
            for name, arr in (("iinfo", ii), ("dinfo", dd), ("first", fi), ("last", la),
                              ("target", ta[:di]), ("weight", we[:di])):
                parts[name].append(np.array(arr))
        k = f"{dx}x{dy}"
        geo[k + "__iinfo"] = np.stack(parts["iinfo"])
        geo[k + "__dinfo"] = np.stack(parts["dinfo"])
        for name in ("first", "last", "target", "weight"):
            geo[k + "__" + name] = np.concatenate(parts[name])
    np.savez_compressed(os.path.join(HERE, "geometry.npz"), **geo)

    digest = {f"{dx}x{dy}": geometry_digest(lib, dx, dy) for dx, dy in GEOMETRY_DIGEST}
    with open(os.path.join(HERE, "geometry_digest.json"), "w") as f:
        json.dump(digest, f, indent=0)
    print("done")


if __name__ == "__main__":
    main()
