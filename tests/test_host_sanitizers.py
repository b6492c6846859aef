"""The library's host code under AddressSanitizer and UBSan.

compute-sanitizer does not run here; the host side of the hot path's inputs is
checked with the compiler's sanitizers instead.  tests/cpp/host_sanitize.cpp is
built with -fsanitize=address,undefined together with the library's own host
sources (the PNG reader and writer, the grid reader and run()'s argument
handling, the sector geometry), and run on seeded damaged PNG files, random
.bil/raw files, headers, sizes and crops, and the tables of every sector of
random grids.  Any sanitizer report fails the run (and the test).  Skipped
where the compiler has no sanitizer runtime.
"""
from __future__ import annotations

import os
import subprocess

import pytest

from tests.conftest import ROOT

CSRC = os.path.join(ROOT, "skewengine_gb300", "csrc")


@pytest.fixture(scope="module")
def sanitized(tmp_path_factory):
    from skewengine_gb300 import build
    exe = str(tmp_path_factory.mktemp("asan") / "host_sanitize")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           "-fno-omit-frame-pointer", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I", CSRC,
           "-I", build.cuda_include(), os.path.join(ROOT, "tests", "cpp", "host_sanitize.cpp"),
           os.path.join(CSRC, "image_io.cpp"), os.path.join(CSRC, "cli.cpp"), os.path.join(CSRC, "geometry.cpp"),
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if "sanitize" in r.stderr or "asan" in r.stderr.lower():
            pytest.skip("no sanitizer runtime for this compiler")
        raise AssertionError(r.stderr[-3000:])
    return exe


def _run(exe, *args):
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=600, env=env)
    assert "AddressSanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-3000:]
    assert r.returncode == 0, r.stdout + r.stderr[-3000:]
    return r.stdout


def test_png_reader_under_sanitizers(sanitized, tmp_path):
    import numpy as np
    from tests.conftest import GOLDEN
    from tests.test_image_io import _mutated_pngs
    images = np.load(os.path.join(GOLDEN, "images.npz"))
    paths = []
    for i, data in enumerate(_mutated_pngs(images, 1500, 91)):
        p = tmp_path / f"m{i:04d}.png"
        p.write_bytes(data)
        paths.append(str(p))
    out = _run(sanitized, "png", *paths)
    assert "png 1500 files" in out


def test_grid_reader_and_run_arguments_under_sanitizers(sanitized, tmp_path):
    out = _run(sanitized, "grid", str(tmp_path))
    assert "grid 3000 cases" in out


def test_sector_geometry_under_sanitizers(sanitized):
    out = _run(sanitized, "geometry")
    assert ", 0 refused" in out
