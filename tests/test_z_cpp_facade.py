"""The C++ facade (include/skewengine.hpp): the reference's skewEngine<float>
class and execute() driver (src/skewEngine.cuh:141-372, src/main.cu:71-172)
over the C ABI, for C++ callers of that class.

tests/cpp/facade_check.cpp is compiled against the header and
libskewengine.so.  Without a device it checks the operator ids, the host
geometry (compared here with the C ABI through ctypes) and the refusals of a
CPU engine and of a missing device; the GPU test runs the reference's
per-sector loop through the class against execute() and a kernelcuda
operator's arguments.
"""
from __future__ import annotations

import os
import subprocess

import pytest

from tests.conftest import ROOT


@pytest.fixture(scope="module")
def facade(tmp_path_factory):
    from skewengine_gb300 import build
    lib = build.build()
    exe = str(tmp_path_factory.mktemp("facade") / "facade_check")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_check.cpp"), "-L", libdir, "-lskewengine",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    return exe


def test_facade_host_geometry_and_refusals(facade):
    import skewengine_gb300 as ske
    r = subprocess.run([facade, "host"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("geom ")]
    assert len(lines) == 40
    for f in lines:
        dx, dy, a = int(f[1]), int(f[2]), int(f[3])
        g = ske.geometry(dx, dy, a)
        want = [g["sector_type"], g["new_angle"], g["dim_i"], g["dim_o"], g["offset"], g["skew_height"],
                g["dim_l"]]
        assert [int(v) for v in f[4:11]] == want, (dx, dy, a)
        assert float(f[11]) == g["scale"]
        assert [int(v) for v in f[12:15]] == [int(g["first"].sum()), int(g["last"].sum()), int(g["target"].sum())]
        w = 0.0
        for v in g["weight"]:  # summed in order in binary64, as the program does
            w += float(v)
        assert float(f[15]) == w


@pytest.mark.gpu
def test_facade_per_sector_loop_equals_execute(facade):
    r = subprocess.run([facade, "gpu"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "facade checks passed" in r.stdout
