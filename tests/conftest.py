"""Shared fixtures.

Markers: ``gpu`` tests need a CUDA device and call the engine through its C ABI;
everything else runs on a CPU-only machine (oracle vs golden fixtures, host
geometry, ABI surface, host-side sharding with gloo ranks).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _build_port() -> str:
    path = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return path


@pytest.fixture(scope="session")
def port():
    """The CPU restatement oracle (oracle/skewport.cpp), used only as a checker."""
    lib = C.CDLL(_build_port())
    fp = np.ctypeslib.ndpointer(np.float32, flags="C")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C")
    dp = np.ctypeslib.ndpointer(np.float64, flags="C")
    up = np.ctypeslib.ndpointer(np.uint16, flags="C")
    lib.port_run.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int]
    lib.port_run_angles.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, ip, C.c_int, C.c_float, C.c_int]
    lib.port_run_angles_ordered.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, ip, C.c_int, C.c_float, C.c_int]
    lib.port_sector.argtypes = [C.c_int, fp, C.c_int, C.c_int, C.c_int, C.c_float, fp, fp, fp]
    lib.port_geometry.argtypes = [C.c_int, C.c_int, C.c_int, ip, dp, up, up, ip, fp]
    lib.port_sdem_counts.argtypes = [fp, C.c_int, C.c_int, C.c_int, C.c_float, fp]
    lib.port_los_steps.argtypes = [C.c_int, C.c_int, C.c_int]
    lib.port_los_steps.restype = C.c_double
    lib.port_accumulate.argtypes = [C.c_int, fp, C.c_int, C.c_int, ip, C.c_int, C.c_float, fp, ip]
    lib.port_run_f64.argtypes = [C.c_int, fp, dp, C.c_int, C.c_int, C.c_int, C.c_float]
    return lib


class PortOracle:
    def __init__(self, lib):
        self.lib = lib

    def run(self, op, x, nsect=180, povh=0.15, threads=1):
        dy, dx = x.shape
        out = np.zeros_like(x)
        assert self.lib.port_run(op, np.ascontiguousarray(x, np.float32), out, dx, dy, nsect, povh, threads) == 0
        return out

    def run_f64(self, op, x, nsect=180, povh=0.15):
        """The same run carried out in binary64 throughout (error reference)."""
        dy, dx = x.shape
        out = np.zeros(x.shape, np.float64)
        assert self.lib.port_run_f64(op, np.ascontiguousarray(x, np.float32), out, dx, dy, nsect, povh) == 0
        return out

    def run_angles(self, op, x, angles, povh=0.15, threads=1):
        dy, dx = x.shape
        out = np.zeros_like(x)
        a = np.ascontiguousarray(angles, np.int32)
        assert self.lib.port_run_angles(op, np.ascontiguousarray(x, np.float32), out, dx, dy, a, len(a), povh,
                                        threads) == 0
        return out

    def run_ordered(self, op, x, angles=None, povh=0.15, threads=None):
        """The single-thread result (reference accumulation order) computed on
        all host cores: sectors in parallel, folded in list order."""
        dy, dx = x.shape
        out = np.zeros_like(x)
        a = np.ascontiguousarray(range(180) if angles is None else angles, np.int32)
        nt = threads or os.cpu_count() or 1
        assert self.lib.port_run_angles_ordered(op, np.ascontiguousarray(x, np.float32), out, dx, dy, a, len(a),
                                                povh, nt) == 0
        return out

    def counts_many(self, x, angles, povh=0.15, threads=None):
        """port_sdem_counts of several sectors, one host thread per sector."""
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 1) as ex:
            return list(ex.map(lambda a: self.counts(x, a, povh), angles))

    def sector(self, op, x, angle, povh=0.15):
        dy, dx = x.shape
        n = dx * dy
        ln = 2 * n + max(dx, dy)
        si = np.zeros(ln, np.float32)
        so = np.zeros(ln, np.float32)
        acc = np.zeros(n, np.float32)
        assert self.lib.port_sector(op, np.ascontiguousarray(x, np.float32), dx, dy, angle, povh, si, so, acc) == 0
        return si, so, acc.reshape(dy, dx)

    def counts(self, x, angle, povh=0.15):
        dy, dx = x.shape
        out = np.zeros(2 * dx * dy + max(dx, dy), np.float32)
        assert self.lib.port_sdem_counts(np.ascontiguousarray(x, np.float32), dx, dy, angle, povh, out) == 0
        return out

    def accumulate(self, op, x, angles, povh=0.15):
        """Per-type accumulators (4 x N) and the used-type mask of one angle list."""
        dy, dx = x.shape
        acc = np.zeros(4 * dx * dy, np.float32)
        used = np.zeros(1, np.int32)
        a = np.ascontiguousarray(angles, np.int32)
        assert self.lib.port_accumulate(op, np.ascontiguousarray(x, np.float32), dx, dy, a, len(a), povh, acc,
                                        used) == 0
        return acc.reshape(4, dx * dy), int(used[0])


@pytest.fixture(scope="session")
def oracle(port):
    return PortOracle(port)


@pytest.fixture(scope="session")
def golden_runs():
    return np.load(os.path.join(GOLDEN, "runs.npz"))


@pytest.fixture(scope="session")
def golden_sectors():
    return np.load(os.path.join(GOLDEN, "sectors.npz"))


@pytest.fixture(scope="session")
def golden_geometry():
    return np.load(os.path.join(GOLDEN, "geometry.npz"))


def run_cases(golden_runs):
    """(key, op_name, input, expected) of every whole-run golden case."""
    from tests.golden.make_golden import OPS  # noqa: E402
    out = []
    for k in sorted(golden_runs.files):
        if not k.endswith("__in"):
            continue
        base = k[:-4]
        out.append((base, OPS[base.split("__")[0]], golden_runs[k], golden_runs[base + "__out"]))
    return out


def bits_equal(a, b) -> bool:
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.fixture(scope="session")
def gpu_lib():
    """libskewengine.so on a GPU machine; a GPU test never falls back to the CPU."""
    from skewengine_gb300 import build, device_count
    build.build()
    if device_count() < 1:
        pytest.fail("gpu test selected but no CUDA device is visible")
    from skewengine_gb300 import _lib
    return _lib.load()
