"""Build the engine's shared library, libskewengine.so, in-tree.

    python -m skewengine_gb300.build [--force]

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), host C++ with g++; the units
compile in parallel and link with nvcc into ``skewengine_gb300/_lib``.  Host and
device code are compiled without floating-point contraction (``-ffp-contract=off``,
``-fmad=false``): the reference's results are defined by an x86-64 build that
fuses no multiply-add, and the kernels place every fused operation they need
explicitly.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(OUT_DIR, "obj")
LIB_NAME = "libskewengine.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["engine.cu", "k_layout.cu", "k_batch.cu", "k_sdem.cu", "k_sdem_noalloc.cu", "k_radon.cu", "k_lradon.cu", "k_lradon_f32.cu", "k_cepstrum.cu", "k_cepstrum_f32.cu",
              "k_peak.cu", "k_conv.cu"]
CPP_SOURCES = ["geometry.cpp", "cli.cpp", "image_io.cpp"]
HEADERS = ["ske_internal.h", "ske_device.cuh", "kernels.h", "image_io.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")


def _compile(cmd: list[str]) -> tuple[list[str], int, str]:
    p = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, p.returncode, p.stdout + p.stderr


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (when stale) and return the path of libskewengine.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "skewengine.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD_DIR, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path, __file__] + headers):
            jobs.append([nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
                         "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", CSRC, "-c", path, "-o", obj])
    for src in CPP_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD_DIR, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path, __file__] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", CSRC,
                         "-I", cuda_include(), "-c", path, "-o", obj])
    if jobs:
        workers = min(len(jobs), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            for cmd, rc, out in ex.map(_compile, jobs):
                if verbose or rc != 0:
                    sys.stderr.write(" ".join(cmd) + "\n" + out)
                if rc != 0:
                    raise RuntimeError(f"compile failed: {cmd[-3]}")
    if force or jobs or _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp]
        _, rc, out = _compile(cmd)
        if rc != 0:
            sys.stderr.write(out)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB_PATH)
    _alias_reference_name()
    return LIB_PATH


# The reference builds its shared library as `sk_engine` (CMakeLists.txt:83):
# a link of that name beside the library lets a caller that loads it by that
# name (its only export, run(argc, argv), is here too) load this one.
REFERENCE_LIB_NAME = "libsk_engine.so"


def _alias_reference_name() -> None:
    alias = os.path.join(OUT_DIR, REFERENCE_LIB_NAME)
    try:
        if os.path.islink(alias) and os.readlink(alias) == LIB_NAME:
            return
        if os.path.lexists(alias):
            os.remove(alias)
        os.symlink(LIB_NAME, alias)
    except OSError:
        pass  # a filesystem without links: the library keeps its own name only


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    args = ap.parse_args()
    print(build(force=args.force, verbose=args.verbose))


if __name__ == "__main__":
    main()
