"""The C ABI surface, host-only entry points and error behaviour (no GPU needed)."""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import re

import numpy as np
import pytest

from tests.conftest import GOLDEN, ROOT


@pytest.fixture(scope="module")
def lib():
    from skewengine_gb300 import _lib, build
    build.build()
    return _lib.load()


def declared_functions() -> list[str]:
    text = open(os.path.join(ROOT, "include", "skewengine.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    # Function declarations: `<type> name(` at line start (typedefs excluded).
    return re.findall(r"^(?:const\s+char\s*\*|int|void)\s+(\w+)\s*\(", text, flags=re.M)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "ske_run" in names and "run" in names and len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_python_signatures_cover_header(lib):
    from skewengine_gb300._lib import SIGNATURES
    bound = {s[0] for s in SIGNATURES}
    assert set(declared_functions()) <= bound


def test_version_and_defaults(lib):
    from skewengine_gb300 import params
    assert lib.ske_abi_version() == 1
    p = params()
    assert p.max_sector == 180 and p.accum == 0 and p.flags == 0
    assert np.float32(p.povh) == np.float32(1.5 / 10.0)


def _geom_digest(g) -> str:
    h = hashlib.sha256()
    ii = np.array([g["sector_type"], g["new_angle"], g["dim_i"], g["dim_o"], g["offset"], g["skew_height"],
                   g["dim_l"]], np.int32)
    dd = np.array([g["scale"], g["skewness"]], np.float64)
    for arr in (ii, dd, g["first"].astype(np.uint16), g["last"].astype(np.uint16), g["target"], g["weight"]):
        h.update(np.ascontiguousarray(arr).tobytes())
    return h.hexdigest()


def test_geometry_matches_reference_small(golden_geometry):
    from skewengine_gb300 import geometry
    shapes = sorted({k.split("__")[0] for k in golden_geometry.files})
    for shp in shapes:
        dx, dy = map(int, shp.split("x"))
        ii, dd = golden_geometry[shp + "__iinfo"], golden_geometry[shp + "__dinfo"]
        off = {"first": 0, "last": 0, "target": 0, "weight": 0}
        for a in range(180):
            g = geometry(dx, dy, a)
            got = [g["sector_type"], g["new_angle"], g["dim_i"], g["dim_o"], g["offset"], g["skew_height"],
                   g["dim_l"]]
            assert got == list(ii[a]), (shp, a)
            assert g["scale"] == dd[a, 0] and g["skewness"] == dd[a, 1], (shp, a)
            for name in ("first", "last", "target", "weight"):
                n = len(g[name])
                ref = golden_geometry[f"{shp}__{name}"][off[name]:off[name] + n]
                assert np.array_equal(g[name].astype(ref.dtype), ref), (shp, a, name)
                off[name] += n


def test_geometry_matches_reference_benchmark_grids():
    """SHA-256 of every angle's tables for the benchmark grid sizes (2000^2 ...)."""
    from skewengine_gb300 import geometry
    digests = json.load(open(os.path.join(GOLDEN, "geometry_digest.json")))
    for shp, want in digests.items():
        dx, dy = map(int, shp.split("x"))
        for a in range(180):
            assert _geom_digest(geometry(dx, dy, a)) == want[a], (shp, a)


def test_geometry_rejects_bad_arguments():
    from skewengine_gb300 import SkeError, geometry
    for args in ((0, 5, 0), (5, 5, 180), (5, 5, -1), (70000, 5, 0)):
        with pytest.raises(SkeError) as ei:
            geometry(*args)
        assert ei.value.status == 1


def test_no_gpu_fails_loudly(lib):
    """Without a GPU the engine refuses to run; there is no CPU fallback."""
    from skewengine_gb300 import SkeError, SkewEngine, device_count
    if device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(SkeError) as ei:
        SkewEngine(16, 16)
    assert ei.value.status == 3
    assert "device" in str(ei.value).lower()
    n = C.c_int64()
    assert lib.ske_selftest_division(0, 16, C.byref(n), C.byref(C.c_int64()), C.byref(C.c_uint32())) == 3


def test_null_engine_is_rejected(lib):
    from skewengine_gb300 import params
    p = params()
    x = np.zeros(4, np.float32)
    assert lib.ske_run(None, 0, x.ctypes.data, 0, x.ctypes.data, 0, C.byref(p)) == 1
    assert b"null" in lib.ske_last_error()
    assert lib.ske_skew(None, 0) == 1
    assert lib.ske_destroy(None) == 0


def test_convolutions_validate_arguments_before_launching(lib):
    """Shapes and alignments the surrogate's convolution kernels cannot take are
    refused before any device work.  The pointers are stand-ins that are never
    dereferenced: every call below fails its argument checks."""
    a = C.c_void_p(0x10000)  # 16-byte aligned
    odd = C.c_void_p(0x10002)
    s = None
    conv = lib.ske_conv3x3_bf16
    assert conv(a, a, None, a, 1, 8, 8, 12, 16, 1, s) == 1  # cin not a multiple of 8
    assert conv(a, a, None, a, 1, 8, 8, 16, 15, 1, s) == 1  # odd cout
    assert conv(a, a, None, a, 0, 8, 8, 16, 16, 1, s) == 1  # empty batch
    assert conv(odd, a, None, a, 1, 8, 8, 16, 16, 1, s) == 1  # misaligned input
    assert conv(a, odd, None, a, 1, 8, 8, 16, 16, 1, s) == 1  # misaligned weights
    assert conv(a, a, None, None, 1, 8, 8, 16, 16, 1, s) == 1  # no output
    upcat = lib.ske_conv3x3_upcat_bf16
    assert upcat(a, a, a, None, a, 1, 7, 8, 16, 16, 16, 1, s) == 1  # odd height
    assert upcat(a, a, a, None, a, 1, 8, 8, 16, 12, 16, 1, s) == 1  # skip channels not a multiple of 8
    wgrad = lib.ske_conv3x3_wgrad_bf16
    assert wgrad(a, a, a, 1, 8, 8, 16, 12, s) == 1  # cout not a multiple of 8
    assert wgrad(a, a, odd, 1, 8, 8, 16, 16, s) == 1  # misaligned float32 gradient
    assert lib.ske_conv_status(None, s) == 1
    head = lib.ske_conv3x3_head_bf16
    assert head(a, a, None, a, a, a, 1, 8, 8, 16, 24, 1, s) == 1  # cout not a multiple of 16
    assert head(a, a, None, None, a, a, 1, 8, 8, 16, 32, 1, s) == 1  # no head weights
    assert head(a, a, None, a, None, a, 1, 8, 8, 16, 32, 1, s) == 1  # no head bias
    assert head(a, a, None, a, a, C.c_void_p(0x10001), 1, 8, 8, 16, 32, 1, s) == 1  # misaligned output
    pool = lib.ske_maxpool2_bf16
    assert pool(a, a, 1, 7, 8, 16, s) == 1  # odd height
    assert pool(a, a, 1, 8, 8, 12, s) == 1  # channels not a multiple of 8
    assert pool(a, C.c_void_p(0x10008), 1, 8, 8, 16, s) == 1  # output not 16-byte aligned
    enc = lib.ske_surrogate_encode_bf16
    assert enc(a, a, a, a, 3, 16.0, a, 1, 256, s) == 1  # side not a multiple of the coarse factor
    assert enc(a, a, a, a, 4, 0.0, a, 1, 256, s) == 1  # scale not positive
    assert enc(a, None, a, a, 4, 16.0, a, 1, 256, s) == 1  # no means
    assert enc(a, a, a, a, 2, 16.0, a, 1, 46342, s) == 1  # side * side past an int
    # kernel choices: valid values are taken, others refused and the choice kept
    assert lib.ske_conv_select(3) == 1 and lib.ske_conv_select(0) == 0
    assert lib.ske_conv_stage_channels(24) == 1 and lib.ske_conv_stage_channels(0) == 0
    assert lib.ske_skew_select(2) == 1 and lib.ske_skew_select(0) == 0
    assert lib.ske_conv_wgrad_select(2) == 1 and lib.ske_conv_wgrad_select(1) == 0


def test_cli_usage_errors():
    from skewengine_gb300 import cli_run
    assert cli_run([]) == 1
    assert cli_run(["nosuchkernel", "x", "1", "1", "y"]) == 1
    assert cli_run(["sdem", "/nonexistent/file.raw", "4", "4", "/tmp/out.raw"]) == 1


def test_sector_tables_within_kernel_bounds():
    """ske_geometry checks every table against the bounds the kernels index
    with (row spans in [0, dim_l], the farthest cell inside the skew buffer,
    column shifts inside the skewed rows) and refuses one that breaks them.
    Every real table passes: all 180 angles of tiny, ragged, strongly
    non-square and benchmark-sized grids."""
    from skewengine_gb300 import engine
    shapes = [(x, y) for x in (1, 2, 3, 7, 33) for y in (1, 2, 3, 7, 33)]
    shapes += [(1, 500), (500, 1), (17, 4000), (4000, 17), (255, 256), (512, 512), (2000, 2000), (4096, 300)]
    for dimx, dimy in shapes:
        n = dimx * dimy
        for a in range(180):
            g = engine.geometry(dimx, dimy, a)
            H, di, dl = g["skew_height"], g["dim_i"], g["dim_l"]
            f, l = g["first"], g["last"]
            assert f.min() >= 0 and l.max() <= dl
            assert int((np.arange(H, dtype=np.int64) * di + l).max()) <= 2 * n + dl
            assert g["target"].min() >= 0 and int(g["target"].max()) + g["dim_o"] <= H


class _FakeCudaGrid:
    """Stands in for a CUDA tensor in checks that run before any device work."""
    is_cuda = True
    dtype = "torch.float32"

    def __init__(self, shape):
        self.shape = tuple(shape)
        self.ndim = len(self.shape)

    def is_contiguous(self):
        return True

    def data_ptr(self):
        return 16  # never dereferenced: the call is refused first


def test_run_batch_refuses_mixed_placements_and_mismatched_outputs(lib):
    """run_batch passes one placement flag for all inputs and one for all
    outputs, so a list mixing host arrays and CUDA tensors, outputs placed
    unlike their grids, outputs of the wrong shape or count, and grids that
    are not 2-D are refused before an engine is made or a pointer is read."""
    from skewengine_gb300 import engine
    h = np.zeros((8, 8), np.float32)
    with pytest.raises(TypeError):
        engine.run_batch(0, [h, _FakeCudaGrid((8, 8))])
    with pytest.raises(TypeError):
        engine.run_batch(0, [h], outs=[_FakeCudaGrid((8, 8))])
    with pytest.raises(TypeError):
        engine.run_batch(0, [_FakeCudaGrid((8, 8))], outs=[np.zeros((8, 8), np.float32)])
    with pytest.raises(TypeError):
        engine.run_batch(0, _FakeCudaGrid((2, 8, 8)), outs=np.zeros((2, 8, 8), np.float32))
    with pytest.raises(ValueError):
        engine.run_batch(0, [h, h], outs=[np.zeros((8, 8), np.float32)])
    with pytest.raises(ValueError):
        engine.run_batch(0, [h], outs=[np.zeros((8, 4), np.float32)])
    with pytest.raises(ValueError):
        engine.run_batch(0, [np.zeros((2, 8, 8), np.float32)])


def test_reference_library_name_loads_this_library(lib):
    """The build places libsk_engine.so (the reference's shared-library name,
    CMakeLists.txt:83) beside libskewengine.so: a caller loading the reference's
    library by name gets this one, with its run(argc, argv)."""
    from skewengine_gb300 import _lib
    alias = os.path.join(os.path.dirname(_lib.LIB_PATH), "libsk_engine.so")
    assert os.path.realpath(alias) == os.path.realpath(_lib.LIB_PATH)
    ref = C.CDLL(alias)
    ref.run.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    argv = (C.c_char_p * 1)(b"run")
    assert ref.run(1, argv) == 1  # usage: too few arguments


def test_fold_refuses_a_state_of_another_grid(lib):
    """SkewEngine.fold hands the library 4 x N accumulators and compensations:
    a saved state of another size raises before the call (checked on an engine
    object that was never opened, so no device is needed)."""
    from skewengine_gb300 import engine
    eng = engine.SkewEngine.__new__(engine.SkewEngine)
    eng.dimx, eng.dimy, eng.N, eng._h = 4, 3, 12, None
    small = {"acc": np.zeros((4, 11), np.float32), "comp": np.zeros((4, 12), np.float32), "used": 1}
    with pytest.raises(ValueError):
        eng.fold(0, small)
    small = {"acc": np.zeros((4, 12), np.float32), "comp": np.zeros(5, np.float32), "used": 1}
    with pytest.raises(ValueError):
        eng.fold(0, small)


def test_header_serves_plain_c_callers(lib, tmp_path):
    """include/skewengine.h compiles as C99 with every warning on, and a C
    program linked against the library runs the whole-run call sequence of
    the reference's replacement (create, run, destroy); without a device the
    create call returns SKE_ERR_NO_DEVICE with a message instead of failing."""
    import subprocess
    from skewengine_gb300 import _lib
    src = tmp_path / "caller.c"
    src.write_text(
        "#include <stdio.h>\n#include \"skewengine.h\"\n"
        "int main(void) {\n"
        "    float in[16] = {0}, out[16];\n    ske_engine e;\n    ske_params p;\n"
        "    if (ske_params_default(&p) != SKE_OK) return 10;\n"
        "    int rc = ske_create(&e, 4, 4, 0, NULL);\n"
        "    if (rc != SKE_OK) { printf(\"create %d %s\\n\", rc, ske_last_error()); return 0; }\n"
        "    rc = ske_run(e, SKE_KERNEL_SDEM, in, 0, out, 0, &p);\n"
        "    ske_destroy(e);\n    printf(\"run %d\\n\", rc);\n    return rc;\n}\n")
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "caller")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-L", libdir, "-lskewengine", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("run 0") or r.stdout.startswith("create 3 "), r.stdout
