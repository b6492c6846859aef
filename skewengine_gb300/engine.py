"""Python host interface of the engine, mirroring the reference's skewEngine API.

The reference drives its engine from ``execute()`` (src/main.cu:71-172)::

    skewer->skew(i); skewer->kernel(); skewer->deskew(isMax);   // every sector
    skewer->reduce(outD, isMax);                                // once

``SkewEngine`` exposes the same per-sector methods (``skew``, ``kernel``,
``deskew``, ``reduce``) plus ``run``, which executes the whole sector loop on the
GPU in batched launches.  Arrays may be NumPy arrays (host) or CUDA tensors
(device, anything exposing ``data_ptr()`` and ``is_cuda``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import Params, SectorGeometry, SectorView, check, load

# Operators: the reference KERNELS enum (src/global.h:77).
KERNEL_SDEM = 0
KERNEL_IDENTITYDEM = 1
KERNEL_RADON = 2
KERNEL_IDENTITYIMG = 3
KERNEL_CEPSTRUM = 4
# The reference's Radon operator with LRT set (kernelRADN.h:212-220): the local
# Radon transform of every skewed cell (no id in the reference's enum).
KERNEL_LOCAL_RADON = 5
KERNELS = {"sdem": KERNEL_SDEM, "identitydem": KERNEL_IDENTITYDEM, "radon": KERNEL_RADON,
           "identityimg": KERNEL_IDENTITYIMG, "cepstrum": KERNEL_CEPSTRUM, "localradon": KERNEL_LOCAL_RADON}

ACCUM_REFERENCE = 0
ACCUM_KAHAN = 1
_ACCUM = {"reference": ACCUM_REFERENCE, "kahan": ACCUM_KAHAN}

DEFAULT_POVH = float(np.float32(1.5 / 10.0))  # obsheight / step, kernelSDEM.h:159


def _kernel_id(k) -> int:
    return KERNELS[k] if isinstance(k, str) else int(k)


def _accum_id(a) -> int:
    return _ACCUM[a] if isinstance(a, str) else int(a)


def _is_device(x) -> bool:
    return bool(getattr(x, "is_cuda", False))


def _ptr(x, shape=None, writable=False):
    """(pointer, on_device) of a float32 C-contiguous array or CUDA tensor."""
    if _is_device(x):
        if str(x.dtype) != "torch.float32" or not x.is_contiguous():
            raise TypeError("device arrays must be contiguous float32 tensors")
        if shape is not None and tuple(x.shape) != tuple(shape):
            raise ValueError(f"expected shape {shape}, got {tuple(x.shape)}")
        return C.c_void_p(x.data_ptr()), 1
    if not isinstance(x, np.ndarray) or x.dtype != np.float32 or not x.flags.c_contiguous:
        raise TypeError("host arrays must be C-contiguous float32 numpy arrays")
    if writable and not x.flags.writeable:
        raise ValueError("output array is read-only")
    if shape is not None and x.shape != tuple(shape):
        raise ValueError(f"expected shape {shape}, got {x.shape}")
    return C.c_void_p(x.ctypes.data), 0


FLAG_NO_TUNE = 1   # keep the sweep's built-in shape (skip the autotuner)
FLAG_NO_GRAPH = 2  # batched runs: plain launches, no captured CUDA graph
FLAG_CEPSTRUM_F32 = 4  # cepstrum in float32, fused sector loop (stated bin-mismatch rate)
FLAG_LOCAL_RADON_F32 = 8  # local Radon transform in float32 (stated mismatch rate)
FLAG_RADON_F32 = 16  # Radon ray sums and filter in float32 (stated error)


def params(max_sector: int = 180, povh: float = DEFAULT_POVH, accum="reference", flags: int = 0) -> Params:
    p = Params()
    check(load().ske_params_default(C.byref(p)))
    p.max_sector = max_sector
    p.povh = povh
    p.accum = _accum_id(accum)
    p.flags = int(flags)
    return p


def device_count() -> int:
    n = C.c_int(0)
    check(load().ske_device_count(C.byref(n)))
    return n.value


def geometry(dimx: int, dimy: int, angle: int) -> dict:
    """Host geometry of one sector: computeParams + skewShape (skewEngine.cuh:504-596)."""
    lib = load()
    g = SectorGeometry()
    check(lib.ske_geometry(dimx, dimy, angle, C.byref(g), None, None, None, None))
    first = np.zeros(g.skew_height, np.int32)
    last = np.zeros(g.skew_height, np.int32)
    target = np.zeros(g.dim_i, np.int32)
    weight = np.zeros(g.dim_i, np.float32)
    check(lib.ske_geometry(dimx, dimy, angle, C.byref(g), first.ctypes.data, last.ctypes.data,
                           target.ctypes.data, weight.ctypes.data))
    out = {f: getattr(g, f) for f, _ in SectorGeometry._fields_}
    out.update(first=first, last=last, target=target, weight=weight)
    return out


class SkewEngine:
    """One engine per grid size, bound to one device and one CUDA stream
    (``skewEngine<float>`` of skewEngine.cuh:147, one per OpenMP thread)."""

    def __init__(self, dimx: int, dimy: int, device: int = 0, stream: int | None = None):
        self._lib = load()
        self.dimx, self.dimy = int(dimx), int(dimy)
        self.N = self.dimx * self.dimy
        self.dim_l = max(self.dimx, self.dimy)
        self.skew_len = 2 * self.N + self.dim_l
        h = C.c_void_p()
        check(self._lib.ske_create(C.byref(h), self.dimx, self.dimy, int(device),
                                   C.c_void_p(stream) if stream else None))
        self._h = h
        self._keep = []
        self.device = int(device)
        self._ext = None  # torch's handle on the engine's stream, made on first device call

    # lifetime -------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            check(self._lib.ske_destroy(self._h))
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        check(self._lib.ske_stream(self._h, C.byref(s)))
        return s.value or 0

    def _after_torch(self, *arrays) -> None:
        """CUDA tensors handed to the engine may still be written (inputs) or
        read (outputs) by work queued on torch's current stream: the engine's
        stream waits for that work first (an event, no host synchronisation).
        Every engine call has finished its own work when it returns."""
        if not any(_is_device(a) for a in arrays if a is not None):
            return
        import torch
        cur = torch.cuda.current_stream(self.device)
        if self._ext is None:
            self._ext = torch.cuda.ExternalStream(self.stream, device=self.device)
        if cur.cuda_stream != self._ext.cuda_stream:
            self._ext.wait_stream(cur)

    # whole run ------------------------------------------------------------
    def run(self, kernel, data, out=None, max_sector: int = 180, povh: float = DEFAULT_POVH,
            accum="reference", angles=None, flags: int = 0):
        """Full sector loop (allocate + execute + reduce of the reference)."""
        shape = (self.dimy, self.dimx)
        pin, in_dev = _ptr(data, shape)
        if out is None:
            if in_dev:
                import torch
                out = torch.empty(shape, dtype=torch.float32, device=data.device)
            else:
                out = np.empty(shape, np.float32)
        pout, out_dev = _ptr(out, shape, writable=True)
        self._after_torch(data, out)
        prm = params(max_sector, povh, accum, flags)
        if angles is None:
            check(self._lib.ske_run(self._h, _kernel_id(kernel), pin, in_dev, pout, out_dev, C.byref(prm)))
        else:
            a = np.ascontiguousarray(np.asarray(angles, dtype=np.int32))
            check(self._lib.ske_run_angles(self._h, _kernel_id(kernel), pin, in_dev, pout, out_dev,
                                           a.ctypes.data, len(a), C.byref(prm)))
        return out

    def accumulate(self, kernel, data, angles, povh: float = DEFAULT_POVH, accum="reference"):
        """Run the listed sectors and return (4 x N per-type accumulators, used-type mask)."""
        pin, in_dev = _ptr(data, (self.dimy, self.dimx))
        self._after_torch(data)
        a = np.ascontiguousarray(np.asarray(angles, dtype=np.int32))
        acc = np.empty((4, self.N), np.float32)
        used = C.c_uint32(0)
        prm = params(180, povh, accum)
        check(self._lib.ske_accumulate(self._h, _kernel_id(kernel), pin, in_dev, a.ctypes.data if len(a) else None,
                                       len(a), C.byref(prm), acc.ctypes.data, 0, C.byref(used)))
        return acc, used.value

    # checkpoint / resume --------------------------------------------------
    def accumulate_resume(self, kernel, data, angles, state=None, povh: float = DEFAULT_POVH, accum="reference"):
        """Continue an accumulation over the listed sectors from ``state`` (a dict
        with ``acc``, ``comp`` (4 x N float32) and ``used``; None = zero) and
        return the new state."""
        pin, in_dev = _ptr(data, (self.dimy, self.dimx))
        self._after_torch(data)
        a = np.ascontiguousarray(np.asarray(angles, dtype=np.int32))
        if state is None:
            state = {"acc": np.zeros((4, self.N), np.float32), "comp": np.zeros((4, self.N), np.float32), "used": 0}
        acc = np.array(state["acc"], np.float32, copy=True).reshape(4, self.N)
        comp = np.array(state["comp"], np.float32, copy=True).reshape(4, self.N)
        used = C.c_uint32(int(state["used"]))
        prm = params(180, povh, accum)
        check(self._lib.ske_accumulate_resume(self._h, _kernel_id(kernel), pin, in_dev,
                                              a.ctypes.data if len(a) else None, len(a), C.byref(prm),
                                              acc.ctypes.data, comp.ctypes.data, 0, C.byref(used)))
        return {"acc": acc, "comp": comp, "used": used.value}

    def fold(self, kernel, state, accum="reference", out=None):
        """The output grid of a saved accumulator state (the final reduce)."""
        shape = (self.dimy, self.dimx)
        if out is None:
            out = np.empty(shape, np.float32)
        p, dev = _ptr(out, shape, writable=True)
        self._after_torch(out)
        # 4 x N each: the library reads that many (a smaller array raises here).
        acc = np.ascontiguousarray(state["acc"], np.float32).reshape(4, self.N)
        comp = np.ascontiguousarray(state["comp"], np.float32).reshape(4, self.N)
        check(self._lib.ske_fold(self._h, _kernel_id(kernel), acc.ctypes.data, comp.ctypes.data, 0,
                                 int(state["used"]), _accum_id(accum), p, dev))
        return out

    def run_checkpointed(self, kernel, data, path, chunk: int = 30, max_sector: int = 180,
                         povh: float = DEFAULT_POVH, accum="reference", stop_after=None):
        """Whole run in chunks of ``chunk`` sectors, saving the accumulator state
        and the next sector index to ``path`` (.npz) after each chunk and resuming
        from it when it exists.  ``stop_after`` (chunks) ends the call early, as an
        interrupted job would; the result equals ``run`` bit for bit."""
        import os
        start, state = 0, None
        if os.path.exists(path):
            z = np.load(path)
            if (int(z["kernel"]), int(z["max_sector"]), str(z["accum"]), int(z["dimx"]), int(z["dimy"])) != \
                    (_kernel_id(kernel), max_sector, str(accum), self.dimx, self.dimy):
                raise ValueError(f"checkpoint {path} belongs to another run")
            start = int(z["next_sector"])
            state = {"acc": z["acc"], "comp": z["comp"], "used": int(z["used"])}
        done = 0
        while start < max_sector:
            if stop_after is not None and done >= stop_after:
                return None
            angles = list(range(start, min(start + chunk, max_sector)))
            state = self.accumulate_resume(kernel, data, angles, state, povh=povh, accum=accum)
            start = angles[-1] + 1
            tmp = str(path) + ".tmp.npz"
            np.savez(tmp, acc=state["acc"], comp=state["comp"], used=state["used"], next_sector=start,
                     kernel=_kernel_id(kernel), max_sector=max_sector, accum=str(accum), dimx=self.dimx,
                     dimy=self.dimy)
            os.replace(tmp, path)
            done += 1
        if state is None:
            state = self.accumulate_resume(kernel, data, [], None, povh=povh, accum=accum)
        return self.fold(kernel, state, accum=accum)

    # per-sector API (main.cu:147-164) -------------------------------------
    def prepare(self, data) -> None:
        p, dev = _ptr(data, (self.dimy, self.dimx))
        self._after_torch(data)
        check(self._lib.ske_prepare(self._h, p, dev))

    def skew(self, angle: int) -> None:
        check(self._lib.ske_skew(self._h, int(angle)))

    def kernel(self, kernel, povh: float = DEFAULT_POVH) -> None:
        check(self._lib.ske_kernel(self._h, _kernel_id(kernel), povh))

    def kernel_custom(self, fn, povh: float = DEFAULT_POVH) -> None:
        """Run ``fn(view: SectorView) -> int`` as the operator of the current sector."""
        cb = _lib.OPERATOR_FN(lambda user, view: int(fn(view.contents)))
        self._keep.append(cb)
        check(self._lib.ske_kernel_custom(self._h, cb, None, povh))

    def deskew(self, is_max: int = 0, accum="reference") -> None:
        check(self._lib.ske_deskew(self._h, int(is_max), _accum_id(accum)))

    def reduce(self, is_max: int = 0, out=None):
        shape = (self.dimy, self.dimx)
        if out is None:
            out = np.empty(shape, np.float32)
        p, dev = _ptr(out, shape, writable=True)
        self._after_torch(out)
        check(self._lib.ske_reduce(self._h, p, dev, int(is_max)))
        return out

    def sector(self) -> SectorView:
        v = SectorView()
        check(self._lib.ske_sector(self._h, C.byref(v)))
        return v

    def skewed(self):
        """(skewed input, skewed output) of the current sector, 2N + dim_l floats each."""
        si = np.empty(self.skew_len, np.float32)
        so = np.empty(self.skew_len, np.float32)
        check(self._lib.ske_copy_skewed(self._h, si.ctypes.data, so.ctypes.data, 0))
        return si, so

    def sdem_counts(self, angle: int, povh: float = DEFAULT_POVH):
        """Integer visibility counts cv of every skewed cell of one sector."""
        out = np.empty(self.skew_len, np.float32)
        check(self._lib.ske_sdem_counts(self._h, int(angle), povh, out.ctypes.data, 0))
        return out

    # profiling ------------------------------------------------------------
    def profile(self, enable: bool = True) -> None:
        check(self._lib.ske_profile_enable(self._h, int(enable)))

    def profile_get(self, name: str):
        ms = C.c_double()
        n = C.c_int64()
        check(self._lib.ske_profile_get(self._h, name.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def sweep_shape(self) -> tuple[int, int, int]:
        """(lvl0, lvl1, CTAs per SM) of the last viewshed sweep (ske_sweep_shape)."""
        v = [C.c_int(), C.c_int(), C.c_int()]
        check(self._lib.ske_sweep_shape(self._h, *[C.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def set_sweep_shape(self, lvl0: int = 0, lvl1: int = 0, ctas_per_sm: int = 0) -> None:
        """Fix the sweep's shape (ske_set_sweep_shape); lvl0 = 0 hands it back to the autotuner."""
        check(self._lib.ske_set_sweep_shape(self._h, int(lvl0), int(lvl1), int(ctas_per_sm)))

    def launch_count(self) -> int:
        n = C.c_int64()
        check(self._lib.ske_launch_count(self._h, C.byref(n)))
        return n.value


def execute(kernel, data, max_sector: int = 180, povh: float = DEFAULT_POVH, accum="reference",
            device: int = 0):
    """One-shot run of the reference's ``execute(skewAlgorithm)`` on a 2-D array."""
    dimy, dimx = data.shape
    with SkewEngine(dimx, dimy, device) as eng:
        return eng.run(kernel, data, max_sector=max_sector, povh=povh, accum=accum)


def run_batch(kernel, grids, max_sector: int = 180, povh: float = DEFAULT_POVH, accum="reference",
              device: int = 0, outs=None, angles=None, engine=None, flags: int = 0):
    """Run one operator over many grids of uneven size (``ske_run_batch``, or
    ``ske_run_batch_angles`` with an angle list).  ``grids`` is a list of 2-D
    arrays or tensors, or one C-contiguous (N, H, W) float32 array or tensor of
    N equal grids (``outs`` then the same, made when None); for the stack the
    pointer tables are computed, not gathered grid by grid.  ``engine``: an
    existing SkewEngine to run on (it keeps the batch's plan and buffers for
    later calls); by default one is made for the largest grid and closed
    afterwards."""
    stacked = getattr(grids, "ndim", 2) == 3
    if stacked:
        n, h, w = (int(v) for v in grids.shape)
        if n == 0:
            return grids if outs is None else outs
        on_dev = _is_device(grids)
        if outs is None:
            if on_dev:
                import torch
                outs = torch.empty_like(grids)
            else:
                outs = np.empty_like(grids)
        if _is_device(outs) != on_dev:
            raise TypeError("the grids and their outputs must both be host arrays or both CUDA tensors")
        for arr in (grids, outs):
            _ptr(arr, (n, h, w), writable=arr is outs)  # dtype, contiguity, shape checks
        step = np.arange(n, dtype=np.uint64) * np.uint64(4 * h * w)
        ip = (np.uint64(_ptr(grids)[0].value) + step).astype(np.uint64)
        op = (np.uint64(_ptr(outs)[0].value) + step).astype(np.uint64)
        ins = (C.c_void_p * n).from_buffer_copy(ip.tobytes())
        ous = (C.c_void_p * n).from_buffer_copy(op.tobytes())
        dx = np.full(n, w, np.int32)
        dy = np.full(n, h, np.int32)
        big, count = (w, h), n
    else:
        grids = list(grids)
        if not grids:
            return []
        if any(len(g.shape) != 2 for g in grids):
            raise ValueError("every grid of a list must be 2-D")
        dims = [(int(g.shape[1]), int(g.shape[0])) for g in grids]
        big = max(dims, key=lambda d: d[0] * d[1])
        # One call takes one placement for all inputs and one for all outputs:
        # a host array passed as a device pointer (or the reverse) would be
        # read or written at the wrong address, so mixed lists are refused.
        on_dev = _is_device(grids[0])
        mixed = TypeError("the grids and their outputs must all be host arrays or all CUDA tensors")
        if any(_is_device(g) != on_dev for g in grids):
            raise mixed
        if outs is None:
            if on_dev:
                import torch
                outs = [torch.empty_like(g) for g in grids]
            else:
                outs = [np.empty_like(g) for g in grids]
        outs = list(outs)
        if len(outs) != len(grids):
            raise ValueError(f"{len(outs)} outputs for {len(grids)} grids")
        if any(_is_device(o) != on_dev for o in outs):
            raise mixed
        ins = (C.c_void_p * len(grids))(*[_ptr(g)[0].value for g in grids])
        ous = (C.c_void_p * len(grids))(*[_ptr(o, (d[1], d[0]), writable=True)[0].value
                                          for o, d in zip(outs, dims)])
        dx = np.array([d[0] for d in dims], np.int32)
        dy = np.array([d[1] for d in dims], np.int32)
        count = len(grids)
    prm = params(max_sector, povh, accum, flags)
    eng = engine if engine is not None else SkewEngine(big[0], big[1], device)
    try:
        if on_dev:
            eng._after_torch(grids if stacked else grids[0], outs if stacked else outs[0])
        if angles is None:
            check(eng._lib.ske_run_batch(eng._h, _kernel_id(kernel), count, dx.ctypes.data, dy.ctypes.data,
                                         ins, int(on_dev), ous, int(on_dev), C.byref(prm)))
        else:
            a = np.ascontiguousarray(np.asarray(angles, dtype=np.int32))
            check(eng._lib.ske_run_batch_angles(eng._h, _kernel_id(kernel), count, dx.ctypes.data,
                                                dy.ctypes.data, ins, int(on_dev), ous, int(on_dev), a.ctypes.data,
                                                len(a), C.byref(prm)))
    finally:
        if engine is None:
            eng.close()
    return outs


def read_grid(path: str, dimx: int = 0, dimy: int = 0, crop_x: int = 0, crop_y: int = 0) -> np.ndarray:
    """The input grid of a file as the reference reads it (ske_read_grid): a
    .bil int16 DEM divided by 10 (size from dimx/dimy, else its .hdr, else a
    square from the file size), a raw float32 grid, or a .png image as R + G + B
    per pixel; crop_x/crop_y drop columns/rows from the right/bottom as
    readBilData's crop does.  float32 (rows, columns)."""
    lib = load()
    w, h = C.c_int(), C.c_int()
    p = str(path).encode()
    check(lib.ske_read_grid(p, int(dimx), int(dimy), int(crop_x), int(crop_y), None, 0, C.byref(w), C.byref(h)))
    out = np.empty((h.value, w.value), np.float32)
    check(lib.ske_read_grid(p, int(dimx), int(dimy), int(crop_x), int(crop_y), out.ctypes.data, out.size,
                            C.byref(w), C.byref(h)))
    return out


def png_size(path: str) -> tuple[int, int]:
    """(width, height) of a PNG file."""
    w, h = C.c_int(), C.c_int()
    check(load().ske_png_size(str(path).encode(), C.byref(w), C.byref(h)))
    return w.value, h.value


def read_png_rgba(path: str) -> np.ndarray:
    """The PNG decoded to 8-bit RGBA (height x width x 4)."""
    w, h = png_size(path)
    out = np.zeros((h, w, 4), np.uint8)
    check(load().ske_png_read_rgba(str(path).encode(), out.ctypes.data, out.nbytes))
    return out


def read_image(path: str) -> np.ndarray:
    """The reference's image input (helper::read_png, src/helper.h:167-184): a
    float32 grid of R + G + B per pixel."""
    w, h = png_size(path)
    out = np.zeros((h, w), np.float32)
    check(load().ske_png_read_image(str(path).encode(), out.ctypes.data, out.size))
    return out


def write_png(path: str, pixels: np.ndarray) -> None:
    """Write uint8 grey (h x w) or RGB (h x w x 3) pixels as a PNG file."""
    px = np.ascontiguousarray(pixels, np.uint8)
    ch = 1 if px.ndim == 2 else px.shape[2]
    check(load().ske_png_write(str(path).encode(), px.ctypes.data, px.shape[1], px.shape[0], ch))


def render(kernel, output: np.ndarray) -> np.ndarray:
    """The reference's colouring of an operator's output (h x w x 3 uint8)."""
    out = np.ascontiguousarray(output, np.float32)
    rgb = np.zeros(out.shape + (3,), np.uint8)
    check(load().ske_render(_kernel_id(kernel), out.ctypes.data, out.shape[1], out.shape[0], rgb.ctypes.data))
    return rgb


def render_input(image: np.ndarray) -> np.ndarray:
    """The grey input image the reference writes beside a result: (R + G + B) / 3."""
    img = np.ascontiguousarray(image, np.float32)
    grey = np.zeros(img.shape, np.uint8)
    check(load().ske_render_input(img.ctypes.data, img.size, grey.ctypes.data))
    return grey


def cli_run(argv: list[str]) -> int:
    """Call the reference-compatible ``run(argc, argv)`` entry point."""
    args = ["run"] + [str(a) for a in argv]
    arr = (C.c_char_p * len(args))(*[a.encode() for a in args])
    return load().run(len(args), arr)
