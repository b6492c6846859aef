#!/usr/bin/env python
"""Benchmark: total viewshed (kernelSDEM) of a 2000 x 2000 DEM over 180 engine
angles = 360 directional sectors, in Mpoint*sectors/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one full total-viewshed computation of the DEM (all 180 angles:
skew, line-of-sight sweep, deskew/accumulate, fold).  The DEM is seeded
diamond-square terrain (H = 0.8, 0-1500 m, 10 m cells, observer 1.5 m) standing
in for the reference's 2000^2 .bil file, which is not distributed.

Output: one JSON line on rank 0.  ``value`` is device-resident throughput (input
and output in HBM); ``e2e`` is the same metric through the C ABI with host
buffers, host<->device copies inside the timed region.  ``roofline`` covers the
sweep kernel: algorithmic FP32 lane operations (3 per line-of-sight step:
subtract, divide, compare-max) per launch over its CUDA-event duration, against
the FP32 lane-operation rate measured on the same GPU.  ``cpu_baseline`` is the
CPU oracle (a restatement of the reference's OpenMP CPU path) on all host cores
over a sample of angles.

With N > 1 (torchrun, one rank per GPU) every rank computes its own DEM
(seed + rank): weak scaling, no collective on the data path.

``--impl reference`` times the reference's CPU implementation of the same
workload on the host cores: its own code (oracle/_ref) where it was compiled,
otherwise the oracle restatement, one bounded sample of angles per step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Viewshed Mpoint·sectors/s (2000² DEM, 360 sect)"
UNIT = "Mpoint·sectors/s"
SIDE = 2000
ANGLES = 180
DIR_SECTORS = 2 * ANGLES  # each skewed row is scanned both ways (kernelSDEM.h:189-217)
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes (read + write) of one 2000x2000 sweep launch (all 180 angles), from
# an ncu capture of this workload (dram__bytes_read.sum + dram__bytes_write.sum,
# one pass).  Other sizes report none: the survivor lists' share of the traffic
# does not scale with the grid.
SWEEP_DRAM_BYTES_2000 = 16.981758208e9 + 34.468489984e9


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def sample_angles(n: int) -> list[int]:
    """n angles spread evenly over [0, 180)."""
    n = max(1, min(ANGLES, n))
    return sorted({int(a) for a in np.floor(np.arange(n) * (ANGLES / n))})


def load_cpu_impl(prefer_reference: bool):
    """(callable(x, angles, threads) -> output, kind).  The reference's own CPU
    code when it was compiled on this machine, else the oracle restatement."""
    fp = np.ctypeslib.ndpointer(np.float32, flags="C")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C")
    ref = os.path.join(ROOT, "oracle", "_ref", "libskewref.so")
    if prefer_reference and os.path.exists(ref):
        try:
            lib = C.CDLL(ref)
            lib.skref_run_angles.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, ip, C.c_int, C.c_float, C.c_int]

            def run_ref(x, angles, threads):
                out = np.zeros_like(x)
                a = np.asarray(angles, np.int32)
                assert lib.skref_run_angles(0, x, out, x.shape[1], x.shape[0], a, len(a), np.float32(0.15),
                                            threads) == 0
                return out

            return run_ref, "reference"
        except OSError:
            pass
    path = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
    if not os.path.exists(path):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    lib = C.CDLL(path)
    lib.port_run_angles.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, ip, C.c_int, C.c_float, C.c_int]

    def run_port(x, angles, threads):
        out = np.zeros_like(x)
        a = np.asarray(angles, np.int32)
        assert lib.port_run_angles(0, x, out, x.shape[1], x.shape[0], a, len(a), np.float32(0.15), threads) == 0
        return out

    return run_port, "port"


_STEPS_ALL = {}


def cpu_sample(x, threads, prefer_reference):
    """Time one bounded sample (one angle per host thread) of the workload and
    extrapolate to all 180 angles by line-of-sight steps: the reference's cost
    per sector is its sweep's sum of L(L-1) over the rows (kernelSDEM.h:180-218),
    counted exactly from the host geometry for the sampled angles and for all."""
    fn, kind = load_cpu_impl(prefer_reference)
    angles = sample_angles(threads)
    t0 = time.perf_counter()
    fn(x, angles, threads)
    dt = time.perf_counter() - t0
    dy, dx = x.shape
    if (dx, dy) not in _STEPS_ALL:
        _STEPS_ALL[(dx, dy)] = los_steps(dx, dy, range(ANGLES))
    steps_sample = los_steps(dx, dy, angles)
    t_full = dt * _STEPS_ALL[(dx, dy)] / max(steps_sample, 1.0)
    value = x.size * DIR_SECTORS / t_full / 1e6
    sample = (f"{len(angles)} of {ANGLES} angles (evenly spread) of the {dx}x{dy} DEM, {threads} threads, "
              f"{dt:.2f} s; extrapolated from {len(angles)} of {ANGLES} angles weighted by their exact "
              f"line-of-sight steps ({steps_sample:.3e} of {_STEPS_ALL[(dx, dy)]:.3e})")
    return value, kind, sample


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def los_steps(dimx: int, dimy: int, angles) -> float:
    """Line-of-sight steps of the sweep: sum over sectors and skewed rows of L(L-1)."""
    import skewengine_gb300 as ske
    total = 0.0
    for a in angles:
        g = ske.geometry(dimx, dimy, a)
        L = (g["last"] - g["first"]).astype(np.float64)
        L = L[L > 0]
        total += float(np.sum(L * (L - 1)))
    return total


def reference_arm(args):
    rank = _env_int("RANK", 0)
    if rank != 0:
        return 0
    from skewengine_gb300 import synthetic
    x = synthetic.fractal_dem(SIDE, 1000)
    threads = os.cpu_count() or 1
    # Warm-up steps load the implementation and start its thread pool on a 256x256
    # crop; every timed step is a full bounded sample of the 2000x2000 workload.
    warm = np.ascontiguousarray(x[:256, :256])
    for _ in range(args.warmup):
        cpu_sample(warm, threads, prefer_reference=True)
    vals = []
    kind = sample = None
    for _ in range(args.steps):
        v, kind, sample = cpu_sample(x, threads, prefer_reference=True)
        vals.append(v)
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded diamond-square DEM)",
            "config": {"workload": f"total viewshed {SIDE}x{SIDE} DEM, {ANGLES} angles / {DIR_SECTORS} "
                                   f"directional sectors, observer 1.5 m, 10 m cells", "sample_per_step": sample,
                       "extrapolated": f"from {len(sample_angles(threads))} of {ANGLES} angles, weighted by "
                                       "their exact line-of-sight steps"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def secondary_workload(args):
    """Radon/back-projection, local Radon or cepstrum on one 512^2 image, 180
    angles per step.

    Not the headline metric: these report images/s, the engine's per-kernel
    times, and a roofline against the measured binary64 FMA rate (both
    operators compute in double precision like the reference)."""
    import torch
    import skewengine_gb300 as ske
    from skewengine_gb300 import build, synthetic
    build.build()
    side = 512
    if args.workload == "radon":
        x = synthetic.ellipse_phantom(side, 2024)
        kernel, families = ske.KERNEL_RADON, ("prepare", "skew", "radon", "deskew", "reduce")
    elif args.workload == "localradon":
        x = synthetic.ellipse_phantom(side, 2024)
        kernel, families = ske.KERNEL_LOCAL_RADON, ("prepare", "skew", "local_radon", "deskew", "reduce")
    else:
        x, _, _ = synthetic.blurred_texture(side, 2024)
        kernel, families = ske.KERNEL_CEPSTRUM, ("prepare", "skew", "cepstrum", "deskew", "reduce")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng = ske.SkewEngine(side, side, stream=stream.cuda_stream)
    x_dev = torch.from_numpy(x).cuda()
    out_dev = torch.empty_like(x_dev)
    for _ in range(args.warmup):
        eng.run(kernel, x_dev, out_dev)
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        eng.run(kernel, x_dev, out_dev)
    t1.record(stream)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / args.steps
    eng.profile(True)
    for _ in range(args.steps):
        eng.run(kernel, x_dev, out_dev)
    breakdown = {k: eng.profile_get(k)[0] / args.steps for k in families}
    eng.profile(False)
    # Algorithmic work: valid skewed cells over all angles.
    cells = 0
    for a in range(ANGLES):
        g = ske.geometry(side, side, a)
        cells += int(np.maximum(g["last"] - g["first"], 0).sum())
    dfma = C.c_double()
    ske.engine.load().ske_measure_fp64_peak(0, C.byref(dfma))
    op_ms = breakdown[families[2]]
    if args.workload == "radon":
        # The reference's binary64 work: one add per valid cell (row sums) and,
        # per sector, two H2-point radix-2 complex FFTs (H2/2 log2 H2
        # butterflies of 10 ops each).  The row sums run on the integer pipes
        # (exact sums), so this is algorithmic work per second, not FP64 pipe use.
        fft_ops = 0
        for a in range(ANGLES):
            h2 = 1
            while h2 < int(ske.geometry(side, side, a)["skew_height"]):
                h2 *= 2
            fft_ops += 2 * (h2 // 2) * (h2.bit_length() - 1) * 10
        ops = float(cells + fft_ops)
        work = (f"the reference's binary64 ops: 1 add per valid skewed cell ({cells}) + two H2-point FFTs per "
                f"sector ({fft_ops}); row sums run as exact integer sums, FFTs in binary64")
    elif args.workload == "localradon":
        # Per valid cell: two 64-point radix-2 complex FFTs (2 x 192 butterflies
        # of 10 binary64 ops), 64 weights, 2 x 64 complex scalings (6 ops), the
        # 26-bin taper, 27 squared magnitudes; plus its share of the 65-term window
        # sums (one per cell).
        ops = float(cells) * (384 * 10 + 64 + 128 * 6 + 26 + 27 * 3 + 65)
        work = ("~4840 binary64 ops per valid skewed cell: the reference's (window sums, weights, two complex "
                "64-point FFTs, scalings); the kernel leaves out products with exact zeros and ones and outputs "
                "nobody reads, so frac is the reference's work per second and can exceed 1")
    else:
        # Per valid cell: 64-point and 32-point radix-2 complex FFTs (192 + 80
        # butterflies of 10 binary64 ops), |X|^2 and scaling (~160 ops).
        ops = float(cells) * (272 * 10 + 160)
        work = ("~2880 binary64 ops per valid skewed cell: the reference's complex 64- and 32-point FFTs and "
                "power spectrum (its 32 logarithms not counted); the kernel leaves out products with exact zeros "
                "and ones and outputs nobody reads")
    line = {"metric": f"{args.workload} 512² images/s (180 angles)", "value": 1e3 / ms, "unit": "images/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "dtype": "f64+f32", "data": "synthetic", "config": {"workload": f"{args.workload} 512x512, 180 angles",
                                                               "kernel_ms_per_step": breakdown,
                                                               "valid_cells": cells},
            "roofline": {"bound": "fp64", "kernel": families[2], "achieved": ops / (op_ms / 1e3) / 1e12,
                         "peak": dfma.value / 1e12, "unit": "Tops/s (binary64 lane ops)",
                         "frac": ops / (op_ms / 1e3) / dfma.value, "work": work, "traffic": None}}
    if args.workload in ("localradon", "radon"):
        # The float32 mode (SKE_FLAG_LOCAL_RADON_F32 / SKE_FLAG_RADON_F32): time,
        # the share of cells that differ from the binary64 result by more than
        # 1e-3 relative, and the largest difference over the output's magnitude.
        exact = out_dev.clone()
        f32 = ske.FLAG_LOCAL_RADON_F32 if args.workload == "localradon" else ske.FLAG_RADON_F32
        out32 = torch.empty_like(x_dev)
        for _ in range(args.warmup):
            eng.run(kernel, x_dev, out32, flags=f32)
        torch.cuda.synchronize()
        t0.record(stream)
        for _ in range(args.steps):
            eng.run(kernel, x_dev, out32, flags=f32)
        t1.record(stream)
        torch.cuda.synchronize()
        ms32 = t0.elapsed_time(t1) / args.steps
        rel = (out32 - exact).abs() / exact.abs().clamp_min(1e-30)
        line["config"]["float32_mode"] = {
            "images_per_s": 1e3 / ms32, "ms_per_step": ms32,
            "cells_off_by_more_than_1e-3_relative": float((rel > 1e-3).float().mean()),
            "median_relative_difference": float(rel.median()),
            "max_difference_over_max_output": float((out32 - exact).abs().max() / exact.abs().max())}
    if not args.no_cpu_baseline:
        fp = np.ctypeslib.ndpointer(np.float32, flags="C")
        ip = np.ctypeslib.ndpointer(np.int32, flags="C")
        lib = C.CDLL(os.path.join(ROOT, "oracle", "_build", "liboracle.so"))
        lib.port_run_angles.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, ip, C.c_int, C.c_float, C.c_int]
        threads = os.cpu_count() or 1
        angles = np.asarray(sample_angles(threads if args.workload in ("cepstrum", "localradon") else ANGLES),
                            np.int32)
        out = np.zeros_like(x)
        c0 = time.perf_counter()
        lib.port_run_angles(kernel, x, out, side, side, angles, len(angles), np.float32(0.15), threads)
        dt = time.perf_counter() - c0
        line["cpu_baseline"] = {"value": len(angles) / ANGLES / dt, "unit": "images/s", "cores": threads,
                                "kind": "port", "sample": f"{len(angles)} of {ANGLES} angles, {dt:.2f} s"}
    print(json.dumps(line), flush=True)
    eng.close()
    return 0


def batch_workload(args):
    """Total viewshed of 64 seeded fractal DEMs with uneven sides (256-2000,
    roughness 0.6-0.9) through ske_run_batch, 180 angles each; Kahan
    accumulation.  Reports Mpoint*sectors/s over the whole batch."""
    import torch
    import skewengine_gb300 as ske
    from skewengine_gb300 import build, synthetic
    build.build()
    # SKE_BATCH_COUNT / SKE_BATCH_MAX_SIDE shrink the batch for profiler captures.
    spec = synthetic.uneven_dem_batch(_env_int("SKE_BATCH_COUNT", 64), 3000,
                                      hi=_env_int("SKE_BATCH_MAX_SIDE", 2000))
    grids = [torch.from_numpy(synthetic.fractal_dem(s, seed, roughness=h)).cuda() for s, h, seed in spec]
    outs = [torch.empty_like(g) for g in grids]
    cells = sum(g.numel() for g in grids)
    big = max(grids, key=lambda g: g.numel())
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng = ske.SkewEngine(big.shape[1], big.shape[0], stream=stream.cuda_stream)
    dx = np.array([g.shape[1] for g in grids], np.int32)
    dy = np.array([g.shape[0] for g in grids], np.int32)
    ins = (C.c_void_p * len(grids))(*[g.data_ptr() for g in grids])
    ous = (C.c_void_p * len(grids))(*[o.data_ptr() for o in outs])
    prm = ske.params(180, ske.DEFAULT_POVH, "kahan")
    lib = ske.engine.load()

    def step():
        ske.engine.check(lib.ske_run_batch(eng._h, ske.KERNEL_SDEM, len(grids), dx.ctypes.data, dy.ctypes.data,
                                           ins, 1, ous, 1, C.byref(prm)))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = eng.launch_count()
    t0.record(stream)
    for _ in range(args.steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / args.steps
    launches = (eng.launch_count() - launches0) / args.steps
    # End to end: the same call with pinned host inputs and outputs (copies in
    # the timed region).
    h_in = [g.cpu().pin_memory() for g in grids]
    h_out = [torch.empty(g.shape, dtype=torch.float32).pin_memory() for g in grids]
    hins = (C.c_void_p * len(grids))(*[g.data_ptr() for g in h_in])
    hous = (C.c_void_p * len(grids))(*[o.data_ptr() for o in h_out])

    def step_host():
        ske.engine.check(lib.ske_run_batch(eng._h, ske.KERNEL_SDEM, len(grids), dx.ctypes.data, dy.ctypes.data,
                                           hins, 0, hous, 0, C.byref(prm)))

    step_host()
    torch.cuda.synchronize()
    c0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - c0) * 1e3 / args.steps
    assert all(torch.equal(o.cpu(), h) for o, h in zip(outs, h_out)), "host-buffer batch differs from device batch"
    lvl0, lvl1, ctas = eng.sweep_shape()
    hi = _env_int("SKE_BATCH_MAX_SIDE", 2000)
    line = {"metric": f"Batched viewshed Mpoint·sectors/s ({len(grids)} uneven DEMs 256-{hi}², 360 sect)",
            "value": cells * DIR_SECTORS / (ms / 1e3) / 1e6, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": "f32",
            "data": f"synthetic ({len(grids)} seeded diamond-square DEMs)",
            "config": {"workload": f"{len(grids)} DEMs, sides uniform 256-{hi}, roughness 0.6-0.9, Kahan accumulation",
                       "cells": cells, "sides": [int(s) for s, _, _ in spec],
                       "sweep_shape": {"lvl0": lvl0, "lvl1": lvl1, "ctas_per_sm": ctas},
                       "timed": "graph replay of the batch plan (captured on the first call)"},
            "e2e": {"value": cells * DIR_SECTORS / (e2e_ms / 1e3) / 1e6, "unit": UNIT,
                    "h2d_bytes_per_step": 4 * cells, "d2h_bytes_per_step": 4 * cells},
            "gpu_launches": int(round(launches))}
    print(json.dumps(line), flush=True)
    eng.close()
    return 0


def cepstrum_batch_workload(args):
    """Batched cepstrum blur estimation: 256 seeded 512x512 1/f^2 textures, each
    blurred by a linear motion kernel (length 5-40 px, angle 0-180 degrees) plus
    Gaussian noise sigma 0.01, 180 angles each.  The timed run is the float32
    mode (SKE_FLAG_CEPSTRUM_F32: one launch sequence for the whole batch); the
    reference's binary64 arithmetic (exact mode, bit-identical bins) is timed on
    a slice of the batch and the float32 mode's output mismatch rate against it
    is measured on 8 images.  images/s."""
    import torch
    import skewengine_gb300 as ske
    from skewengine_gb300 import build, synthetic
    build.build()
    n_img, side = _env_int("SKE_CEPSTRUM_IMAGES", 256), 512
    imgs = [torch.from_numpy(synthetic.blurred_texture(side, 4000 + i)[0]).cuda() for i in range(n_img)]
    outs = [torch.empty_like(g) for g in imgs]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng = ske.SkewEngine(side, side, stream=stream.cuda_stream)
    lib = ske.engine.load()
    dims = np.full(n_img, side, np.int32)
    ins = (C.c_void_p * n_img)(*[g.data_ptr() for g in imgs])
    ous = (C.c_void_p * n_img)(*[o.data_ptr() for o in outs])
    fast = ske.params(180, ske.DEFAULT_POVH, "reference", ske.FLAG_CEPSTRUM_F32)

    def step():
        ske.engine.check(lib.ske_run_batch(eng._h, ske.KERNEL_CEPSTRUM, n_img, dims.ctypes.data, dims.ctypes.data,
                                           ins, 1, ous, 1, C.byref(fast)))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    clocks.start()
    launches0 = eng.launch_count()
    t0.record(stream)
    for _ in range(args.steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = t0.elapsed_time(t1) / args.steps
    launches = (eng.launch_count() - launches0) / args.steps
    # End to end with pinned host images.
    h_in = [g.cpu().pin_memory() for g in imgs]
    h_out = [torch.empty(g.shape, dtype=torch.float32).pin_memory() for g in imgs]
    hins = (C.c_void_p * n_img)(*[g.data_ptr() for g in h_in])
    hous = (C.c_void_p * n_img)(*[o.data_ptr() for o in h_out])
    ske.engine.check(lib.ske_run_batch(eng._h, ske.KERNEL_CEPSTRUM, n_img, dims.ctypes.data, dims.ctypes.data,
                                       hins, 0, hous, 0, C.byref(fast)))
    c0 = time.perf_counter()
    for _ in range(args.steps):
        ske.engine.check(lib.ske_run_batch(eng._h, ske.KERNEL_CEPSTRUM, n_img, dims.ctypes.data, dims.ctypes.data,
                                           hins, 0, hous, 0, C.byref(fast)))
    e2e_ms = (time.perf_counter() - c0) * 1e3 / args.steps
    # Exact (binary64) mode on a slice, and the float32 mode's mismatch rate.
    n_exact = min(8, n_img)
    exact = ske.params(180, ske.DEFAULT_POVH, "reference", 0)
    ex_out = [torch.empty_like(g) for g in imgs[:n_exact]]
    eins = (C.c_void_p * n_exact)(*[g.data_ptr() for g in imgs[:n_exact]])
    eous = (C.c_void_p * n_exact)(*[o.data_ptr() for o in ex_out])
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    ske.engine.check(lib.ske_run_batch(eng._h, ske.KERNEL_CEPSTRUM, n_exact, dims.ctypes.data, dims.ctypes.data,
                                       eins, 1, eous, 1, C.byref(exact)))
    torch.cuda.synchronize()
    exact_ips = n_exact / (time.perf_counter() - e0)
    mism = float(np.mean([(o.cpu().numpy() != x.cpu().numpy()).mean() for o, x in zip(outs[:n_exact], ex_out)]))
    line = {"metric": "Batched cepstrum blur estimation images/s (256 x 512², 180 angles)",
            "value": n_img / (ms / 1e3), "unit": "images/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded 1/f² textures, linear motion blur 5-40 px, noise 0.01)",
            "config": {"workload": f"{n_img} x {side}x{side} textures, 180 angles, float32 mode "
                                   "(fused skew + cepstrum + max-deskew)",
                       "l2": "inputs and orientations L2-resident per image; no flush (compute-bound)"},
            "exact_mode": {"images_per_s": exact_ips, "images": n_exact,
                           "note": "binary64 operator, bit-identical to the reference"},
            "f32_output_mismatch_vs_exact": mism,
            "e2e": {"value": n_img / (e2e_ms / 1e3), "unit": "images/s",
                    "h2d_bytes_per_step": 4 * side * side * n_img, "d2h_bytes_per_step": 4 * side * side * n_img},
            "clocks": clk, "gpu_launches": int(round(launches))}
    print(json.dumps(line), flush=True)
    eng.close()
    return 0


def convs_workload(args):
    """Every 3x3 convolution of the surrogate U-Net, forward, on a batch of
    SKE_CONV_BATCH (default 256, the inference batch) 256x256 tiles: per-layer time and TFLOP/s for the
    default kernel choice (warp-specialised where it applies), the halo-staged
    kernel and the im2col kernel (ske_conv_select), CUDA events, and the whole
    set on the default choice against the measured bf16 peak."""
    import torch
    from skewengine_gb300 import _lib, build
    build.build()
    from skewengine_gb300 import surrogate as sur
    lib = _lib.load()
    n = _env_int("SKE_CONV_BATCH", 256)
    # SKE_CONV_STAGE: input channels per pipeline step of the warp-specialised kernel (0 = its own choice).
    stage = _env_int("SKE_CONV_STAGE", 0)
    assert lib.ske_conv_stage_channels(stage) == 0
    res = {"e1": 256, "e2": 128, "e3": 64, "b4": 32, "d3": 64, "d2": 128, "d1": 256}
    skip_ch = {"d3": 128, "d2": 64, "d1": 32}
    layers, total = [], {0: 0.0, 1: 0.0, 2: 0.0}
    names = {0: "ws", 1: "im2col", 2: "halo"}
    flops_all = 0.0
    g = torch.Generator(device="cuda").manual_seed(0)
    # SKE_CONV_LAYERS: comma-separated layer names to run (profiler captures); default all.
    only = [x for x in os.environ.get("SKE_CONV_LAYERS", "").split(",") if x]
    # SKE_CONV_GRAPH=0 times the eager calls (host launch work included) instead of graph replays.
    graphs = _env_int("SKE_CONV_GRAPH", 1) != 0
    for name, cin, cout in sur.LAYERS:
        if only and name not in only:
            continue
        r = res[name[:2]]
        w = (torch.randn(cout, sur.kpad(cin), device="cuda", generator=g) * 0.05).to(torch.bfloat16)
        b = torch.zeros(cout, device="cuda")
        if name[0] == "d" and name[2] == "a":
            c2 = skip_ch[name[:2]]
            low = torch.randn(n, r // 2, r // 2, cin - c2, device="cuda", generator=g).to(torch.bfloat16)
            skip = torch.randn(n, r, r, c2, device="cuda", generator=g).to(torch.bfloat16)
            fn = (lambda lo=low, sk=skip, w=w, b=b: sur.conv3x3_upcat(lo, sk, w, b, True))
        else:
            x = torch.randn(n, r, r, cin, device="cuda", generator=g).to(torch.bfloat16)
            fn = (lambda x=x, w=w, b=b: sur.conv3x3(x, w, b, True))
        flops = 2.0 * 9 * cin * cout * r * r * n
        flops_all += flops
        row = {"layer": name, "cin": cin, "cout": cout, "side": r}
        for path in (1, 2, 0):
            lib.ske_conv_select(path)
            for _ in range(max(1, args.warmup)):
                fn()
            torch.cuda.synchronize()
            run = fn
            if graphs:
                # One call captured as a CUDA graph and replayed: the layer's kernels
                # back to back without the host's per-call launch work.
                graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(graph, capture_error_mode="relaxed"):
                    fn()
                run = graph.replay
                run()
                torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                run()
            e1.record()
            torch.cuda.synchronize()
            us = e0.elapsed_time(e1) / args.steps * 1e3
            total[path] += us
            row[names[path]] = {"us": round(us, 1), "tflops": round(flops / us / 1e6, 1)}
        sur.conv_check()
        layers.append(row)
    lib.ske_conv_select(0)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"bf16_tflops": 1900.0}
    achieved = flops_all / (total[0] / 1e6) / 1e12
    line = {"metric": f"surrogate U-Net 3x3 convolutions TFLOP/s (batch {n} x 256², forward)", "value": achieved,
            "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total[0] / 1e3, "higher_is_better": True, "dtype": "bf16 (f32 accumulation)",
            "data": "synthetic (random activations and weights)",
            "config": {"workload": "the 14 convolutions of the 4-level, 32-channel U-Net, one forward pass",
                       "stage_channels": stage or "auto",
                       "timing": "CUDA graph replay of each layer's call" if graphs else "eager calls",
                       "im2col_ms": total[1] / 1e3,
                       "halo_ms": total[2] / 1e3, "layers": layers},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peaks.get("bf16_tflops", 1900.0),
                         "unit": "TFLOP/s", "frac": achieved / peaks.get("bf16_tflops", 1900.0),
                         "peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 GEMM burst) of measured"}}
    print(json.dumps(line), flush=True)
    return 0


def surrogate_workload(args):
    """Learned total-viewshed surrogate on a 4000x4000 DEM cut into 256 tiles of
    256x256: the network predicts every tile, the engine checks 5% of them and
    recomputes any checked tile off by more than 2% in total visible area.  The
    same tiles computed by the plain engine (180 angles each) are the baseline;
    the value is plain time / surrogate time (higher is better)."""
    import torch
    import skewengine_gb300 as ske
    from skewengine_gb300 import build, synthetic
    from skewengine_gb300 import surrogate as sur
    build.build()
    side = 4000
    dem = synthetic.fractal_dem(side, 4000, roughness=0.8)
    tiles, _ = sur.cut_tiles(dem)
    net = sur.load_net()
    eng = ske.SkewEngine(sur.TILE, sur.TILE)
    tdev = torch.as_tensor(np.ascontiguousarray(tiles, np.float32), device="cuda")
    truth = torch.empty_like(tdev)

    def plain():
        for i in range(len(tiles)):
            eng.run(0, tdev[i], truth[i])
        torch.cuda.synchronize()

    beng = ske.SkewEngine(sur.TILE, sur.TILE)
    truth_b = torch.empty_like(tdev)

    def plain_batched():  # every tile in one batched engine call (five launches, graph replay)
        ske.run_batch(0, tdev, engine=beng, outs=truth_b)
        torch.cuda.synchronize()

    dem_dev = torch.as_tensor(np.ascontiguousarray(dem, np.float32), device="cuda")

    def surrogate():  # device-resident like the plain arm: DEM in HBM, area map left in HBM
        out = sur.infer_dem(net, dem_dev, engine=eng, check_fraction=0.05, bound=0.02, seed=7)
        torch.cuda.synchronize()
        return out

    def timed(fn, reps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            r = fn()
        return (time.perf_counter() - t) / reps, r

    for _ in range(max(1, args.warmup)):
        surrogate()
    plain()
    plain_s, _ = timed(plain, max(1, args.steps // 2))
    plain_batched()
    plain_b_s, _ = timed(plain_batched, max(1, args.steps))
    assert torch.equal(truth, truth_b), "batched engine run differs from per-tile runs"
    sur_s, (_, stats) = timed(surrogate, args.steps)
    # accuracy of the network alone on every tile, against the engine
    x = sur.encode_tiles(tiles)
    with torch.no_grad():  # the network forward over all tiles at the inference batch (256)
        pred = net(x)
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(3):
            net(x)
        t1.record()
        torch.cuda.synchronize()
    fwd_ms = t0.elapsed_time(t1) / 3
    # The plain engine's headline throughput on this GPU (2000x2000 DEM, 360
    # directional sectors, device-resident), the reference point of the target
    # "surrogate throughput >= 10x the plain engine's".
    d2k = torch.as_tensor(synthetic.fractal_dem(SIDE, 1000, roughness=0.8), device="cuda")
    o2k = torch.empty_like(d2k)
    with ske.SkewEngine(SIDE, SIDE) as e2k:
        e2k.run(0, d2k, o2k)
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(3):
            e2k.run(0, d2k, o2k)
        torch.cuda.synchronize()
        head_s = (time.perf_counter() - t) / 3
    head_tput = SIDE * SIDE * DIR_SECTORS / head_s / 1e6
    err = sur.tile_area_error(pred, torch.log1p(truth))
    # the whole DEM's visible area (the sum over its tiles), network alone
    net_total = float(torch.expm1(pred).clamp_min(0).sum())
    true_total = float(truth.sum())
    dem_err = abs(net_total - true_total) / true_total
    flops = sur.conv_flops_per_tile() * len(tiles)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"bf16_tflops": 1900.0}
    achieved = flops / (fwd_ms / 1e3) / 1e12
    line = {"metric": "Surrogate viewshed speedup over the plain engine (4000² DEM, 256 tiles of 256², 360 sect)",
            "value": plain_s / sur_s, "unit": "x", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sur_s * 1e3, "higher_is_better": True, "dtype": "bf16 (f32 accumulation)",
            "data": "synthetic (seeded diamond-square DEM; network trained on 20000 seeded fractal tiles)",
            "config": {"workload": "4000x4000 DEM, 256x256 tiles, 5% engine spot checks, 2% fallback bound",
                       "plain_ms": plain_s * 1e3, "plain_batched_ms": plain_b_s * 1e3,
                       "speedup_vs_batched_plain": plain_b_s / sur_s, "surrogate_ms": sur_s * 1e3,
                       "surrogate_mpoint_sectors_s": side * side * DIR_SECTORS / sur_s / 1e6,
                       "plain_2000_mpoint_sectors_s": head_tput,
                       "throughput_vs_plain_2000": side * side * DIR_SECTORS / sur_s / 1e6 / head_tput,
                       "plain_mpoint_sectors_s": len(tiles) * sur.TILE ** 2 * DIR_SECTORS / plain_s / 1e6,
                       "checked_tiles": len(stats["checked"]), "fell_back": len(stats["fell_back"]),
                       "tile_area_error_median": float(np.median(err)),
                       "tile_area_error_p90": float(np.quantile(err, 0.9)),
                       "tiles_within_2pct": float(np.mean(err <= 0.02)),
                       "dem_total_area_error_network": dem_err},
            "roofline": {"bound": "tensor", "kernel": "k_conv3x3 (network forward, all tiles)",
                         "achieved": achieved, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                         "frac": achieved / peaks["bf16_tflops"],
                         "work": f"{sur.conv_flops_per_tile() / 1e9:.2f} GFLOP of 3x3 convolutions per tile",
                         "note": "forward convolutions on tcgen05 (bf16, f32 accumulator in tensor memory); "
                                 "pooling, upsampling, the fused head and the tile-context head included; "
                                 "all 256 tiles in one batch", "forward_ms": fwd_ms, "traffic": None}}
    print(json.dumps(line), flush=True)
    eng.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--side", type=int, default=SIDE,
                    help="DEM side (the metric is quoted at 2000; smaller sides are for profiling)")
    ap.add_argument("--workload", choices=["sdem", "radon", "localradon", "cepstrum", "sdem_batch", "cepstrum_batch",
                                           "surrogate", "convs"],
                    default="sdem",
                    help="sdem = the headline metric; the others are secondary measurements")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "sdem_batch":
        return batch_workload(args)
    if args.workload == "cepstrum_batch":
        return cepstrum_batch_workload(args)
    if args.workload == "convs":
        return convs_workload(args)
    if args.workload == "surrogate":
        return surrogate_workload(args)
    if args.workload != "sdem":
        return secondary_workload(args)

    import torch
    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    local = _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    import skewengine_gb300 as ske
    from skewengine_gb300 import build, synthetic
    build.build()

    side = args.side
    x = synthetic.fractal_dem(side, 1000 + rank)
    # One stream for the engine, the L2 flush and the timing events.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng = ske.SkewEngine(side, side, device=local, stream=stream.cuda_stream)
    assert eng.stream == stream.cuda_stream
    x_dev = torch.from_numpy(x).cuda()
    out_dev = torch.empty_like(x_dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):  # the flush kernel too: its first launch loads torch's module
        flush.zero_()
        eng.run(ske.KERNEL_SDEM, x_dev, out_dev)
    torch.cuda.synchronize()

    def timed_steps(profile: bool):
        """Time args.steps device-resident steps; returns (event ms, wall ms) per step."""
        eng.profile(profile)
        barrier()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        w0 = time.perf_counter()
        t0.record(stream)
        for _ in range(args.steps):
            flush.zero_()  # inputs are L2-resident (16 MB); flush between steps
            eng.run(ske.KERNEL_SDEM, x_dev, out_dev)
        t1.record(stream)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - w0) * 1e3 / args.steps
        barrier()
        return t0.elapsed_time(t1) / args.steps, wall

    clocks = ClockSampler(local)
    clocks.start()
    launches0 = eng.launch_count()
    ms, wall_ms = timed_steps(False)
    launches = eng.launch_count() - launches0
    # Per-kernel CUDA events (recorded by the engine on its stream) over a second,
    # identical pass: the sweep's launch duration for the roofline.
    prof_ms, _ = timed_steps(True)
    sweep_ms, sweep_n = eng.profile_get("sdem_sweep")
    breakdown = {k: eng.profile_get(k)[0] / args.steps for k in ("prepare", "skew", "sdem_sweep", "deskew", "reduce")}
    eng.profile(False)
    clocks.stop()
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())

    # End to end through the C ABI with pinned host buffers: H2D + compute + D2H.
    x_pin = torch.from_numpy(x).pin_memory()
    o_pin = torch.empty(x_pin.shape, dtype=torch.float32).pin_memory()
    xh, oh = x_pin.numpy(), o_pin.numpy()
    eng.run(ske.KERNEL_SDEM, xh, oh)
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        flush.zero_()
        eng.run(ske.KERNEL_SDEM, xh, oh)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    if dist is not None:
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    assert np.array_equal(oh.view(np.uint32), out_dev.cpu().numpy().view(np.uint32))

    if rank != 0:
        eng.close()
        if dist is not None:
            dist.destroy_process_group()
        return 0

    cells = side * side
    value = world * cells * DIR_SECTORS / (ms / 1e3) / 1e6
    e2e = world * cells * DIR_SECTORS / (e2e_ms / 1e3) / 1e6

    steps_total = los_steps(side, side, range(ANGLES))
    sweep_per_launch_ms = sweep_ms / max(sweep_n, 1)
    launches_per_step = max(sweep_n, 1) / args.steps
    ops_per_launch = 3.0 * steps_total / launches_per_step
    achieved = ops_per_launch / (sweep_per_launch_ms / 1e3)
    scalar_ops, packed_ops = C.c_double(), C.c_double()
    ske.engine.load().ske_measure_fp32_peak(local, C.byref(scalar_ops), C.byref(packed_ops))
    peak = max(scalar_ops.value, packed_ops.value)

    line = {
        "metric": METRIC if side == SIDE else METRIC.replace("2000²", f"{side}²"), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded diamond-square DEM, H=0.8, 0-1500 m)",
        "config": {"workload": f"total viewshed (kernelSDEM) {side}x{side} DEM, {ANGLES} angles = {DIR_SECTORS} "
                               f"directional sectors, observer 1.5 m, 10 m cells, reference accumulation order",
                   "dem": f"{side}x{side}", "sectors": DIR_SECTORS, "parallelism": f"replicas{world}",
                   "kernel_ms_per_step": breakdown, "wall_ms_per_step": wall_ms,
                   "profiled_pass_ms_per_step": prof_ms,
                   "sweep_shape": dict(zip(("lvl0", "lvl1", "ctas_per_sm"), eng.sweep_shape())),
                   "l2": f"{L2_FLUSH_BYTES >> 20} MiB written between steps (inputs {x.nbytes >> 20} MB are L2-resident)"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(x.nbytes), "d2h_bytes_per_step": int(x.nbytes),
                "ms_per_step": e2e_ms},
        "roofline": {"bound": "fp32", "kernel": "sdem_sweep", "achieved": achieved / 1e12,
                     "peak": peak / 1e12, "unit": "Tops/s (FP32 lane ops)", "frac": achieved / peak,
                     "traffic": SWEEP_DRAM_BYTES_2000 / launches_per_step if side == SIDE else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one 2000x2000 "
                                       "sweep launch",
                     "work_per_launch": ops_per_launch,
                     "work": "3 FP32 lane ops (sub, div, max) per line-of-sight step; "
                             f"{steps_total:.4g} steps per DEM",
                     "note": "work counts every line-of-sight step the reference takes; the sweep proves most "
                             "of them invisible without taking them (it executes about 22% at 2000x2000), so "
                             "frac is algorithmic work per second against the FP32 lane-op peak, not pipe "
                             "utilisation",
                     "launch_ms": sweep_per_launch_ms, "launches": int(sweep_n),
                     "peak_source": "measured on this GPU: fused multiply-add lane ops/s, best of scalar "
                                    f"({scalar_ops.value / 1e12:.2f} T) and packed f32x2 "
                                    f"({packed_ops.value / 1e12:.2f} T)"},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, kind, sample = cpu_sample(x, threads, prefer_reference=False)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample}
    print(json.dumps(line), flush=True)
    eng.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
