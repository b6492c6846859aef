"""Synthetic inputs and the host side of sector sharding (CPU only).

The multi-rank test runs two gloo ranks; each rank's "GPU" is stood in for by
the CPU oracle through a fake engine, so only the product's sharding, gather and
fold logic is under test.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from skewengine_gb300 import parallel, synthetic
from tests.conftest import bits_equal


def test_fractal_dem_deterministic_and_scaled():
    a = synthetic.fractal_dem(100, 7)
    b = synthetic.fractal_dem(100, 7)
    c = synthetic.fractal_dem(100, 8)
    assert a.dtype == np.float32 and a.shape == (100, 100)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() == 0.0 and abs(a.max() - 150.0) < 1e-3  # 1500 m / 10 m cells
    assert synthetic.fractal_dem(48, 3, side_y=20).shape == (20, 48)


def test_phantom_and_texture():
    p = synthetic.ellipse_phantom(64, 1)
    assert p.shape == (64, 64) and p.dtype == np.float32 and np.abs(p).max() > 0
    t, length, ang = synthetic.blurred_texture(64, 2)
    assert t.shape == (64, 64) and 5 <= length <= 40 and 0 <= ang < 180
    k = synthetic.motion_kernel(10.0, 30.0)
    assert abs(k.sum() - 1.0) < 1e-12


def test_uneven_batch_spec():
    spec = synthetic.uneven_dem_batch(64, 100)
    assert len(spec) == 64
    assert all(256 <= s <= 2000 and 0.6 <= h <= 0.9 for s, h, _ in spec)
    assert [s for _, _, s in spec] == list(range(100, 164))


def test_shard_angles_partition():
    for world in (1, 2, 3, 4, 7, 8):
        got = sum((parallel.shard_angles(180, world, r) for r in range(world)), [])
        assert got == list(range(180))
    costs = np.linspace(1, 10, 180)
    blocks = [parallel.shard_angles(180, 4, r, costs) for r in range(4)]
    assert sum(blocks, []) == list(range(180))
    sums = [costs[b].sum() for b in blocks]
    assert max(sums) / min(sums) < 1.2


def test_fold_max_mode():
    acc = np.zeros((4, 6), np.float32)
    acc[0] = [1, 5, 3, 0, 0, 0]
    acc[3] = [2, 2, 2, 2, 2, 2]
    out = parallel.fold_accumulators([acc], [0b1001], 3, 2, is_max=True)
    assert out.shape == (2, 3) and out.max() == 5


class _OracleEngine:
    """Stands in for SkewEngine on a CPU-only rank: accumulate() via the oracle."""

    def __init__(self, oracle, dimx, dimy):
        self.oracle, self.dimx, self.dimy = oracle, dimx, dimy

    def accumulate(self, kernel, data, angles, povh, accum="reference"):
        return self.oracle.accumulate(kernel, data, angles, povh=povh)


def _rank_main(rank, world, port_path, x, port_expect, result_path, master_port, balance=False):
    import ctypes as C
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(master_port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lib = C.CDLL(port_path)
    from tests.conftest import PortOracle
    fp = np.ctypeslib.ndpointer(np.float32, flags="C")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C")
    lib.port_accumulate.argtypes = [C.c_int, fp, C.c_int, C.c_int, ip, C.c_int, C.c_float, fp, ip]
    eng = _OracleEngine(PortOracle(lib), x.shape[1], x.shape[0])
    out = parallel.run_sharded(eng, 0, x, povh=np.float32(0.15), balance=balance)
    if rank == 0:
        np.save(result_path, out)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharded_run(oracle, port, tmp_path):
    import torch.multiprocessing as mp
    x = synthetic.fractal_dem(40, 5)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        master_port = s.getsockname()[1]
    port_path = port._name
    res = str(tmp_path / "out.npy")
    mp.start_processes(_rank_main, args=(2, port_path, x, None, res, master_port), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(res)
    # Same arithmetic as two reference threads with a static schedule:
    a0, u0 = oracle.accumulate(0, x, list(range(0, 90)), povh=np.float32(0.15))
    a1, u1 = oracle.accumulate(0, x, list(range(90, 180)), povh=np.float32(0.15))
    want = parallel.fold_accumulators([a0, a1], [u0, u1], 40, 40)
    assert bits_equal(got, want)
    single = oracle.run(0, x, povh=np.float32(0.15))
    np.testing.assert_allclose(got, single, rtol=1e-5)


def test_sector_costs_balance_the_shards(port):
    """sector_costs: each angle's line-of-sight steps from the host geometry
    (their sum is the oracle's count for the grid); cutting blocks by them
    evens out a non-square grid's ranks, which equal-length blocks do not."""
    costs = parallel.sector_costs(200, 120, 0)
    assert abs(costs.sum() - port.port_los_steps(200, 120, 180)) <= 1e-9 * costs.sum()
    cells = parallel.sector_costs(200, 120, "radon")
    assert (cells > 0).all() and cells.sum() < costs.sum()
    for world in (3, 4, 8):
        equal = [costs[parallel.shard_angles(180, world, r)].sum() for r in range(world)]
        blocks = [parallel.shard_angles(180, world, r, costs) for r in range(world)]
        assert sum(blocks, []) == list(range(180))
        even = [costs[b].sum() for b in blocks]
        assert max(even) / np.mean(even) < min(1.1, max(equal) / np.mean(equal)), (world, equal, even)


def test_two_rank_sharded_run_balanced(oracle, port, tmp_path):
    """Two gloo ranks with work-balanced angle blocks: the fold of the two
    blocks the cost cut gives, bit for bit."""
    import torch.multiprocessing as mp
    x = synthetic.fractal_dem(48, 6, side_y=30)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        master_port = s.getsockname()[1]
    res = str(tmp_path / "out.npy")
    mp.start_processes(_rank_main, args=(2, port._name, x, None, res, master_port, True), nprocs=2, join=True,
                       start_method="spawn")
    costs = parallel.sector_costs(48, 30, 0)
    blocks = [parallel.shard_angles(180, 2, r, costs) for r in range(2)]
    assert blocks[0] != list(range(90))  # the cut moved off the equal split
    parts = [oracle.accumulate(0, x, b, povh=np.float32(0.15)) for b in blocks]
    want = parallel.fold_accumulators([p[0] for p in parts], [p[1] for p in parts], 48, 30)
    assert bits_equal(np.load(res), want)


class _FailingEngine(_OracleEngine):
    def accumulate(self, *a, **k):
        raise RuntimeError("injected failure of this rank's sectors")


def _resilient_main(rank, world, port_path, x, result_path, store_port, mode):
    import ctypes as C
    import json
    from datetime import timedelta
    import torch.distributed as dist
    if mode == "fail" and rank == 2:
        return  # dies before contributing anything
    store = dist.TCPStore("127.0.0.1", store_port, world, rank == 0, timedelta(seconds=60), wait_for_workers=False)
    lib = C.CDLL(port_path)
    from tests.conftest import PortOracle
    fp = np.ctypeslib.ndpointer(np.float32, flags="C")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C")
    lib.port_accumulate.argtypes = [C.c_int, fp, C.c_int, C.c_int, ip, C.c_int, C.c_float, fp, ip]
    cls = _FailingEngine if (mode == "fail" and rank == 1) else _OracleEngine
    eng = cls(PortOracle(lib), x.shape[1], x.shape[0])
    try:
        out, recovered = parallel.run_sharded_resilient(eng, 0, x, store, rank, world, povh=np.float32(0.15),
                                                        timeout=5.0)
    except RuntimeError:
        assert mode == "fail" and rank == 1
        return
    if rank == 0:
        np.save(result_path, out)
        with open(result_path + ".json", "w") as f:
            json.dump(recovered, f)


@pytest.mark.parametrize("mode", ["ok", "fail"])
def test_resilient_sharding_recovers_failed_ranks(oracle, port, tmp_path, mode):
    """Three CPU ranks; with mode "fail" rank 1 raises inside its work and rank 2
    exits before contributing.  Rank 0 detects both on the host (an error key,
    a deadline) and runs their sectors itself; the output has the same bits as
    the run without failures."""
    import json
    import torch.multiprocessing as mp
    x = synthetic.fractal_dem(36, 8)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        store_port = s.getsockname()[1]
    res = str(tmp_path / "out.npy")
    mp.start_processes(_resilient_main, args=(3, port._name, x, res, store_port, mode), nprocs=3, join=True,
                       start_method="spawn")
    got = np.load(res)
    blocks = [parallel.shard_angles(180, 3, r) for r in range(3)]
    parts = [oracle.accumulate(0, x, b, povh=np.float32(0.15)) for b in blocks]
    want = parallel.fold_accumulators([p[0] for p in parts], [p[1] for p in parts], 36, 36)
    assert bits_equal(got, want)
    with open(res + ".json") as f:
        assert json.load(f) == ([1, 2] if mode == "fail" else [])


def test_shard_batch_partition():
    """Whole grids dealt out largest first to the least-loaded rank: every grid
    on exactly one rank, the same answer on every rank, and every rank's cost
    within the largest grid's cost of every other's."""
    shapes = [(s, s) for s, _, _ in synthetic.uneven_dem_batch(64, 3000)] + [(300, 500), (480, 270)]
    for world in (1, 2, 3, 4, 8):
        parts = [parallel.shard_batch(shapes, world, r) for r in range(world)]
        assert sorted(sum(parts, [])) == list(range(len(shapes)))
        assert parts == [parallel.shard_batch(shapes, world, r) for r in range(world)]
        loads = [sum(parallel.grid_cost(w, h) for i, (h, w) in enumerate(shapes) if i in p) for p in parts]
        assert max(loads) - min(loads) <= max(parallel.grid_cost(w, h) for h, w in shapes)
    assert parallel.shard_batch([], 2, 1) == []
    with pytest.raises(ValueError):
        parallel.shard_batch(shapes, 2, 2)


def _batch_rank_main(rank, world, port_path, grids, result_path, master_port):
    import ctypes as C
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(master_port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lib = C.CDLL(port_path)
    from tests.conftest import PortOracle
    fp = np.ctypeslib.ndpointer(np.float32, flags="C")
    lib.port_run.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int]
    oracle = PortOracle(lib)
    seen = []

    def batch(kernel, shard, povh):  # stands in for run_batch: one call per rank
        seen.append(len(shard))
        return [oracle.run(kernel, g, povh=povh) for g in shard]

    out = parallel.run_batch_sharded(batch, 0, grids, povh=np.float32(0.15))
    own = parallel.run_batch_sharded(batch, 0, grids, gather=False, povh=np.float32(0.15))
    assert seen[0] == seen[1] == len(own) and set(own) == set(parallel.shard_batch(
        [g.shape for g in grids], world, rank))
    if rank == 0:
        np.savez(result_path, *out)
    else:
        assert out is None
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_batch_sharded(oracle, port, tmp_path):
    """Independent grids of uneven size split over two gloo ranks, one batched
    call per rank, gathered on rank 0 in input order: bit-identical to running
    every grid alone."""
    import torch.multiprocessing as mp
    grids = [synthetic.fractal_dem(s, 40 + s, roughness=0.7) for s in (24, 40, 17, 33)]
    grids.append(synthetic.fractal_dem(30, 7)[:, :21].copy())
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        master_port = s.getsockname()[1]
    res = str(tmp_path / "outs.npz")
    mp.start_processes(_batch_rank_main, args=(2, port._name, grids, res, master_port), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(res)
    assert len(got.files) == len(grids)
    for k, g in enumerate(grids):
        assert bits_equal(got[f"arr_{k}"], oracle.run(0, g, povh=np.float32(0.15))), k


def _batch_resilient_main(rank, world, port_path, grids, result_path, store_port, mode):
    import ctypes as C
    import json
    from datetime import timedelta
    import torch.distributed as dist
    if mode == "fail" and rank == 2:
        return  # dies before contributing anything
    store = dist.TCPStore("127.0.0.1", store_port, world, rank == 0, timedelta(seconds=60), wait_for_workers=False)
    lib = C.CDLL(port_path)
    from tests.conftest import PortOracle
    fp = np.ctypeslib.ndpointer(np.float32, flags="C")
    lib.port_run.argtypes = [C.c_int, fp, fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int]
    oracle = PortOracle(lib)

    def batch(kernel, shard, povh):
        if mode == "fail" and rank == 1:
            raise RuntimeError("injected failure of this rank's grids")
        return [oracle.run(kernel, g, povh=povh) for g in shard]

    try:
        outs, recovered = parallel.run_batch_sharded_resilient(batch, 0, grids, store, rank, world, timeout=5.0,
                                                               povh=np.float32(0.15))
    except RuntimeError:
        assert mode == "fail" and rank == 1
        return
    if rank == 0:
        np.savez(result_path, *outs)
        with open(result_path + ".json", "w") as f:
            json.dump(recovered, f)


@pytest.mark.parametrize("mode", ["ok", "fail"])
def test_resilient_batch_sharding_recovers_failed_ranks(oracle, port, tmp_path, mode):
    """Three CPU ranks share a batch of uneven grids; with mode "fail" rank 1
    raises inside its batched call and rank 2 exits before contributing.  Rank 0
    detects both on the host (an error key, a deadline) and runs their grids
    itself; every output has the same bits as the grid run alone."""
    import json
    import torch.multiprocessing as mp
    grids = [synthetic.fractal_dem(s, 60 + s, roughness=0.75) for s in (20, 31, 26, 18, 35, 23)]
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        store_port = s.getsockname()[1]
    res = str(tmp_path / "outs.npz")
    mp.start_processes(_batch_resilient_main, args=(3, port._name, grids, res, store_port, mode), nprocs=3,
                       join=True, start_method="spawn")
    got = np.load(res)
    for k, g in enumerate(grids):
        assert bits_equal(got[f"arr_{k}"], oracle.run(0, g, povh=np.float32(0.15))), k
    with open(res + ".json") as f:
        assert json.load(f) == ([1, 2] if mode == "fail" else [])
