"""Sector sharding across ranks (one process per GPU).

The reference spreads sectors over OpenMP threads, one thread per GPU in GPU
mode (src/main.cu:86-168, src/main.h:102); each thread keeps four per-type
accumulators and folds them into the shared output inside a critical section
(``reduce``, skewEngine.cuh:862-914).  Here each rank takes a contiguous block of
angles, computes its four accumulators on its GPU, and rank 0 gathers them and
folds them in rank order: the same arithmetic as the reference run with one
thread per rank and a static schedule.  The only exchange is that one gather of
4*N floats per rank.

A batch of independent grids (ske_run_batch) shards by whole grids instead
(``shard_batch``, ``run_batch_sharded``): each rank runs its grids in one
batched call and no data crosses ranks until the optional gather of outputs.
"""
from __future__ import annotations

import numpy as np


def shard_angles(n_angles: int, world: int, rank: int, costs=None) -> list[int]:
    """Contiguous block of angles for `rank`.

    With ``costs`` (one per angle) blocks are cut so their summed costs are as
    even as possible; otherwise blocks have equal length.
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    if costs is None:
        lo = (n_angles * rank) // world
        hi = (n_angles * (rank + 1)) // world
        return list(range(lo, hi))
    c = np.cumsum(np.asarray(costs, np.float64))
    total = c[-1] if len(c) else 0.0
    cuts = [0]
    for r in range(1, world):
        cuts.append(int(np.searchsorted(c, total * r / world, side="left")) + 1)
    cuts.append(n_angles)
    cuts = np.maximum.accumulate(np.clip(cuts, 0, n_angles))
    return list(range(int(cuts[rank]), int(cuts[rank + 1])))


def sector_costs(dimx: int, dimy: int, kernel=0, max_sector: int = 180) -> np.ndarray:
    """Work of each angle 0..max_sector-1 of one operator, from the host
    geometry (ske_geometry, no device): for the total-viewshed sweep its line of
    sight steps, the sum over skewed rows of L(L-1) (kernelSDEM.h:180-218); for
    the other operators the valid skewed cells, the sum of L."""
    from .engine import KERNEL_SDEM, _kernel_id, geometry
    sdem = _kernel_id(kernel) == KERNEL_SDEM
    out = np.zeros(max_sector, np.float64)
    for a in range(max_sector):
        g = geometry(dimx, dimy, a)
        L = (g["last"] - g["first"]).astype(np.float64)
        L = L[L > 0]
        out[a] = float(np.sum(L * (L - 1.0))) if sdem else float(L.sum())
    return out


def grid_cost(dimx: int, dimy: int) -> float:
    """A grid's total-viewshed work up to a constant factor: every sector's
    skewed rows hold about dimx*dimy cells, and each cell's line of sight runs
    the length of its row (at most max(dimx, dimy)), so cells x longest row."""
    return float(dimx) * float(dimy) * float(max(dimx, dimy))


def shard_batch(shapes, world: int, rank: int) -> list[int]:
    """Indices (ascending) of the grids of a batch that `rank` runs.

    ``shapes``: one (dimy, dimx) per grid.  The grids are independent, as the
    reference's one-grid-per-program runs are (src/main.cu:86-168 per grid), so
    whole grids are dealt out: largest ``grid_cost`` first, each to the rank
    with the least cost so far (ties to the lower rank), which keeps every
    rank's share within one grid's cost of the others'.  Every rank computes
    the same assignment from the shapes alone.
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    costs = [grid_cost(int(w), int(h)) for h, w in shapes]
    load = [0.0] * world
    mine = []
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        load[r] += costs[i]
        if r == rank:
            mine.append(i)
    return sorted(mine)


def _orient_index(dimx: int, dimy: int):
    """Index of output cell (i, j) inside each orientation's accumulator."""
    i, j = np.meshgrid(np.arange(dimy), np.arange(dimx), indexing="ij")
    ci, cj = dimy - 1 - i, dimx - 1 - j
    return [(i * dimx + j).ravel(), (cj * dimy + ci).ravel(), (j * dimy + ci).ravel(), (i * dimx + cj).ravel()]


def fold_accumulators(accs, used_masks, dimx: int, dimy: int, is_max: bool = False) -> np.ndarray:
    """Fold per-rank accumulators (each 4 x N float32) into the output, rank by
    rank and type by type, exactly as successive reference ``reduce`` calls
    (skewEngine.cuh:885-912) on a zeroed output."""
    idx = _orient_index(dimx, dimy)
    out = np.zeros(dimx * dimy, np.float32)
    for acc, used in zip(accs, used_masks):
        acc = np.asarray(acc, np.float32).reshape(4, dimx * dimy)
        for t in range(4):
            if not used & (1 << t):
                continue
            v = acc[t][idx[t]]
            out = np.where(out > v, out, v) if is_max else (out + v).astype(np.float32)
    return out.reshape(dimy, dimx)


def run_sharded(engine, kernel, data, group=None, max_sector: int = 180, povh=None, accum="reference",
                balance: bool = False):
    """Run one operator with sectors sharded over a torch.distributed group.

    Every rank passes the same input; rank 0 returns the folded result, other
    ranks return None.  balance=False cuts equal-length angle blocks (the
    reference's static schedule over that many threads); balance=True cuts
    contiguous blocks of equal work (``sector_costs``), which evens out the
    ranks' time when the angles' work differs.  Either way the fold is in block
    order; the blocks differ, so in add mode the two give slightly different
    sums, as the reference's results differ with its thread count.
    """
    import torch.distributed as dist
    from .engine import DEFAULT_POVH, KERNEL_CEPSTRUM

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    costs = sector_costs(engine.dimx, engine.dimy, kernel, max_sector) if balance else None
    angles = shard_angles(max_sector, world, rank, costs)
    acc, used = engine.accumulate(kernel, data, angles, povh=DEFAULT_POVH if povh is None else povh, accum=accum)
    payload = {"acc": np.asarray(acc, np.float32), "used": int(used)}
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(payload, gathered, dst=0, group=group)
    if rank != 0:
        return None
    return fold_accumulators([g["acc"] for g in gathered], [g["used"] for g in gathered], engine.dimx,
                             engine.dimy, is_max=int(kernel) == KERNEL_CEPSTRUM)


def run_sharded_resilient(engine, kernel, data, store, rank: int, world: int, max_sector: int = 180, povh=None,
                          accum="reference", timeout: float = 60.0, poll: float = 0.01, balance: bool = False):
    """Sector sharding with failure detection and recovery on the host.

    Each rank accumulates its block of angles and posts the result under
    ``acc/<rank>`` of a shared key-value store (a ``torch.distributed.Store``:
    TCPStore, FileStore ...), or its error message under ``err/<rank>`` when its
    work raises.  Rank 0 waits for every rank: one that reports an error or posts
    nothing within ``timeout`` seconds (it died, hung or never started) is taken
    over, and rank 0 accumulates that block itself.  No collective runs on the
    data path, so a lost rank cannot block the others; the fold is in block
    order, so the result has the same bits as a run without failures.

    ``balance`` cuts the blocks as ``run_sharded`` does.

    Returns (output, recovered ranks) on rank 0 and (None, []) elsewhere.
    """
    import time
    from .engine import DEFAULT_POVH, KERNEL_CEPSTRUM

    pv = DEFAULT_POVH if povh is None else povh
    costs = sector_costs(engine.dimx, engine.dimy, kernel, max_sector) if balance else None
    blocks = [shard_angles(max_sector, world, r, costs) for r in range(world)]
    if rank != 0:
        try:
            acc, used = engine.accumulate(kernel, data, blocks[rank], povh=pv, accum=accum)
            # Raw float32 bytes and the type mask (no pickle: nothing on rank 0
            # executes what a store holds).  The accumulator key is set last.
            store.set(f"used/{rank}", str(int(used)))
            store.set(f"acc/{rank}", np.ascontiguousarray(acc, np.float32).tobytes())
        except Exception as exc:  # report, then let the caller see the failure too
            store.set(f"err/{rank}", repr(exc).encode())
            raise
        return None, []
    results = {0: engine.accumulate(kernel, data, blocks[0], povh=pv, accum=accum)}
    recovered = []
    deadline = time.monotonic() + timeout
    for r in range(1, world):
        got = None
        while got is None:
            if store.check([f"acc/{r}"]):
                got = np.frombuffer(store.get(f"acc/{r}"), np.float32)
                if got.size != 4 * engine.dimx * engine.dimy:
                    raise ValueError(f"rank {r} posted {got.size} accumulator values")
                results[r] = (got.reshape(4, -1), int(store.get(f"used/{r}")))
            elif store.check([f"err/{r}"]) or time.monotonic() > deadline:
                results[r] = engine.accumulate(kernel, data, blocks[r], povh=pv, accum=accum)
                recovered.append(r)
                break
            else:
                time.sleep(poll)
    out = fold_accumulators([results[r][0] for r in range(world)], [results[r][1] for r in range(world)],
                            engine.dimx, engine.dimy, is_max=int(kernel) == KERNEL_CEPSTRUM)
    return out, recovered


def run_batch_sharded(run_batch, kernel, grids, group=None, gather: bool = True, **kwargs):
    """Run a batch of independent grids with whole grids sharded over a
    torch.distributed group: each rank passes its shard (``shard_batch``) to
    ``run_batch(kernel, shard, **kwargs)`` — one batched engine call on its GPU,
    e.g. ``skewengine_gb300.run_batch`` (``ske_run_batch``) — and nothing is
    exchanged on the data path.  Every rank passes the same list of grids.

    gather=True: rank 0 receives every grid's output (host arrays, in the order
    of ``grids``) over the group and returns the list; other ranks return None.
    gather=False: each rank returns ``{index: output}`` for its own grids.
    """
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    mine = shard_batch([tuple(g.shape[-2:]) for g in grids], world, rank)
    outs = run_batch(kernel, [grids[i] for i in mine], **kwargs) if mine else []
    if len(outs) != len(mine):
        raise RuntimeError(f"run_batch returned {len(outs)} outputs for {len(mine)} grids")
    local = {i: o for i, o in zip(mine, outs)}
    if not gather:
        return local
    payload = {i: (o.cpu().numpy() if hasattr(o, "cpu") else np.asarray(o)) for i, o in local.items()}
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(payload, gathered, dst=0, group=group)
    if rank != 0:
        return None
    merged = {}
    for part in gathered:
        merged.update(part)
    return [merged[i] for i in range(len(grids))]


def run_batch_sharded_resilient(run_batch, kernel, grids, store, rank: int, world: int, timeout: float = 60.0,
                                poll: float = 0.01, **kwargs):
    """``run_batch_sharded`` with failure detection and recovery on the host,
    as ``run_sharded_resilient`` does for sectors.

    Each rank runs its grids (``shard_batch``) in one ``run_batch`` call and
    posts every output as raw float32 bytes under ``grid/<index>`` of the
    shared store, then ``done/<rank>``; a rank whose work raises posts its error
    under ``err/<rank>``.  Rank 0 runs its own grids, then waits for every other
    rank: one that reports an error or has not finished within ``timeout``
    seconds is taken over, and rank 0 runs that rank's grids itself (one
    batched call).  Each grid's output is computed alone, so the results have
    the same bits as a run without failures.

    Returns (outputs in the order of ``grids``, recovered ranks) on rank 0 and
    (None, []) elsewhere.
    """
    import time

    shapes = [tuple(g.shape[-2:]) for g in grids]
    shards = [shard_batch(shapes, world, r) for r in range(world)]

    def host(o):
        return np.ascontiguousarray(o.cpu().numpy() if hasattr(o, "cpu") else o, np.float32)

    def run(idx):
        outs = run_batch(kernel, [grids[i] for i in idx], **kwargs) if idx else []
        if len(outs) != len(idx):
            raise RuntimeError(f"run_batch returned {len(outs)} outputs for {len(idx)} grids")
        return {i: host(o) for i, o in zip(idx, outs)}

    if rank != 0:
        try:
            for i, o in run(shards[rank]).items():
                store.set(f"grid/{i}", o.tobytes())
            store.set(f"done/{rank}", b"1")  # set last: every grid of the rank is posted
        except Exception as exc:
            store.set(f"err/{rank}", repr(exc).encode())
            raise
        return None, []
    results = run(shards[0])
    recovered = []
    deadline = time.monotonic() + timeout
    for r in range(1, world):
        while True:
            if store.check([f"done/{r}"]):
                for i in shards[r]:
                    v = np.frombuffer(store.get(f"grid/{i}"), np.float32)
                    if v.size != shapes[i][0] * shapes[i][1]:
                        raise ValueError(f"rank {r} posted {v.size} values for grid {i}")
                    results[i] = v.reshape(shapes[i])
                break
            if store.check([f"err/{r}"]) or time.monotonic() > deadline:
                results.update(run(shards[r]))
                recovered.append(r)
                break
            time.sleep(poll)
    return [results[i] for i in range(len(grids))], recovered
