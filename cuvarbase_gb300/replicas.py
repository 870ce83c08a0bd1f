"""Replica sharding of independent light curves, one process per GPU.

The GLS / adjoint-NFFT path has no exchange step: every light curve is
independent (cuvarbase runs them one after another, `cuvarbase/core.py:42-56`,
`cuvarbase/lombscargle.py:923-1010`).  N GPUs therefore run N replicas, each on
a contiguous share of the curves balanced by cost, and the results are
gathered on the host.  Nothing but the results (and, for timing, one scalar)
crosses ranks.

    import torch.distributed as dist
    dist.init_process_group("nccl")          # or "gloo"
    proc = LombScargleAsyncProcess()
    results = run_sharded(lambda part: proc.run(part, freqs=freqs), data,
                          freqs=freqs, sync=proc.finish)

``run`` returns views of page-locked buffers that the GPU fills
asynchronously, so ``sync`` (here ``finish``) must run before the results are
gathered; ``run_sharded`` calls it between ``fn`` and the gather.

A single curve whose band is too wide for one GPU splits by frequency
instead (``run_band_sharded``): each rank computes a contiguous slice of the
grid, and the slices are gathered in order.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


def curve_cost(n_points: int, nf: int) -> float:
    """Relative cost of one curve: bytes moved by the batched path, about
    40 per point (records) plus 52 per frequency (grids and output)."""
    return 40.0 * n_points + 52.0 * nf


def shard_bounds(costs: Sequence[float], world: int) -> list[tuple[int, int]]:
    """Contiguous [start, end) ranges, one per rank, of about equal total cost.

    Every item lands in exactly one range and the ranges are in order, so
    concatenating the ranks' results restores the input order.
    """
    if world < 1:
        raise ValueError("world must be >= 1")
    n = len(costs)
    c = np.asarray(costs, dtype=np.float64)
    if n and (c < 0).any():
        raise ValueError("costs must be non-negative")
    cum = np.concatenate([[0.0], np.cumsum(c)])
    total = cum[-1]
    bounds = []
    start = 0
    for r in range(world):
        if r == world - 1:
            end = n
        elif total <= 0:
            end = min(n, (r + 1) * n // world)
        else:
            # first index whose prefix reaches this rank's share
            end = int(np.searchsorted(cum, total * (r + 1) / world, side="left"))
            end = min(max(end, start), n)
        bounds.append((start, end))
        start = end
    return bounds


def _dist():
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        raise RuntimeError("torch.distributed is not initialised")
    return dist


def _n_freqs(data, freqs, nf):
    """Frequencies per item: ``nf`` (one count or one per item), else the
    length of ``freqs`` (one grid or one per item), else the reference's
    default grid (utils.autofrequency of the item's times)."""
    if nf is not None:
        return list(nf) if np.ndim(nf) else [int(nf)] * len(data)
    if freqs is not None:
        if len(freqs) and np.ndim(freqs[0]) == 0:
            return [len(freqs)] * len(data)
        return [len(f) for f in freqs]
    from .utils import autofrequency
    return [len(autofrequency(d[0])) for d in data]


def run_sharded(fn: Callable[[list], Sequence], data: Sequence, group=None,
                costs: Sequence[float] | None = None, sync: Callable[[], object] | None = None,
                freqs=None, nf=None) -> list:
    """Run ``fn`` on this rank's share of ``data``; return all results, in order.

    ``fn`` maps a list of items to a list of results of the same length (as
    ``LombScargleAsyncProcess.run`` does).  ``sync`` (e.g. the process's
    ``finish``) is called after ``fn`` and before the results leave the rank:
    results that the GPU is still writing must not be gathered.  ``costs``
    defaults to ``curve_cost`` of each ``(t, y, dy)`` item with its frequency
    count from ``nf`` or ``freqs`` (see ``_n_freqs``).  Every rank returns
    the full list.
    """
    dist = _dist()
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    if costs is None:
        nfs = _n_freqs(data, freqs, nf)
        costs = [curve_cost(len(d[0]), k) for d, k in zip(data, nfs)]
    if len(costs) != len(data):
        raise ValueError("one cost per item")
    lo, hi = shard_bounds(costs, world)[rank]
    local = list(fn(list(data[lo:hi]))) if hi > lo else []
    if sync is not None:
        sync()
    if len(local) != hi - lo:
        raise ValueError(f"fn returned {len(local)} results for {hi - lo} items")
    parts = [None] * world
    dist.all_gather_object(parts, (lo, local), group=group)
    out = [None] * len(data)
    for start, res in parts:
        out[start:start + len(res)] = res
    return out


def band_bounds(nf: int, world: int) -> list[tuple[int, int]]:
    """Contiguous [start, end) slices of nf frequencies, one per rank, equal
    to within one frequency."""
    if world < 1:
        raise ValueError("world must be >= 1")
    return [(r * nf // world, (r + 1) * nf // world) for r in range(world)]


def run_band_sharded(fn: Callable, t, y, dy, freqs, group=None,
                     sync: Callable[[], object] | None = None):
    """The periodogram of ONE light curve over a grid split by frequency:
    rank r computes ``fn(t, y, dy, freqs[lo:hi])`` for its contiguous slice
    (a slice of f_k = df (k0 + k) is itself such a grid, with first index
    k0 + lo), ``sync`` runs before the gather, and every rank returns the
    powers of the whole grid, in order.  For a curve whose band alone fills
    a GPU (the sub-bands of the library's wide-band split, spread over
    GPUs instead of run one after another); the points are not split.

        run_band_sharded(lambda t, y, dy, f: proc.run([(t, y, dy)], freqs=f)[0][1],
                         t, y, dy, freqs, sync=proc.finish)
    """
    dist = _dist()
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    freqs = np.asarray(freqs)
    lo, hi = band_bounds(len(freqs), world)[rank]
    local = np.asarray(fn(t, y, dy, freqs[lo:hi])) if hi > lo else np.empty(0)
    if sync is not None:
        sync()
    local = np.array(local, copy=True)  # results may be views of buffers reused later
    if len(local) != hi - lo:
        raise ValueError(f"fn returned {len(local)} powers for {hi - lo} frequencies")
    parts = [None] * world
    dist.all_gather_object(parts, (lo, local), group=group)
    out = np.empty(len(freqs), dtype=local.dtype if len(local) else np.float32)
    for start, res in parts:
        out[start:start + len(res)] = res
    return out


def max_over_ranks(value: float, group=None) -> float:
    """Largest ``value`` over the ranks (the timing rule: slowest replica)."""
    dist = _dist()
    import torch
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
