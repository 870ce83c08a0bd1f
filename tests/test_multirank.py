"""Replica sharding across ranks (world size 2, gloo on the CPU).

The GPU computation of each rank is stood in for by the FP64 oracle, so the
test checks the host side of the multi-GPU path: every curve is computed by
exactly one rank, results come back in input order on every rank, and the
timing reduce takes the slowest rank.
"""
import os
import socket
import tempfile
import threading
import time

import numpy as np
import pytest

from cuvarbase_gb300.replicas import (band_bounds, curve_cost, max_over_ranks,
                                     run_band_sharded, run_sharded, shard_bounds)


def _curves(n=7, seed=11):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        N = int(rng.integers(20, 200))
        t = np.sort(rng.uniform(0, 100, N))
        y = 0.3 * np.sin(2 * np.pi * t / (1.5 + i)) + 0.05 * rng.standard_normal(N)
        dy = np.full(N, 0.05)
        out.append((t, y, dy))
    return out


FREQS = 0.01 * (1 + np.arange(64))


def _gls(part):
    from oracle import oracle as O
    res = []
    for t, y, dy in part:
        tt, yw, w, YY, _ = O.prepare_curve(t, y, dy)
        res.append(O.gls_flmean_np(tt, yw, w, FREQS, YY))
    return res


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}",
                            rank=rank, world_size=world)
    try:
        data = _curves()
        seen = []

        def fn(part):
            seen.extend(len(p[0]) for p in part)
            return _gls(part)

        res = run_sharded(fn, data, freqs=FREQS)
        # results that are still being written when fn returns (as the GPU
        # writes run()'s page-locked views): correct only because sync runs
        # before the gather
        pending = []

        def fn_async(part):
            out = [np.zeros(len(FREQS)) for _ in part]

            def fill():
                time.sleep(0.3)
                for o, r in zip(out, _gls(part)):
                    o[:] = r
            th = threading.Thread(target=fill)
            th.start()
            pending.append(th)
            return out

        res_async = run_sharded(fn_async, data, nf=len(FREQS),
                                sync=lambda: [th.join() for th in pending])
        np.save(os.path.join(outdir, f"async{rank}.npy"), np.stack(res_async))
        np.save(os.path.join(outdir, f"res{rank}.npy"), np.stack(res))
        np.save(os.path.join(outdir, f"seen{rank}.npy"), np.array(seen, dtype=np.int64))
        np.save(os.path.join(outdir, f"max{rank}.npy"), np.array([max_over_ranks(10.0 + rank)]))
        # one curve, its band split by frequency across the ranks
        t, y, dy = data[3]
        band = 0.004 * (7 + np.arange(101))    # f_k = df (k0 + k), k0 = 7, odd nf

        def fn_band(t_, y_, dy_, f):
            from oracle import oracle as O
            tt, yw, w, YY, _ = O.prepare_curve(t_, y_, dy_)
            return O.gls_flmean_np(tt, yw, w, f, YY)

        np.save(os.path.join(outdir, f"band{rank}.npy"),
                run_band_sharded(fn_band, t, y, dy, band))
    finally:
        dist.destroy_process_group()


def test_shard_bounds_cover_in_order():
    rng = np.random.default_rng(0)
    for world in (1, 2, 3, 4, 8):
        for n in (0, 1, 5, 40):
            costs = rng.uniform(0, 10, n)
            b = shard_bounds(costs, world)
            assert len(b) == world
            assert b[0][0] == 0 and b[-1][1] == n
            for (s0, e0), (s1, e1) in zip(b, b[1:]):
                assert e0 == s1 and s0 <= e0
    # balanced by cost: one huge item takes a rank of its own
    b = shard_bounds([1, 1, 100, 1, 1], 2)
    assert b == [(0, 3), (3, 5)] or b == [(0, 2), (2, 5)]
    assert shard_bounds([0, 0, 0, 0], 2) == [(0, 2), (2, 4)]
    with pytest.raises(ValueError):
        shard_bounds([1.0], 0)


def test_band_bounds_cover_in_order():
    for world in (1, 2, 3, 8):
        for nf in (0, 1, 7, 100_001):
            b = band_bounds(nf, world)
            assert b[0][0] == 0 and b[-1][1] == nf and len(b) == world
            assert all(e0 == s1 for (_, e0), (s1, _) in zip(b, b[1:]))
            assert max(e - s for s, e in b) - min(e - s for s, e in b) <= 1


def test_curve_cost_monotone():
    assert curve_cost(100, 1000) < curve_cost(200, 1000) < curve_cost(200, 2000)


def test_default_costs_count_frequencies():
    """The default shard cost includes each curve's frequency count."""
    from cuvarbase_gb300.replicas import _n_freqs
    from cuvarbase_gb300.utils import autofrequency
    data = _curves(3)
    assert _n_freqs(data, None, 500) == [500] * 3
    assert _n_freqs(data, None, [1, 2, 3]) == [1, 2, 3]
    assert _n_freqs(data, FREQS, None) == [len(FREQS)] * 3
    assert _n_freqs(data, [FREQS, FREQS[:10], FREQS[:5]], None) == [len(FREQS), 10, 5]
    assert _n_freqs(data, None, None) == [len(autofrequency(d[0])) for d in data]
    # a curve with few points but a huge grid gets a rank of its own
    costs = [curve_cost(10, k) for k in (100, 100, 10 ** 6, 100)]
    assert shard_bounds(costs, 2)[0][1] in (2, 3)


def test_two_ranks_gloo():
    import torch.multiprocessing as mp
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_worker, args=(2, _free_port(), d), nprocs=2, join=True,
                           start_method="spawn")
        ref = np.stack(_gls(_curves()))
        seen = [np.load(os.path.join(d, f"seen{r}.npy")) for r in range(2)]
        for r in range(2):
            np.testing.assert_array_equal(np.load(os.path.join(d, f"res{r}.npy")), ref)
            np.testing.assert_array_equal(np.load(os.path.join(d, f"async{r}.npy")), ref)
            assert float(np.load(os.path.join(d, f"max{r}.npy"))[0]) == 11.0
        t, y, dy = _curves()[3]
        from oracle import oracle as O
        tt, yw, w, YY, _ = O.prepare_curve(t, y, dy)
        whole = O.gls_flmean_np(tt, yw, w, 0.004 * (7 + np.arange(101)), YY)
        for r in range(2):
            np.testing.assert_allclose(np.load(os.path.join(d, f"band{r}.npy")), whole,
                                       rtol=0, atol=1e-12)
        # each curve computed by exactly one rank, both ranks did work
        assert sum(len(s) for s in seen) == len(_curves())
        assert all(len(s) > 0 for s in seen)
