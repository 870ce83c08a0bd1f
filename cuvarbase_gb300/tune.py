"""Run-time grid-shape tuner for the GLS plans.

The planner chooses each plan's grid shape G1 x G2 from pass costs per
grid cell measured once on GB300 (``kPass1PsPerCell`` / ``kPass2PsPerCell``
in ``csrc/plan_rules.h``).  Pass 1 also pays per point, so the best shape
shifts with the caller's point counts; :func:`autotune` times every shape the
planner weighs (``cuvgls_plan_shapes``: all that fit and are at most 10 %
above the smallest grid) on the caller's own curves and pins the fastest on
the handle (``cuvgls_plan_pin``), so later batches with that frequency count
use it.  The window, sigma and m stay the planner's.  No reference
counterpart: cuvarbase sizes its grids as sigma * nf for cuFFT
(cuvarbase/lombscargle.py:154-181).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .lombscargle import _grid_df, get_k0

__all__ = ["autotune"]


def _raw_input(data, nf, k0, df, mode):
    """A RawInput over (t, y, dy) curves, each with nf frequencies
    (k0 + k) df, host input and host output; returns (input, keep-alive)."""
    n = np.fromiter((len(d[0]) for d in data), np.int64, len(data))
    off = np.zeros(len(data) + 1, np.int64)
    off[1:] = np.cumsum(n)
    t = np.concatenate([np.asarray(d[0], np.float64) for d in data])
    y = np.concatenate([np.asarray(d[1], np.float64) for d in data])
    dy = np.concatenate([np.asarray(d[2], np.float64) for d in data])
    curves = (_lib.RawCurve * len(data))()
    for i in range(len(data)):
        c = curves[i]
        c.pt_off, c.n, c.nf, c.k0 = int(off[i]), int(n[i]), int(nf), int(k0[i])
        c.df, c.out_off = float(df[i]), i * int(nf)
    inp = _lib.RawInput()
    inp.n_curves, inp.mode = len(data), int(mode)
    inp.curves = ctypes.cast(curves, ctypes.c_void_p)
    inp.t, inp.y, inp.dy = t.ctypes.data, y.ctypes.data, dy.ctypes.data
    inp.reg[0], inp.reg[1], inp.reg[2] = 0.0, 0.0, 0.0
    inp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
    inp.n_points_total, inp.n_out_total = int(off[-1]), len(data) * int(nf)
    out = np.empty(len(data) * int(nf), np.float32)
    return inp, (curves, t, y, dy, out)


def autotune(handle, data, freqs, steps=3, max_shapes=8, pin=True, mode=1):
    """Time the grid shapes the planner weighs for the band ``freqs`` on the
    curves ``data`` ([(t, y, dy)], every curve on a grid of len(freqs)
    frequencies, or ``freqs`` a list with one grid of that length per curve)
    and, with ``pin``, pin the fastest on ``handle`` (a ``_lib.Handle``).

    Each shape is timed by the library's CUDA events around its kernels
    (preparation and both passes, ``steps`` calls after one warm-up call), so
    the host copies of the timing calls do not count.  Returns the shapes
    fastest first as dicts {"G1", "G2", "ms"} (kernel ms per call).
    """
    if not data:
        raise ValueError("autotune needs at least one curve")
    grids = freqs if isinstance(freqs, (list, tuple)) else [freqs] * len(data)
    if len(grids) != len(data):
        raise ValueError("one frequency grid per curve")
    nf = len(grids[0])
    if any(len(g) != nf for g in grids):
        raise ValueError("autotune tunes one frequency count: every grid needs the same length")
    k0 = [get_k0(np.asarray(g)) for g in grids]
    df = [_grid_df(np.asarray(g)) for g in grids]
    shapes = handle.plan_shapes(nf, max_shapes)
    if not shapes:
        raise ValueError(f"no grid plan for nf={nf}")
    inp, keep = _raw_input(data, nf, k0, df, mode)
    out = keep[-1]
    L = _lib.load()
    results = []
    try:
        for G1, G2 in shapes:
            handle.plan_pin(nf, G1, G2)
            handle.check(L.cuvgls_gls_raw(handle.ptr, ctypes.byref(inp), out.ctypes.data,
                                          None, None, None), "autotune warm-up")
            handle.sync(None, -1)
            handle.profile(True)
            for _ in range(int(steps)):
                handle.check(L.cuvgls_gls_raw(handle.ptr, ctypes.byref(inp), out.ctypes.data,
                                              None, None, None), "autotune")
            handle.sync(None, -1)
            prof = handle.profile_read()
            handle.profile(False)
            ms = sum(prof[k][1] for k in ("prep", "pass1", "pass2")) / max(int(steps), 1)
            results.append({"G1": G1, "G2": G2, "ms": ms})
    finally:
        handle.plan_pin(nf, 0, 0)
    results.sort(key=lambda r: r["ms"])
    if pin:
        handle.plan_pin(nf, results[0]["G1"], results[0]["G2"])
    return results
