"""Continuous-batching GLS server (Python front end of cuvgls_server_*).

Requests (one light curve and its frequency grid each) arrive on any thread
with ``submit``.  The library prepares each one on the submitting thread
(nan-means removed, weights, ybar, yw, YY, as LombScargleMemory.setdata does)
and queues it; its loop thread admits queued requests under the HBM budget
into the next free slot and runs everything admitted as one batched
``cuvgls_gls_batch`` call.  ``inflight`` slots (one handle, stream and
``hbm_budget / inflight`` workspace each) keep batches in flight at once, so
requests that arrive while one batch runs are admitted into the next batch,
which overlaps it on the device; a request's budget is returned when its
batch completes.  A request larger than one slot's share is rejected with
MemoryError.

A poll thread here resolves the futures.  Results are read straight from the
slot's page-locked result buffer: ``on_result(freqs, power)`` receives a view
that is valid during the call (streaming consumers, no copy); without it the
future resolves to ``(freqs, power)`` with a private copy.  Latency is
measured from the request's arrival (``arrival=`` perf_counter time, e.g. its
scheduled arrival, else the submit call) to the delivery of its result
(``latencies``), and to the moment the library had the result in page-locked
host memory (``ready_latencies``: the submit call's start plus the library's
own submit-to-completion time), which excludes the Python delivery.  The
two parts of the latter are kept as well: ``lags`` (arrival to the submit
call, the client's own delay) and ``lib_latencies`` (submit call to
completion, in the library).

There is no reference counterpart (cuvarbase runs one synchronous batch per
call); the GLS arithmetic is that of ``cuvgls_gls_batch``.
"""
from __future__ import annotations

import ctypes
import itertools
import threading
import time
from concurrent.futures import Future

import numpy as np

from . import _lib
from .lombscargle import _grid_df, check_k0, get_k0


class GLSServer:
    """Serve floating-mean GLS periodograms with continuous batching.

    Parameters
    ----------
    sigma, m : grid oversampling and Gaussian half-width ('auto' autotunes
        the window too)
    hbm_budget : bytes of device memory the requests in flight may use
    max_batch : most requests in one batch
    device : CUDA device ordinal
    inflight : batches in flight at once
    warm : (nf_min, nf_max) -- build the grid tables of every plan in that
        range and reserve each slot's workspace at creation, so that nothing
        is allocated or built while requests wait
    stage_points, stage_results : page-locked staging per slot (points and
        powers); a batch is admitted within them
    """

    _POLL = 256

    def __init__(self, sigma="auto", m=8, hbm_budget=80 << 30, max_batch=4096,
                 device=0, inflight=2, warm=None, stage_points=16 << 20,
                 stage_results=64 << 20):
        L = _lib.load()
        sig = -1.0 if sigma == "auto" else float(sigma)
        self.hbm_budget = int(hbm_budget)
        self.max_batch = int(max_batch)
        wlo, whi = (0, 0) if warm is None else (int(warm[0]), int(warm[1]))
        o = _lib.ServerOpts(sig, int(m), int(device), self.hbm_budget, self.max_batch,
                            int(inflight), _lib.PREC_MIXED, _lib.MODE_FLOATING_MEAN, 0.0, 0,
                            wlo, whi, int(stage_points), int(stage_results))
        ptr = ctypes.c_void_p()
        _lib.raise_for(L.cuvgls_server_create(ctypes.byref(ptr), ctypes.byref(o)),
                       what="server create")
        self._srv = ptr
        self._L = L
        self._ids = itertools.count(1)
        self._pending = {}
        self._plock = threading.Lock()
        self.latencies = []
        self.ready_latencies = []
        self.lib_latencies = []   # submit call to completion, in the library
        self.lags = []            # arrival to the submit call
        self.rejected = 0
        self._base = (0, 0)
        self._final = None
        self.slot_budget = int(self._counts()[5])
        n = self._POLL
        self._buf = ((ctypes.c_int64 * n)(), (ctypes.c_int32 * n)(),
                     (ctypes.c_void_p * n)(), (ctypes.c_int64 * n)(), (ctypes.c_double * n)())
        self._closed = False
        self._inflight = int(inflight)
        self._views = self._slot_views()
        self._thread = threading.Thread(target=self._deliver, daemon=True)
        self._thread.start()

    # ------------------------------------------------------------------
    def _counts(self):
        c = (ctypes.c_int64 * 8)()
        _lib.raise_for(self._L.cuvgls_server_stats(self._srv, c), what="server stats")
        return list(c)

    def request_bytes(self, n, nf):
        """Device bytes one request occupies while in flight."""
        out = ctypes.c_int64()
        _lib.raise_for(self._L.cuvgls_server_request_bytes(self._srv, int(n), int(nf),
                                                            ctypes.byref(out)),
                       what="request bytes")
        return int(out.value)

    def submit(self, t, y, dy, freqs=None, nf=None, df=None, k0=1, on_result=None,
               arrival=None):
        """Queue one light curve; returns a Future of (freqs, power).

        The grid is ``freqs`` (df (k0 + arange(nf)), as cuvarbase requires)
        or, without building the array, ``nf``, ``df`` and ``k0``; then the
        result's freqs is None.  With ``on_result(freqs, power)`` the power
        (a view valid during the call) is handed to the callback on the
        delivery thread and the future resolves to None.
        """
        if arrival is None:
            arrival = time.perf_counter()
        t = np.ascontiguousarray(t, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        dy = np.ascontiguousarray(dy, np.float64)
        if freqs is not None:
            freqs = np.asarray(freqs, np.float64)
            k0 = get_k0(freqs)
            check_k0(freqs, k0=k0)
            nf, df = len(freqs), _grid_df(freqs)
        elif nf is None or df is None:
            raise ValueError("give freqs, or nf and df")
        if not (len(t) == len(y) == len(dy)):
            raise ValueError("t, y and dy must have the same length")
        fut = Future()
        rid = next(self._ids)
        with self._plock:
            self._pending[rid] = (fut, freqs, on_result, arrival, time.perf_counter())
        rc = self._L.cuvgls_server_submit(self._srv, rid, t.ctypes.data, y.ctypes.data,
                                          dy.ctypes.data, len(t), int(nf), float(df), int(k0))
        if rc != _lib.OK:
            with self._plock:
                self._pending.pop(rid, None)
            if rc == _lib.EBUDGET:
                self.rejected += 1
                fut.set_exception(MemoryError(
                    f"request needs {self.request_bytes(len(t), nf)} bytes, a batch may use "
                    f"{self.slot_budget} (budget {self.hbm_budget})"))
            else:
                try:
                    _lib.raise_for(rc, what="submit")
                except Exception as e:  # noqa: BLE001 - delivered through the future
                    fut.set_exception(e)
        return fut

    def _slot_views(self):
        """(base address, float32 view) of every slot's result buffer."""
        out = []
        for k in range(self._inflight):
            ptr, n = ctypes.c_void_p(), ctypes.c_int64()
            _lib.raise_for(self._L.cuvgls_server_slot_buffer(self._srv, k, ctypes.byref(ptr),
                                                             ctypes.byref(n)), what="slot")
            if ptr.value and n.value > 0:
                arr = (ctypes.c_float * int(n.value)).from_address(ptr.value)
                out.append((ptr.value, ptr.value + 4 * int(n.value), np.frombuffer(arr, np.float32)))
        return out

    def _view(self, addr, n):
        for _ in range(2):
            for lo, hi, v in self._views:
                if lo <= addr and addr + 4 * n <= hi:
                    o = (addr - lo) // 4
                    return v[o:o + n]
            self._views = self._slot_views()   # a slot buffer grew
        raise RuntimeError("result outside the slot buffers")

    def _deliver(self):
        ids, st, res, nfs, lat = self._buf
        L, srv = self._L, self._srv
        rel = (ctypes.c_int64 * self._POLL)()
        pending, lock = self._pending, self._plock
        perf = time.perf_counter
        while True:
            k = L.cuvgls_server_poll(srv, self._POLL, 20, ids, st, res, nfs, lat)
            if k == _lib.ECLOSED:
                return
            if k < 0:
                time.sleep(0.001)
                continue
            with lock:
                items = [pending.pop(int(ids[i])) for i in range(k)]
            for i in range(k):
                fut, freqs, on_result, arrival, t_sub = items[i]
                rel[i] = ids[i]
                self.ready_latencies.append(t_sub - arrival + 1e-3 * lat[i])
                self.lib_latencies.append(1e-3 * lat[i])
                self.lags.append(t_sub - arrival)
                try:
                    if st[i] != _lib.OK:
                        try:
                            _lib.raise_for(int(st[i]), what="serve batch")
                        except Exception as e:  # noqa: BLE001
                            fut.set_exception(e)
                        continue
                    P = self._view(res[i], int(nfs[i]))
                    if on_result is not None:
                        on_result(freqs, P)
                        self.latencies.append(perf() - arrival)
                        fut.set_result(None)
                    else:
                        P = P.copy()
                        self.latencies.append(perf() - arrival)
                        fut.set_result((freqs, P))
                except Exception as e:  # noqa: BLE001 - a failing callback fails its future
                    if not fut.done():
                        fut.set_exception(e)
            L.cuvgls_server_release_many(srv, rel, k)

    def close(self):
        if self._closed:
            return
        self._L.cuvgls_server_shutdown(self._srv)
        self._thread.join()
        self._final = self._counts()
        self._closed = True
        self._L.cuvgls_server_destroy(self._srv)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------
    def stats(self):
        """p50 / p99 / mean latency (ms) of delivered requests, batches and
        mean batch size since the last reset_stats(), rejected requests."""
        lat = np.asarray(self.latencies) * 1000.0
        rdy = np.asarray(self.ready_latencies) * 1000.0
        c = self._final if self._closed else self._counts()
        nb, nr = c[3] - self._base[0], c[4] - self._base[1]
        out = {"requests": int(len(lat)), "rejected": self.rejected, "batches": int(nb),
               "mean_batch": float(nr) / max(1, nb)}
        if len(lat):
            out.update(p50_ms=float(np.percentile(lat, 50)),
                       p99_ms=float(np.percentile(lat, 99)), mean_ms=float(lat.mean()),
                       max_ms=float(lat.max()))
        if len(rdy):
            lib = np.asarray(self.lib_latencies) * 1000.0
            lag = np.asarray(self.lags) * 1000.0
            out.update(ready_p50_ms=float(np.percentile(rdy, 50)),
                       ready_p99_ms=float(np.percentile(rdy, 99)),
                       lib_p99_ms=float(np.percentile(lib, 99)), lib_max_ms=float(lib.max()),
                       lag_p99_ms=float(np.percentile(lag, 99)), lag_max_ms=float(lag.max()))
        return out

    def reset_stats(self):
        self.latencies.clear()
        self.ready_latencies.clear()
        self.lib_latencies.clear()
        self.lags.clear()
        c = self._counts()
        self._base = (c[3], c[4])


def poisson_workload(rate, duration, seed=0, nmin=100, nmax=20000, fmin=1e4, fmax=1e6,
                     with_freqs=True):
    """Requests with Poisson arrivals: (arrival_s, t, y, dy, freqs) with N and
    nf log-uniform, data as the single-curve configuration (seasonal gaps,
    one sinusoid plus noise, dy = 0.05).  With with_freqs=False the last item
    is (nf, df) instead of the frequency array."""
    rng = np.random.default_rng(seed)
    out = []
    at = 0.0
    while True:
        at += rng.exponential(1.0 / rate)
        if at > duration:
            break
        N = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        nf = int(round(np.exp(rng.uniform(np.log(fmin), np.log(fmax)))))
        T = 3650.0
        c = rng.uniform(0, T, 3 * N)
        c = c[(c / 365.25) % 1.0 >= 0.5]
        while len(c) < N:
            d = rng.uniform(0, T, 3 * N)
            c = np.concatenate([c, d[(d / 365.25) % 1.0 >= 0.5]])
        t = np.sort(c[:N])
        y = 0.1 * np.sin(2 * np.pi * t / rng.uniform(0.2, 50) + rng.uniform(0, 6.28))
        y = y + rng.normal(0, 0.05, N)
        df = 1.0 / (5 * (t.max() - t.min()))
        grid = df * (1 + np.arange(nf)) if with_freqs else (nf, df)
        out.append((at, t, y, 0.05 * np.ones(N), grid))
    return out


def run_poisson(server, workload, on_result=None, threads=1):
    """Replay a workload against a server in real time; returns futures (in
    workload order).  Each request's latency counts from its scheduled
    arrival, so time spent behind a lagging submitter is included.  With
    threads > 1 the requests are submitted by that many client threads
    (request i by thread i mod threads), each keeping to the schedule."""
    t0 = time.perf_counter()
    futs = [None] * len(workload)

    def client(k):
        for i in range(k, len(workload), threads):
            at, t, y, dy, fr = workload[i]
            dt = at - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            if isinstance(fr, tuple):
                futs[i] = server.submit(t, y, dy, nf=fr[0], df=fr[1], on_result=on_result,
                                        arrival=t0 + at)
            else:
                futs[i] = server.submit(t, y, dy, fr, on_result=on_result, arrival=t0 + at)

    if threads <= 1:
        client(0)
    else:
        ths = [threading.Thread(target=client, args=(k,)) for k in range(threads)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
    return futs
