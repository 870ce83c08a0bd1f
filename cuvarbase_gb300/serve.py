"""Continuous-batching GLS server.

Requests (one light curve and its frequency grid each) arrive on any thread
with ``submit``; a background loop admits them under an HBM budget and runs
everything admitted so far as one batched libcuvgls call.  Two handles on two
streams keep up to two batches in flight, so requests that arrive while one
batch runs on the GPU are admitted into the next batch, which overlaps it on
the device; a request's budget is returned when its batch completes.  Each
request's latency (arrival to result) is recorded for p50 / p99.

Admission: a request needs its own temporaries (three grid intermediates of
G complex64, 40 bytes per point of spreading records, bin offsets) plus its
inputs and outputs.  Each in-flight batch runs in its own workspace of
``hbm_budget / inflight`` bytes and admits requests up to that size, so the
batches in flight together stay within ``hbm_budget``.  A request larger than
one batch's share is rejected with MemoryError at submit.

There is no reference counterpart (cuvarbase runs one synchronous batch per
call); the GLS arithmetic is that of ``cuvgls_gls_batch``.
"""
from __future__ import annotations

import ctypes
import threading
import time
from collections import deque
from concurrent.futures import Future

import numpy as np

from . import _lib
from .lombscargle import check_k0, get_k0
from .utils import weights


class _Request:
    __slots__ = ("t", "yw", "w", "yy", "ybar", "yw_sum", "w_sum", "nf", "k0", "df",
                 "freqs", "bytes", "future", "arrival", "done", "on_result")

    def __init__(self):
        self.done = None


class GLSServer:
    """Serve floating-mean GLS periodograms with continuous batching.

    Parameters
    ----------
    sigma, m : grid oversampling and Gaussian half-width ('auto' autotunes)
    hbm_budget : bytes of device memory the requests in flight may use
    max_batch : most requests in one batch
    device : CUDA device ordinal
    """

    def __init__(self, sigma="auto", m=8, hbm_budget=80 << 30, max_batch=4096,
                 device=0, inflight=2):
        sig = -1.0 if sigma == "auto" else float(sigma)
        self.hbm_budget = int(hbm_budget)
        self.max_batch = int(max_batch)
        # each in-flight batch runs in its own handle's workspace; a batch is
        # admitted up to that workspace, so all batches in flight together stay
        # within hbm_budget
        ws = max(32 << 20, self.hbm_budget // max(1, inflight))
        self.slot_budget = ws
        self._slots = []
        for _ in range(max(1, inflight)):
            h = _lib.Handle(sigma=sig, m=m, device=device, workspace_bytes=ws)
            self._slots.append({"h": h, "s": _lib.Stream(), "busy": None, "out": None})
        # sizing on the submitting threads uses its own handle
        self._planner = _lib.Handle(sigma=sig, m=m, device=device)
        self._plock = threading.Lock()
        self._q = deque()
        self._cv = threading.Condition()
        self._inflight_bytes = 0
        self._stop = False
        self.latencies = []
        self.batches = []          # (n_requests, launch time, finish time)
        self.rejected = 0
        self._thread = threading.Thread(target=self._loop, daemon=True)
        self._thread.start()

    # ------------------------------------------------------------------
    def request_bytes(self, n, nf):
        """Device bytes one request occupies while in flight."""
        nn = (ctypes.c_int64 * 1)(int(n))
        ff = (ctypes.c_int64 * 1)(int(nf))
        out = ctypes.c_int64()
        h = self._planner
        with self._plock:
            h.check(_lib.load().cuvgls_batch_bytes(h.ptr, 1, nn, ff, 1, ctypes.byref(out)),
                    "request bytes")
        return int(out.value)

    def submit(self, t, y, dy, freqs=None, nf=None, df=None, k0=1, on_result=None):
        """Queue one light curve; returns a Future of (freqs, power).

        The grid is ``freqs`` (df (k0 + arange(nf)), as cuvarbase requires)
        or, without building the array, ``nf``, ``df`` and ``k0``; then the
        result's freqs is None.  With ``on_result(freqs, power)`` the power is
        handed to the callback on the server thread and the future resolves
        to None (streaming consumers).
        """
        t = np.asarray(t, np.float64)
        y = np.asarray(y, np.float64)
        dy = np.asarray(dy, np.float64)
        if freqs is not None:
            freqs = np.asarray(freqs, np.float64)
            k0 = get_k0(freqs)
            check_k0(freqs, k0=k0)
            nf, df = len(freqs), float(freqs[1] - freqs[0])
        elif nf is None or df is None:
            raise ValueError("give freqs, or nf and df")
        r = _Request()
        r.on_result = on_result
        # host preparation as cuvarbase does it (normalize, weights, YY)
        t = t - np.nanmean(t)
        y = y - np.nanmean(y)
        w = weights(dy)
        ybar = float(np.dot(y, w))
        yw = w * (y - ybar)
        r.t = np.ascontiguousarray(t)
        r.yw = yw.astype(np.float32)
        r.w = w.astype(np.float32)
        r.yy = float(np.dot(w, (y - ybar) ** 2))
        r.ybar = ybar
        r.yw_sum = float(np.cumsum(r.yw, dtype=np.float32)[-1])
        r.w_sum = float(np.sum(r.w, dtype=np.float64))
        r.nf, r.k0, r.df, r.freqs = int(nf), int(k0), float(df), freqs
        r.bytes = self.request_bytes(len(t), r.nf)
        r.future = Future()
        r.arrival = time.perf_counter()
        if r.bytes > self.slot_budget:
            self.rejected += 1
            r.future.set_exception(MemoryError(
                f"request needs {r.bytes} bytes, a batch may use {self.slot_budget} "
                f"(budget {self.hbm_budget})"))
            return r.future
        with self._cv:
            self._q.append(r)
            self._cv.notify()
        return r.future

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify()
        self._thread.join()
        for sl in self._slots:
            sl["h"].close()
            sl["s"].close()
            if sl["out"] is not None:
                sl["out"].close()
        self._planner.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------
    def _launch(self, slot, reqs):
        n_tot = sum(len(r.t) for r in reqs)
        nf_tot = sum(r.nf for r in reqs)
        t = np.empty(n_tot, np.float64)
        yw = np.empty(n_tot, np.float32)
        w = np.empty(n_tot, np.float32)
        curves = (_lib.Curve * len(reqs))()
        out = slot["out"]
        if out is None or out.nbytes < nf_tot * 4:  # grow-only page-locked results
            if out is not None:
                out.close()
            out = slot["out"] = _lib.PinnedBuffer(max(nf_tot * 4, 64 << 20))
        o = fo = 0
        for i, r in enumerate(reqs):
            n = len(r.t)
            t[o:o + n], yw[o:o + n], w[o:o + n] = r.t, r.yw, r.w
            c = curves[i]
            c.pt_off, c.n, c.nf, c.k0, c.df = o, n, r.nf, r.k0, r.df
            c.yy, c.ybar, c.yw_sum, c.w_sum, c.out_off = r.yy, r.ybar, r.yw_sum, r.w_sum, fo
            o += n
            fo += r.nf
        inp = _lib.GlsInput()
        inp.n_curves, inp.mode = len(reqs), _lib.MODE_FLOATING_MEAN
        inp.curves = ctypes.cast(curves, ctypes.c_void_p)
        inp.t, inp.yw, inp.w = t.ctypes.data, yw.ctypes.data, w.ctypes.data
        inp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
        inp.n_points_total, inp.n_out_total = n_tot, nf_tot
        h = slot["h"]
        h.check(_lib.load().cuvgls_gls_batch(h.ptr, ctypes.byref(inp), out.ptr,
                                             slot["s"].ptr), "serve batch")
        slot["busy"] = (reqs, out, time.perf_counter())

    def _poll(self, slot):
        """Complete the slot's batch if the GPU is done; True if it was."""
        if slot["busy"] is None:
            return False
        h = slot["h"]
        try:
            h.sync(slot["s"].ptr, 0)
        except TimeoutError:
            return False
        reqs, out, t_launch = slot["busy"]
        slot["busy"] = None
        now = time.perf_counter()
        fo = 0
        freed = 0
        for r in reqs:
            P = out.view(np.float32, r.nf, fo * 4).copy()
            fo += r.nf
            self.latencies.append(now - r.arrival)
            if r.on_result is not None:
                r.on_result(r.freqs, P)
                r.future.set_result(None)
            else:
                r.future.set_result((r.freqs, P))
            freed += r.bytes
        self.batches.append((len(reqs), t_launch, now))
        with self._cv:
            self._inflight_bytes -= freed
        return True

    def _loop(self):
        while True:
            progressed = False
            for sl in self._slots:
                progressed |= self._poll(sl)
            free = [sl for sl in self._slots if sl["busy"] is None]
            with self._cv:
                if self._stop and not self._q and len(free) == len(self._slots):
                    return
                batch = []
                if free and self._q:
                    budget = min(self.slot_budget, self.hbm_budget - self._inflight_bytes)
                    while self._q and len(batch) < self.max_batch and \
                            self._q[0].bytes <= budget:
                        r = self._q.popleft()
                        budget -= r.bytes
                        batch.append(r)
                    self._inflight_bytes += sum(r.bytes for r in batch)
                elif not progressed and not self._stop and len(free) == len(self._slots):
                    self._cv.wait(0.001)
            if batch:
                try:
                    self._launch(free[0], batch)
                except Exception as e:  # report to every request of the batch
                    with self._cv:
                        self._inflight_bytes -= sum(r.bytes for r in batch)
                    for r in batch:
                        r.future.set_exception(e)
            elif not progressed:
                time.sleep(5e-5)

    # ------------------------------------------------------------------
    def stats(self):
        lat = np.asarray(self.latencies) * 1000.0
        if len(lat) == 0:
            return {"requests": 0}
        return {"requests": int(len(lat)), "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                "batches": len(self.batches),
                "mean_batch": float(np.mean([b[0] for b in self.batches])),
                "rejected": self.rejected}


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


def run_poisson(server, workload, on_result=None):
    """Replay a workload against a server in real time; returns futures."""
    t0 = time.perf_counter()
    futs = []
    for at, t, y, dy, fr in workload:
        dt = at - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        if isinstance(fr, tuple):
            futs.append(server.submit(t, y, dy, nf=fr[0], df=fr[1], on_result=on_result))
        else:
            futs.append(server.submit(t, y, dy, fr, on_result=on_result))
    return futs
