"""Benchmark of the batched GLS path (one JSON line on rank 0).

Workload (the batched configuration of the GLS path): 10,000 light curves,
N log-uniform in [50, 5000] points over baselines uniform in [100, 3650] d,
sinusoids (period log-uniform 0.1-100 d, amplitude 0.05-0.5) plus noise
(sigma 0.02-0.2), heteroscedastic dy ~ lognormal(ln 0.05, 0.3); nf = 100,000
frequencies per curve at df = 1 / (5 T); floating-mean GLS, FP32 bulk with
FP64 offsets and phases; grid oversampling and window width chosen by the
library's autotuner (--sigma auto, the default) or fixed (--sigma 2 --m 8).
Synthetic, seeded.  Every run checks max |dP| on sample curves against the
FP64 oracle and reports it.

A step is one pass of the GLS path over the whole batch.  `value` is
periodograms per second with inputs resident in HBM; `e2e` is the same
metric through the C ABI from raw (t, y, dy) in page-locked host memory to
powers in host memory (cuvgls_gls_raw: H2D, the reference's host preparation
done on the device, the GLS, D2H, all inside the timed region);
`e2e.prepared_input` repeats it with yw, w prepared on the host beforehand.
The inputs (160-240 MB) and outputs (4 GB) are larger than L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the reference's CPU implementation of the path
(FP64 direct-sum GLS of cuvarbase/lombscargle.py:539-576, restated in C with
OpenMP in oracle/) on the host cores, on a bounded sample of the workload.
"""
from __future__ import annotations

import argparse
import ctypes
import gc
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched LS periodograms/s vs plain per-curve path, |dP|<=1e-4; serve p50/p99 ms"
UNIT = "periodograms/s"


# ----------------------------------------------------------------------------
# workload
# ----------------------------------------------------------------------------
def make_batch(n_curves, seed=1002, nmin=50, nmax=5000):
    rng = np.random.default_rng(seed)
    N = np.round(np.exp(rng.uniform(np.log(nmin), np.log(nmax), n_curves))).astype(np.int64)
    T = rng.uniform(100, 3650, n_curves)
    per = np.exp(rng.uniform(np.log(0.1), np.log(100), n_curves))
    amp = rng.uniform(0.05, 0.5, n_curves)
    sn = rng.uniform(0.02, 0.2, n_curves)
    ph = rng.uniform(0, 2 * np.pi, n_curves)
    off = np.zeros(n_curves + 1, np.int64)
    off[1:] = np.cumsum(N)
    ntot = int(off[-1])
    cid = np.repeat(np.arange(n_curves), N)
    t = rng.uniform(0, 1, ntot) * T[cid]
    # sort within each curve
    order = np.lexsort((t, cid))
    t = t[order]
    y = amp[cid] * np.sin(2 * np.pi * t / per[cid] + ph[cid]) + rng.normal(0, 1, ntot) * sn[cid]
    dy = np.exp(rng.normal(np.log(0.05), 0.3, ntot))
    return dict(N=N, off=off, t=t, y=y, dy=dy, period=per, cid=cid)


def prepare(b):
    """Host preparation as the reference does it (normalize, weights, YY)."""
    off, cid, N = b["off"], b["cid"], b["N"]
    red = lambda a: np.add.reduceat(a, off[:-1])  # noqa: E731
    t = b["t"] - (red(b["t"]) / N)[cid]
    y = b["y"] - (red(b["y"]) / N)[cid]
    w = b["dy"] ** -2
    w = w / red(w)[cid]
    ybar = red(w * y)
    yw = w * (y - ybar[cid])
    yy = red(w * (y - ybar[cid]) ** 2)
    yw32, w32 = yw.astype(np.float32), w.astype(np.float32)
    T = np.maximum.reduceat(t, off[:-1]) - np.minimum.reduceat(t, off[:-1])
    return dict(t=np.ascontiguousarray(t), yw=yw32, w=w32, yy=yy, ybar=ybar,
                yw_sum=red(yw32.astype(np.float64)), w_sum=red(w32.astype(np.float64)),
                df=1.0 / (5.0 * T), off=off, N=N)


def curve_table(p, nf, first=0, count=None, out_base=None):
    from cuvarbase_gb300 import _lib
    n = len(p["N"]) if count is None else count
    arr = (_lib.Curve * n)()
    for i in range(n):
        c = first + i
        a = arr[i]
        a.pt_off, a.n, a.nf, a.k0 = int(p["off"][c]), int(p["N"][c]), nf, 1
        a.df, a.yy, a.ybar = float(p["df"][c]), float(p["yy"][c]), float(p["ybar"][c])
        a.yw_sum, a.w_sum = float(p["yw_sum"][c]), float(p["w_sum"][c])
        a.out_off = (c if out_base is None else out_base + i) * nf
    return arr


# ----------------------------------------------------------------------------
# clocks
# ----------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------
# reference arm: the CPU implementation of the path
# ----------------------------------------------------------------------------
def cpu_model():
    """The host CPU's model name (/proc/cpuinfo, else lscpu, else the
    machine type)."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                if k.strip() in ("model name", "Model Name", "cpu model") and v.strip():
                    return v.strip()
    except OSError:
        pass
    try:
        import subprocess
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            k, _, v = line.partition(":")
            if k.strip() == "Model name" and v.strip():
                return v.strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.machine()


def cpu_gls_sample(b, p, nf, curves, nthreads=0):
    from oracle import oracle as O
    t0 = time.perf_counter()
    for c in curves:
        s, e = p["off"][c], p["off"][c + 1]
        O.gls_flmean(p["t"][s:e], p["yw"][s:e], p["w"][s:e],
                     p["df"][c] * (1 + np.arange(nf)), p["yy"][c], nthreads=nthreads)
    return time.perf_counter() - t0


def run_reference(args, rank):
    if rank != 0:
        return None
    from oracle import oracle as O
    O.build()
    b = make_batch(args.curves, seed=args.seed)
    p = prepare(b)
    cores = O.max_threads()
    rng = np.random.default_rng(7)
    per_step = args.ref_curves
    for _ in range(args.warmup):
        cpu_gls_sample(b, p, args.nf, rng.integers(0, args.curves, 1))
    tot, ncur = 0.0, 0
    for _ in range(args.steps):
        cs = rng.integers(0, args.curves, per_step)
        tot += cpu_gls_sample(b, p, args.nf, cs)
        ncur += per_step
    v = ncur / tot
    sample = (f"{per_step} curves per step (of the {args.curves}-curve batch, "
              f"nf={args.nf}), FP64 direct sums")
    return {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(args),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "cpu": cpu_model(),
                             "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def config(args):
    grid = ("autotuned window/sigma/m (ES window, max |dP| <= 2e-5 budget)" if args.sigma == "auto"
            else f"sigma={args.sigma}, m={args.m}")
    return {"workload": f"batched GLS: {args.curves} light curves, N log-uniform [50, 5000], "
                        f"nf={args.nf} per curve, floating mean, {grid}",
            "n_curves": args.curves, "nf": args.nf, "sigma": args.sigma,
            "m": "auto" if args.sigma == "auto" else args.m,
            "l2": "inputs (160 MB) and outputs (4 GB) exceed L2; no flush",
            "parallelism": f"replicas x{args.gpus} (curves sharded per rank, no collective)"}


# ----------------------------------------------------------------------------
# our arm
# ----------------------------------------------------------------------------
def stage_bytes(p, nf, plan, curves):
    """Algorithmic bytes per stage for the given curves:
    prep reads t, yw, w (16 B/pt) + t again (8 B/pt) and writes 40 B/pt of
    records; pass 1 reads 40 B/pt of records and writes 3 G complex64; pass 2
    reads 3 G complex64 and writes 4 B per frequency."""
    G = plan[0]
    n = float(np.sum(p["N"][curves]))
    k = len(curves)
    return {"prep": 64.0 * n, "pass1": 40.0 * n + 24.0 * G * k,
            "pass2": 24.0 * G * k + 4.0 * nf * k}


def gls_input(curves, n, t_ptr, yw_ptr, w_ptr, flags, npts, nout):
    from cuvarbase_gb300 import _lib
    inp = _lib.GlsInput()
    inp.n_curves, inp.mode = n, _lib.MODE_FLOATING_MEAN
    inp.curves = ctypes.cast(curves, ctypes.c_void_p)
    inp.t, inp.yw, inp.w = t_ptr, yw_ptr, w_ptr
    inp.flags = flags
    inp.n_points_total, inp.n_out_total = npts, nout
    return inp


def time_device_batch(h, p, nf, steps, warmup):
    """Device-resident timed loop of one GLS batch (inputs and outputs in
    HBM): returns (ms per step, per-stage (launches, ms) over the timed steps,
    the output tensor)."""
    import torch

    from cuvarbase_gb300 import _lib
    L = _lib.load()
    nc = len(p["N"])
    ntot = int(p["off"][-1])
    t_d = torch.from_numpy(p["t"]).cuda()
    yw_d = torch.from_numpy(p["yw"]).cuda()
    w_d = torch.from_numpy(p["w"]).cuda()
    out_d = torch.empty(nc * nf, dtype=torch.float32, device="cuda")
    curves = curve_table(p, nf)
    inp = gls_input(curves, nc, t_d.data_ptr(), yw_d.data_ptr(), w_d.data_ptr(), 0, ntot, nc * nf)
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)

    def step():
        h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(inp), ctypes.c_void_p(out_d.data_ptr()),
                                   sptr), "gls batch")

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    h.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    prof = h.profile_read()
    h.profile(False)
    return e0.elapsed_time(e1) / steps, prof, out_d


E2E_REPS = 5


def _time_host_steps(step, steps, stream, e0, e1, world):
    """Times E2E_REPS repetitions of `steps` host-to-host calls (each the
    larger of the CUDA-event and the host-clock time, max over ranks) and
    returns (the median, all of them) in ms: the page-locked host link is
    shared with the machine's other work, so one repetition can be slowed
    by traffic that is not this program's."""
    import torch

    from cuvarbase_gb300.replicas import max_over_ranks
    reps = []
    for _ in range(E2E_REPS):
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        e0.record(stream)
        t0 = time.perf_counter()
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = max(e0.elapsed_time(e1), 1000.0 * (time.perf_counter() - t0))
        reps.append(max_over_ranks(ms) if world > 1 else ms)
    return float(np.median(reps)), reps


def time_best_e2e(h, p, nf, steps, warmup):
    """Best frequency of every curve end to end (cuvgls_gls_best with
    page-locked host inputs and outputs): H2D of t, yw, w and D2H of one
    index and power per curve inside the timed region."""
    import torch

    from cuvarbase_gb300 import _lib
    L = _lib.load()
    nc = len(p["N"])
    ntot = int(p["off"][-1])
    bufs = [_lib.PinnedBuffer(ntot * 8), _lib.PinnedBuffer(ntot * 4), _lib.PinnedBuffer(ntot * 4),
            _lib.PinnedBuffer(nc * 8), _lib.PinnedBuffer(nc * 4)]
    bufs[0].view(np.float64, ntot)[:] = p["t"]
    bufs[1].view(np.float32, ntot)[:] = p["yw"]
    bufs[2].view(np.float32, ntot)[:] = p["w"]
    curves = curve_table(p, nf)
    inp = gls_input(curves, nc, bufs[0].ptr.value, bufs[1].ptr.value, bufs[2].ptr.value,
                    _lib.HOST_INPUT | _lib.HOST_OUTPUT, ntot, 0)
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)

    def step():
        h.check(L.cuvgls_gls_best(h.ptr, ctypes.byref(inp), bufs[3].ptr, bufs[4].ptr, sptr),
                "gls best")

    for _ in range(warmup):
        step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ms, reps = _time_host_steps(step, steps, stream, e0, e1, 1)
    ms /= steps
    k = bufs[3].view(np.int64, nc).copy()
    for b in bufs:
        b.close()
    return {"ms_per_step": ms, "periodograms_per_s": nc / (ms / 1000.0),
            "repetitions_ms_per_step": [round(r / steps, 3) for r in reps],
            "lc_freq_per_s": nc * nf / (ms / 1000.0),
            "h2d_bytes_per_step": int(ntot * 16 + nc * 96), "d2h_bytes_per_step": int(nc * 12),
            "valid_peaks": int(np.sum(k >= 0)),
            "path": "cuvgls_gls_best with CUVGLS_HOST_INPUT|CUVGLS_HOST_OUTPUT"}


def run_api(args, b, p):
    """The reference-compatible Python API end to end on the first
    args.api_curves curves of the batch: LombScargleAsyncProcess.run(data,
    freqs=...) + finish() from raw (t, y, dy) numpy arrays to powers in host
    memory; against the same API with preallocated memory (host preparation
    per curve, as cuvarbase does it)."""
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    nc = min(args.api_curves, len(b["N"]))
    data = [(b["t"][b["off"][i]:b["off"][i + 1]], b["y"][b["off"][i]:b["off"][i + 1]],
             b["dy"][b["off"][i]:b["off"][i + 1]]) for i in range(nc)]
    freqs = [p["df"][i] * (1 + np.arange(args.nf)) for i in range(nc)]
    sigma = "auto" if args.sigma == "auto" else float(args.sigma)
    out = {"curves": nc, "nf": args.nf}
    for name, pre in (("run", False), ("run_preallocated", True)):
        proc = LombScargleAsyncProcess(sigma=sigma)
        mem = proc.preallocate(int(max(b["N"][:nc])), nlcs=nc, nf=args.nf, k0=1) if pre else None
        times = []
        for it in range(3 + args.api_steps):
            t0 = time.perf_counter()
            proc.run(data, freqs=freqs, memory=mem)
            proc.finish()
            times.append(time.perf_counter() - t0)
        el = float(np.median(times[3:]))
        out[name] = {"periodograms_per_s": nc / el, "s_per_call": el}
        del proc, mem
    out["path"] = ("run: host arrays -> cuvgls_gls_raw (preparation on the GPU); "
                   "run_preallocated: LombScargleMemory.setdata per curve -> cuvgls_gls_batch")
    return out


def cfg1_curve(seed=1001, N=1000, T=3650.0):
    """Single-curve configuration: N times uniform over a 3650-d baseline with
    a half-year seasonal gap, sorted; y = 0.1 sin(2 pi t / 0.73 d + phi) +
    N(0, 0.05^2); dy = 0.05."""
    rng = np.random.default_rng(seed)
    t = []
    while len(t) < N:
        c = rng.uniform(0, T, 4 * N)
        t.extend(c[(c / 365.25) % 1.0 >= 0.5].tolist())
    t = np.sort(np.array(t[:N]))
    y = 0.1 * np.sin(2 * np.pi * t / 0.73 + rng.uniform(0, 2 * np.pi)) + rng.normal(0, 0.05, N)
    return t, y, 0.05 * np.ones(N)


def run_single(args):
    """Plain GLS of one light curve (N = 1000, nf = 50,000 at df = 1/(5 T),
    sigma = 2, m = 8): time per periodogram through the reference-style
    Python API (run + finish, host arrays in, powers in host memory) and
    through the C ABI from device-resident raw input; the whole band against
    the FP64 oracle, and the peak bin against the injected period."""
    from cuvarbase_gb300 import _lib
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    from oracle import oracle as O
    import torch
    t, y, dy = cfg1_curve()
    nf = 50_000
    df = 1.0 / (5 * 3650.0)
    freqs = df * (1 + np.arange(nf))
    proc = LombScargleAsyncProcess(sigma=2, m=8)
    times = []
    for it in range(3 + args.single_steps):
        t0 = time.perf_counter()
        (f, P), = proc.run([(t, y, dy)], freqs=freqs)
        proc.finish()
        times.append(time.perf_counter() - t0)
    P = np.copy(P)
    api_ms = 1000.0 * float(np.median(times[3:]))
    # C ABI, raw input already on the device, powers to device memory
    h = _lib.Handle(sigma=2.0, m=8)
    L = _lib.load()
    td, yd, dyd = (torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda() for a in (t, y, dy))
    out = torch.empty(nf, dtype=torch.float32, device="cuda")
    rc = (_lib.RawCurve * 1)()
    rc[0].pt_off, rc[0].n, rc[0].nf, rc[0].k0, rc[0].df, rc[0].out_off = 0, len(t), nf, 1, df, 0
    ri = _lib.RawInput()
    ri.n_curves, ri.mode = 1, _lib.MODE_FLOATING_MEAN
    ri.curves = ctypes.cast(rc, ctypes.c_void_p)
    ri.t, ri.y, ri.dy = td.data_ptr(), yd.data_ptr(), dyd.data_ptr()
    ri.flags, ri.n_points_total, ri.n_out_total = 0, len(t), nf
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)

    def call():
        h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(ri), ctypes.c_void_p(out.data_ptr()),
                                 None, None, sptr), "single raw")

    for _ in range(5):
        call()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = max(10, args.single_steps * 10)
    e0.record(stream)
    for _ in range(n):
        call()
    e1.record(stream)
    torch.cuda.synchronize()
    dev_ms = e0.elapsed_time(e1) / n
    Pd = out.cpu().numpy()
    h.close()
    tt, yw, w, YY, _ = O.prepare_curve(t, y, dy)
    Pref = O.gls_flmean(tt, yw, w, freqs, YY)
    k_inj = int(np.rint((1.0 / 0.73) / df)) - 1
    return {"workload": "1 curve, N=1000 over 3650 d with seasonal gaps, nf=50000, sigma=2, m=8",
            "api_ms_per_periodogram": api_ms, "device_ms_per_periodogram": dev_ms,
            "max_abs_dP_api": float(np.abs(P - Pref).max()),
            "max_abs_dP_device": float(np.abs(Pd - Pref).max()),
            "peak_bin": int(np.argmax(P)), "oracle_peak_bin": int(np.argmax(Pref)),
            "injected_bin": k_inj}


def _time_events(fn, steps, warmup):
    """Mean ms per call of fn on the current stream (CUDA events)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def run_fft_check(args):
    """cuFFT as a timing and accuracy cross-check of the adjoint NFFT.

    The reference's NFFT pipeline rebuilt on this GPU with cuFFT for the FFT
    (cuvarbase/cunfft.py:163-308): the reference-convention Gaussian grid of
    ng = 2 nf cells per curve (cuvgls_spread_ref, cunfft.cu:84-163), cuFFT's
    unnormalised inverse FFT of all grids as one batch (torch.fft), then the
    phase and deconvolution of cunfft.cu:214-248 on the first nf bins.
    Against cuvgls_nfft_adjoint_batch (spreading fused into the column FFTs,
    deconvolution into the row FFTs) on the same curves, sigma = 2, m = 8,
    f_k = k / (tmax - tmin).  Reports both times, cuFFT's alone, and
    max |difference| / sum |y| per curve.
    """
    import torch

    from cuvarbase_gb300 import _lib
    L = _lib.load()
    nc, nf = args.fft_curves, args.fft_nf
    b = make_batch(nc, seed=1010)
    ntot = int(b["off"][-1])
    sigma, m = 2.0, 8
    ng = int(sigma * nf)
    h = _lib.Handle(sigma=sigma, m=m)
    t_d = torch.from_numpy(b["t"]).cuda()
    y32 = b["y"].astype(np.float32)
    y_d = torch.from_numpy(y32).cuda()
    tmin = np.minimum.reduceat(b["t"], b["off"][:-1])
    tmax = np.maximum.reduceat(b["t"], b["off"][:-1])
    out = {"curves": nc, "nf": nf, "ng": ng, "sigma": sigma, "m": m}
    try:
        # ours
        ncv = (_lib.NfftCurve * nc)()
        for i in range(nc):
            c = ncv[i]
            c.pt_off, c.n, c.nf = int(b["off"][i]), int(b["N"][i]), nf
            c.f0, c.df, c.out_off = 0.0, 1.0 / (tmax[i] - tmin[i]), i * nf
        ninp = _lib.NfftInput()
        ninp.n_curves, ninp.flags = nc, 0
        ninp.curves = ctypes.cast(ncv, ctypes.c_void_p)
        ninp.t, ninp.y = t_d.data_ptr(), y_d.data_ptr()
        ninp.n_points_total, ninp.n_out_total = ntot, nc * nf
        ours_d = torch.empty(nc * nf, dtype=torch.complex64, device="cuda")
        sptr = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

        def ours():
            h.check(L.cuvgls_nfft_adjoint_batch(h.ptr, ctypes.byref(ninp),
                                                ctypes.c_void_p(ours_d.data_ptr()), sptr),
                    "nfft batch")

        out["ours_ms"] = _time_events(ours, args.fft_steps, 3)
        # the reference's pipeline with cuFFT
        gcv = (_lib.GridCurve * nc)()
        for i in range(nc):
            c = gcv[i]
            c.pt_off, c.n, c.ng = int(b["off"][i]), int(b["N"][i]), ng
            c.tmin, c.tmax, c.spp, c.out_off = float(tmin[i]), float(tmax[i]), 1.0, i * ng
        grid_d = torch.empty(nc * ng, dtype=torch.float32, device="cuda")
        bw = 2 * sigma * m / ((2 * sigma - 1) * np.pi)
        k = torch.arange(nf, dtype=torch.float64, device="cuda")
        n0 = torch.from_numpy(tmin / (tmax - tmin) * ng).cuda()           # spp = 1
        th = torch.remainder(n0[:, None] * k[None, :] / ng, 1.0) * (2 * np.pi)
        fac = (torch.exp(1j * th) * torch.exp(bw * (np.pi * k / ng) ** 2)[None, :]).to(
            torch.complex64)
        ref_d = torch.empty(nc, nf, dtype=torch.complex64, device="cuda")

        def grid():
            h.check(L.cuvgls_spread_ref(h.ptr, nc, ctypes.cast(gcv, ctypes.c_void_p),
                                        t_d.data_ptr(), y_d.data_ptr(), ntot, nc * ng, 0,
                                        ctypes.c_void_p(grid_d.data_ptr()), sptr), "spread ref")

        def fft_only(g):
            return torch.fft.ifft(g, dim=1, norm="forward")

        def pipeline():
            grid()
            G = fft_only(grid_d.view(nc, ng).to(torch.complex64))
            torch.mul(G[:, :nf], fac, out=ref_d)

        out["cufft_pipeline_ms"] = _time_events(pipeline, args.fft_steps, 3)
        gc64 = grid_d.view(nc, ng).to(torch.complex64)
        out["cufft_ifft_only_ms"] = _time_events(lambda: fft_only(gc64), args.fft_steps, 3)
        ours()
        pipeline()
        torch.cuda.synchronize()
        # accuracy of both against FP64 direct sums (the oracle, as the
        # checker) on sample curves: bins over the whole band, and the lower
        # half alone (the reference convention puts the band's top at the
        # grid's Nyquist edge, where its deconvolution amplifies aliasing)
        from oracle import oracle as O
        O.build()
        rng = np.random.default_rng(3)
        ours_h = ours_d.view(nc, nf)
        e_ours, e_ref, e_ours_lo, e_ref_lo = 0.0, 0.0, 0.0, 0.0
        for i in rng.integers(0, nc, args.fft_check_curves):
            s0, s1 = int(b["off"][i]), int(b["off"][i + 1])
            kk = np.unique(np.concatenate([np.arange(200), np.arange(nf - 200, nf),
                                           rng.integers(0, nf, 1000)]))
            dfi = 1.0 / (tmax[i] - tmin[i])
            direct = O.nfft_direct(b["t"][s0:s1], y32[s0:s1], kk * dfi)
            sc = float(np.abs(y32[s0:s1].astype(np.float64)).sum())
            a = np.abs(ours_h[i].cpu().numpy()[kk] - direct) / sc
            r = np.abs(ref_d[i].cpu().numpy()[kk] - direct) / sc
            lo = kk < nf // 2
            e_ours, e_ref = max(e_ours, a.max()), max(e_ref, r.max())
            e_ours_lo, e_ref_lo = max(e_ours_lo, a[lo].max()), max(e_ref_lo, r[lo].max())
        out["max_err_over_sum_abs_y"] = {"ours": e_ours, "cufft_pipeline": e_ref,
                                         "ours_lower_half": e_ours_lo,
                                         "cufft_pipeline_lower_half": e_ref_lo,
                                         "curves_checked": args.fft_check_curves,
                                         "against": "FP64 direct sums (oracle)"}
        out["path"] = ("ours: cuvgls_nfft_adjoint_batch; cuFFT: cuvgls_spread_ref grid + "
                       "torch.fft.ifft (cuFFT, batched) + deconvolution, as "
                       "cuvarbase/cunfft.py:163-308")
    finally:
        h.close()
    return out


def run_plan(args, b, p):
    """Small fixed-shape batches from raw device inputs (t, y, dy in HBM):
    cuvgls_gls_raw called per batch against the same batch recorded once as
    a CUDA graph (cuvgls_gls_plan_create) and replayed; per-batch time over
    back-to-back launches on one stream."""
    import torch

    from cuvarbase_gb300 import _lib
    L = _lib.load()
    h = _lib.Handle(sigma=2.0, m=8)
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    out = {"nf": args.plan_nf, "shapes": []}
    try:
        for nc in args.plan_curves:
            nc = min(nc, len(b["N"]))
            o1 = int(b["off"][nc])
            t_d = torch.from_numpy(b["t"][:o1].copy()).cuda()
            y_d = torch.from_numpy(b["y"][:o1].copy()).cuda()
            dy_d = torch.from_numpy(b["dy"][:o1].copy()).cuda()
            out_d = torch.empty(nc * args.plan_nf, dtype=torch.float32, device="cuda")
            cv = (_lib.RawCurve * nc)()
            for i in range(nc):
                c = cv[i]
                c.pt_off, c.n, c.nf, c.k0 = int(b["off"][i]), int(b["N"][i]), args.plan_nf, 1
                c.df, c.out_off = float(p["df"][i]), i * args.plan_nf
            inp = _lib.RawInput()
            inp.n_curves, inp.mode = nc, _lib.MODE_FLOATING_MEAN
            inp.curves = ctypes.cast(cv, ctypes.c_void_p)
            inp.t, inp.y, inp.dy = t_d.data_ptr(), y_d.data_ptr(), dy_d.data_ptr()
            inp.n_points_total, inp.n_out_total = o1, nc * args.plan_nf
            outp = ctypes.c_void_p(out_d.data_ptr())
            plan = ctypes.c_void_p()
            h.check(L.cuvgls_gls_plan_create(h.ptr, ctypes.byref(inp), outp, None, None,
                                             ctypes.byref(plan)), "plan create")
            legs = {
                "call": lambda: h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(inp), outp, None,
                                                         None, sptr), "raw"),
                "graph": lambda: h.check(L.cuvgls_gls_plan_launch(plan, sptr), "plan launch"),
            }
            row = {"curves": nc, "points": o1}
            try:
                for name, fn in legs.items():
                    for _ in range(20):
                        fn()
                    torch.cuda.synchronize()
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    t0 = time.perf_counter()
                    e0.record(stream)
                    for _ in range(args.plan_iters):
                        fn()
                    e1.record(stream)
                    torch.cuda.synchronize()
                    us = 1000.0 * e0.elapsed_time(e1) / args.plan_iters
                    host_us = 1e6 * (time.perf_counter() - t0) / args.plan_iters
                    row[name] = {"us_per_batch": us, "host_us_per_batch": host_us,
                                 "periodograms_per_s": nc / (us * 1e-6)}
            finally:
                L.cuvgls_gls_plan_destroy(plan)
            out["shapes"].append(row)
            del t_d, y_d, dy_d, out_d
    finally:
        h.close()
    return out


def make_precision_batch(n_curves=8, N=1_000_000, T=3650.0, seed=1003):
    """N points uniform over a 3650-d baseline, one injected sinusoid on an
    exact bin plus white noise; f up to 1000 / d at df = 1 / (5 T)."""
    rng = np.random.default_rng(seed)
    df = 1.0 / (5.0 * T)
    nf = int(round(1000.0 / df))
    off = np.arange(n_curves + 1, dtype=np.int64) * N
    t = np.concatenate([np.sort(rng.uniform(0, T, N)) for _ in range(n_curves)])
    cid = np.repeat(np.arange(n_curves), N)
    k_inj = rng.integers(nf // 10, nf - 1000, n_curves)
    ph = rng.uniform(0, 2 * np.pi, n_curves)
    sn = 0.1
    y = 0.05 * np.sin(2 * np.pi * (df * (1 + k_inj))[cid] * t + ph[cid]) + rng.normal(0, sn, t.size)
    b = dict(N=np.full(n_curves, N, dtype=np.int64), off=off, t=t, y=y, dy=np.full(t.size, sn),
             cid=cid)
    return b, df, nf, k_inj


def run_precision(args, peak):
    """Precision stress: 8 curves x 1e6 points, nf = 18,250,000 (bands wider
    than one grid, run as sub-bands); mixed precision (FP64 offsets, cell
    index and phases) against all-FP32 positions, both timed and both checked
    against the FP64 block oracle on blocks of 1000 bins of curve 0 (one
    block around the injected bin; --prec-blocks 100 gives the 1e5-bin
    subsample)."""
    from cuvarbase_gb300 import _lib
    from oracle import oracle as O
    b, df, nf, k_inj = make_precision_batch(args.prec_curves, args.prec_n)
    p = prepare(b)
    p["df"][:] = df
    nc = len(p["N"])
    rng = np.random.default_rng(17)
    starts = np.concatenate([[max(0, int(k_inj[0]) - 500)],
                             rng.integers(0, nf - 1000, args.prec_blocks - 1)]).astype(np.int64)
    s0, e0 = int(p["off"][0]), int(p["off"][1])
    t0 = time.perf_counter()
    Pref = O.gls_flmean_blocks(p["t"][s0:e0], p["yw"][s0:e0], p["w"][s0:e0],
                               df * (1 + starts), df, 1000, p["yy"][0])
    oracle_s = time.perf_counter() - t0
    idx = (starts[:, None] + np.arange(1000)[None, :]).ravel()
    res = {"workload": f"{nc} curves x N={args.prec_n}, T=3650 d, nf={nf} (f <= 1000/d, "
                       f"df=1/(5T)), one injected sinusoid + white noise",
           "lc_freq_per_step": nc * nf, "bins_checked": int(len(starts)) * 1000,
           "oracle": f"FP64 block oracle (phasor recurrence, reseeded every 64 bins) on curve 0: "
                     f"{args.prec_blocks} blocks x 1000 bins (one around the injected bin), "
                     f"{oracle_s:.1f} s on {O.max_threads()} threads"}
    for name, prec in (("mixed", _lib.PREC_MIXED), ("fp32", _lib.PREC_FP32)):
        h = _lib.Handle(sigma=-1.0, m=8, workspace_bytes=args.workspace_gb << 30,
                        precision=prec)
        ms, prof, out = time_device_batch(h, p, nf, args.prec_steps, args.prec_warmup)
        P = out.view(nc, nf)
        gpu_peak = P.argmax(dim=1).cpu().numpy()
        P0 = P[0].cpu().numpy()[idx].reshape(Pref.shape)
        d = np.abs(P0 - Pref)
        res[name] = {"ms_per_step": ms, "lc_freq_per_s": nc * nf / (ms / 1000.0),
                     "max_abs_dP": float(np.nanmax(d)),
                     "peak_bin_exact": int(np.sum(gpu_peak == k_inj)),
                     "curves": nc,
                     "subsample_peak_equal": bool(np.argmax(P0.ravel()) == np.nanargmax(Pref.ravel())),
                     "stage_ms_per_step": {k: prof[k][1] / args.prec_steps
                                           for k in ("prep", "pass1", "pass2")},
                     "launches_per_step": int(sum(v[0] for v in prof.values()) / args.prec_steps)}
        h.close()
        del out, P
    return res


def make_survey_batch(n_curves=200_000, seed=1005):
    """Survey batch: N uniform in [20, 300], T = 1000 d; 30 % pure noise,
    70 % sinusoid or sawtooth with period uniform in [0.05, 10] d."""
    rng = np.random.default_rng(seed)
    N = rng.integers(20, 301, n_curves).astype(np.int64)
    off = np.zeros(n_curves + 1, np.int64)
    off[1:] = np.cumsum(N)
    cid = np.repeat(np.arange(n_curves), N)
    t = rng.uniform(0, 1000.0, int(off[-1]))
    order = np.lexsort((t, cid))
    t = t[order]
    kind = rng.choice(3, n_curves, p=[0.3, 0.35, 0.35])   # noise, sinusoid, sawtooth
    per = rng.uniform(0.05, 10.0, n_curves)
    amp = rng.uniform(0.1, 0.5, n_curves)
    ph = rng.uniform(0, 1, n_curves)
    sn = 0.1
    x = t / per[cid] + ph[cid]
    sig = np.where(kind[cid] == 1, np.sin(2 * np.pi * x), 2.0 * (x - np.floor(x)) - 1.0)
    y = np.where(kind[cid] == 0, 0.0, amp[cid] * sig) + rng.normal(0, sn, t.size)
    b = dict(N=N, off=off, t=t, y=y, dy=np.full(t.size, sn), cid=cid)
    return b, kind, per


def run_survey(args, peak):
    """Memory-bound survey batch: 200,000 short curves, nf = 20,000 at
    df = 1 / T (f up to 20 / d, every injected period in band); HBM GB/s of
    the dominant kernel against the roofline; false-peak rate on noise
    curves and exact-bin recovery on signal curves against the oracle."""
    from cuvarbase_gb300 import _lib
    from oracle import oracle as O
    nf = args.survey_nf
    b, kind, per = make_survey_batch(args.survey_curves)
    p = prepare(b)
    p["df"][:] = 1.0 / 1000.0
    nc = len(p["N"])
    h = _lib.Handle(sigma=-1.0, m=8, workspace_bytes=args.workspace_gb << 30)
    plan = h.plan(nf)
    window = h.plan_window(nf)[0]
    ms, prof, out = time_device_batch(h, p, nf, args.survey_steps, args.survey_warmup)
    best = time_best_e2e(h, p, nf, args.survey_steps, args.survey_warmup)
    st = {k: prof[k] for k in ("prep", "pass1", "pass2")}
    dom = max(st, key=lambda k: st[k][1])
    sb = stage_bytes(p, nf, plan, np.arange(nc))
    gbs = {k: sb[k] / (st[k][1] / args.survey_steps / 1000.0) / 1e9 for k in st}
    # oracle on a sample of noise and signal curves, full band
    rng = np.random.default_rng(23)
    noise = rng.choice(np.flatnonzero(kind == 0), args.survey_check, replace=False)
    signal = rng.choice(np.flatnonzero(kind > 0), args.survey_check, replace=False)
    freqs = (1 + np.arange(nf)) / 1000.0
    P = out.view(nc, nf)
    false_peaks, worst, recovered = 0, 0.0, 0
    for c in np.concatenate([noise, signal]):
        s, e = int(p["off"][c]), int(p["off"][c + 1])
        Pr = O.gls_flmean(p["t"][s:e], p["yw"][s:e], p["w"][s:e], freqs, p["yy"][c])
        Pg = P[c].cpu().numpy()
        worst = max(worst, float(np.abs(Pg - Pr).max()))
        if kind[c] == 0:
            false_peaks += int(np.argmax(Pg) != np.argmax(Pr))
        else:
            recovered += int(np.argmax(Pg) == np.argmax(Pr))
    h.close()
    del out, P
    return {"workload": f"{nc} curves, N uniform [20, 300], T=1000 d, nf={nf} at df=1/T "
                        "(f <= 20/d), 30% noise / 35% sinusoid / 35% sawtooth",
            "ms_per_step": ms, "lc_freq_per_s": nc * nf / (ms / 1000.0),
            "periodograms_per_s": nc / (ms / 1000.0),
            "plan": {"G1": plan[1], "G2": plan[2], "m": plan[3], "window": window},
            "e2e_best": best,
            "dominant": dom, "stage_ms_per_step": {k: st[k][1] / args.survey_steps for k in st},
            "stage_gbs": gbs, "roofline_frac": gbs[dom] / peak,
            "oracle_check": {"noise_curves": int(len(noise)), "false_peaks": false_peaks,
                             "signal_curves": int(len(signal)),
                             "peak_bin_equal_to_oracle": recovered,
                             "max_abs_dP": worst}}


def run_ours(args, rank, world):
    import torch

    from cuvarbase_gb300 import _lib
    from cuvarbase_gb300.replicas import max_over_ranks
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    b = make_batch(args.curves, seed=args.seed + 7919 * rank)
    p = prepare(b)
    nf = args.nf
    nc = args.curves
    ntot = int(p["off"][-1])
    sig = -1.0 if args.sigma == "auto" else float(args.sigma)
    h = _lib.Handle(sigma=sig, m=args.m, device=dev, workspace_bytes=args.workspace_gb << 30,
                    chunk_mb=args.chunk_mb)
    L = _lib.load()
    plan = h.plan(nf)
    window = h.plan_window(nf)
    t_d = torch.from_numpy(p["t"]).cuda()
    yw_d = torch.from_numpy(p["yw"]).cuda()
    w_d = torch.from_numpy(p["w"]).cuda()
    out_d = torch.empty(nc * nf, dtype=torch.float32, device="cuda")
    curves = curve_table(p, nf)

    def gls_input(t_ptr, yw_ptr, w_ptr, flags, cv=curves, n=nc, npts=ntot, nout=nc * nf):
        inp = _lib.GlsInput()
        inp.n_curves, inp.mode = n, _lib.MODE_FLOATING_MEAN
        inp.curves = ctypes.cast(cv, ctypes.c_void_p)
        inp.t, inp.yw, inp.w = t_ptr, yw_ptr, w_ptr
        inp.flags = flags
        inp.n_points_total, inp.n_out_total = npts, nout
        return inp

    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    dinp = gls_input(t_d.data_ptr(), yw_d.data_ptr(), w_d.data_ptr(), 0)

    def step():
        h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(dinp), ctypes.c_void_p(out_d.data_ptr()),
                                   sptr), "gls batch")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    h.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    prof = h.profile_read()
    h.profile(False)
    clk = clocks.stop()
    barrier()
    if world > 1:
        ms = max_over_ranks(ms)
    value = world * nc * args.steps / (ms / 1000.0)

    # accuracy check of this run's output on a few curves (oracle, subsample)
    acc = None
    if rank == 0 and args.check:
        from oracle import oracle as O
        P = out_d.view(nc, nf)
        worst, peaks = 0.0, 0
        rng = np.random.default_rng(3)
        cs = rng.integers(0, nc, args.check)
        for c in cs:
            s, e = p["off"][c], p["off"][c + 1]
            Pg = P[c].cpu().numpy()
            # every bin of the band, and the peak bin, against the oracle
            Pf = O.gls_flmean(p["t"][s:e], p["yw"][s:e], p["w"][s:e],
                              p["df"][c] * (1 + np.arange(nf)), p["yy"][c])
            worst = max(worst, float(np.abs(Pg - Pf).max()))
            peaks += int(int(np.argmax(Pf)) == int(np.argmax(Pg)))
        # injected periods: the GPU peak of every curve whose injected
        # frequency lies in the band (at most fmax - 10 df) against the bin
        # nearest to it, f_k = (1 + k) df
        fin = 1.0 / b["period"]
        kin = np.rint(fin / p["df"]).astype(np.int64) - 1
        inband = (fin <= p["df"] * (nf - 10)) & (kin >= 0)
        gpk = torch.argmax(P, dim=1).cpu().numpy()
        exact = int(np.sum(gpk[inband] == kin[inband]))
        # misses are the data's (low S/N, aliases): the oracle peaks where
        # the GPU does on a sample of them
        miss = np.flatnonzero(inband & (gpk != kin))[:args.check_misses]
        miss_same = 0
        for c in miss:
            s, e = p["off"][c], p["off"][c + 1]
            Pf = O.gls_flmean(p["t"][s:e], p["yw"][s:e], p["w"][s:e],
                              p["df"][c] * (1 + np.arange(nf)), p["yy"][c])
            miss_same += int(int(np.argmax(Pf)) == int(gpk[c]))
        acc = {"max_abs_dP": worst, "curves_checked": int(len(cs)),
               "bins_per_curve": f"{nf} (the whole band)",
               "peak_bin_equal_to_oracle": peaks,
               "injected_bin_recovered": exact, "injected_in_band": int(inband.sum()),
               "curves": nc, "misses_checked": int(len(miss)),
               "misses_with_oracle_peak_equal": miss_same}

    # roofline of the dominant stage
    st = {k: prof[k] for k in ("prep", "pass1", "pass2")}
    dom = max(st, key=lambda k: st[k][1])
    sb = stage_bytes(p, nf, plan, np.arange(nc))
    launches_dom = st[dom][0]
    bytes_per_launch = sb[dom] * args.steps / max(launches_dom, 1)
    avg_ms = st[dom][1] / max(launches_dom, 1)
    achieved = bytes_per_launch / (avg_ms / 1000.0) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
        per_curve = tr.get(dom, {}).get("dram_bytes_per_curve")
        if per_curve:
            traffic = per_curve * nc * args.steps / max(launches_dom, 1)
    except (OSError, ValueError):
        pass
    gpu_launches = int(sum(v[0] for v in prof.values()))

    # plain path: one curve per library call (same kernels, no batching)
    plain = None
    if args.plain_curves > 0:
        pc = min(args.plain_curves, nc)
        single = [curve_table(p, nf, first=c, count=1) for c in range(pc)]
        inps = [gls_input(t_d.data_ptr(), yw_d.data_ptr(), w_d.data_ptr(), 0, cv=single[c],
                          n=1) for c in range(pc)]
        for c in range(min(3, pc)):
            h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(inps[c]),
                                       ctypes.c_void_p(out_d.data_ptr()), sptr))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        for c in range(pc):
            h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(inps[c]),
                                       ctypes.c_void_p(out_d.data_ptr()), sptr))
        e1.record(stream)
        torch.cuda.synchronize()
        pms = max(e0.elapsed_time(e1), 1000.0 * (time.perf_counter() - t0))
        plain = {"value": pc / (pms / 1000.0), "unit": UNIT, "curves": pc,
                 "mode": "one curve per library call (binning, pass 1, pass 2), device-resident"}

    # e2e through the C ABI with page-locked host buffers
    e2e = None
    if args.e2e:
        tb = _lib.PinnedBuffer(ntot * 8)
        yb = _lib.PinnedBuffer(ntot * 4)
        wb = _lib.PinnedBuffer(ntot * 4)
        ob = _lib.PinnedBuffer(nc * nf * 4)
        tb.view(np.float64, ntot)[:] = p["t"]
        yb.view(np.float32, ntot)[:] = p["yw"]
        wb.view(np.float32, ntot)[:] = p["w"]
        hinp = gls_input(tb.ptr.value, yb.ptr.value, wb.ptr.value,
                         _lib.HOST_INPUT | _lib.HOST_OUTPUT)

        def hstep():
            h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(hinp), ob.ptr, sptr), "e2e")

        for _ in range(max(1, min(args.warmup, 2))):
            hstep()
        ems, reps = _time_host_steps(hstep, args.steps, stream, e0, e1, world)
        e2e = {"value": world * nc * args.steps / (ems / 1000.0), "unit": UNIT,
               "repetitions": [round(world * nc * args.steps / (r / 1000.0)) for r in reps],
               "h2d_bytes_per_step": int(ntot * 16 + nc * 96),
               "d2h_bytes_per_step": int(nc * nf * 4),
               "path": "cuvgls_gls_batch with CUVGLS_HOST_INPUT|CUVGLS_HOST_OUTPUT"}
        Ph = ob.view(np.float32, nc * nf)
        np.testing.assert_allclose(Ph[:nf], out_d[:nf].cpu().numpy(), atol=1e-5)
        e2e_prepared = e2e

        # the headline e2e: raw (t, y, dy) from page-locked host memory, the
        # host preparation of the reference (normalisation, weights, yw, YY)
        # done on the device (cuvgls_gls_raw), powers back to host memory
        rt = _lib.PinnedBuffer(ntot * 8)
        ry = _lib.PinnedBuffer(ntot * 8)
        rd = _lib.PinnedBuffer(ntot * 8)
        rt.view(np.float64, ntot)[:] = b["t"]
        ry.view(np.float64, ntot)[:] = b["y"]
        rd.view(np.float64, ntot)[:] = b["dy"]
        rcv = (_lib.RawCurve * nc)()
        for i in range(nc):
            c = rcv[i]
            c.pt_off, c.n, c.nf, c.k0 = int(b["off"][i]), int(b["N"][i]), nf, 1
            c.df, c.out_off = float(p["df"][i]), i * nf
        rinp = _lib.RawInput()
        rinp.n_curves, rinp.mode = nc, _lib.MODE_FLOATING_MEAN
        rinp.curves = ctypes.cast(rcv, ctypes.c_void_p)
        rinp.t, rinp.y, rinp.dy = rt.ptr.value, ry.ptr.value, rd.ptr.value
        rinp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
        rinp.n_points_total, rinp.n_out_total = ntot, nc * nf

        def rstep():
            h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(rinp), ob.ptr, None, None, sptr),
                    "e2e raw")

        for _ in range(max(1, min(args.warmup, 2))):
            rstep()
        ems, reps = _time_host_steps(rstep, args.steps, stream, e0, e1, world)
        e2e = {"value": world * nc * args.steps / (ems / 1000.0), "unit": UNIT,
               "repetitions": [round(world * nc * args.steps / (r / 1000.0)) for r in reps],
               "h2d_bytes_per_step": int(ntot * 24 + nc * ctypes.sizeof(_lib.RawCurve)),
               "d2h_bytes_per_step": int(nc * nf * 4),
               "path": "cuvgls_gls_raw (raw t, y, dy; preparation on the device) with "
                       "CUVGLS_HOST_INPUT|CUVGLS_HOST_OUTPUT",
               "prepared_input": e2e_prepared}
        Ph = ob.view(np.float32, nc * nf)
        # raw vs host-prepared input: sum(yw) differs in its last bits
        np.testing.assert_allclose(Ph[:4 * nf], out_d[:4 * nf].cpu().numpy(), atol=2e-5)
        for buf in (rt, ry, rd):
            buf.close()

    serve = run_serve(args) if (args.serve and rank == 0) else None
    if rank != 0:
        return None
    cpu = None
    if args.cpu_seconds > 0:
        from oracle import oracle as O
        O.build()
        rng = np.random.default_rng(11)
        done, tot = 0, 0.0
        while tot < args.cpu_seconds and done < 64:
            tot += cpu_gls_sample(b, p, nf, rng.integers(0, nc, 1))
            done += 1
        cpu = {"value": done / tot, "unit": UNIT, "cores": O.max_threads(), "cpu": cpu_model(),
               "kind": "port",
               "sample": f"{done} random curves of the batch, full nf={nf}, FP64 direct sums "
                         f"(oracle/gls_oracle.c, OpenMP)"}
    res = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 (FP64 offsets/phases)", "data": "synthetic", "config": config(args),
           "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                        "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                        "peak_source": peak_src,
                        "stage_ms_per_step": {k: v[1] / args.steps for k, v in st.items()},
                        "stage_launches_per_step": {k: v[0] / args.steps for k, v in st.items()},
                        "stage_gbs": {k: sb[k] / (v[1] / args.steps / 1000.0) / 1e9
                                      if v[1] > 0 else None for k, v in st.items()},
                        "plan": {"G": plan[0], "G1": plan[1], "G2": plan[2], "m": plan[3],
                                 "sigma_eff": plan[0] / nf, "window": window[0],
                                 "sigma_window": window[1]}},
           "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": gpu_launches,
           "clocks": clk, "plain": plain, "accuracy": acc, "serve": serve}
    if plain:
        res["batched_over_plain"] = value / world / plain["value"]
    legs = {}
    if args.api_curves > 0:
        res["api"] = run_api(args, b, p)
    if args.plan_curves:
        res["plan"] = run_plan(args, b, p)
    if args.fft_curves > 0:
        res["fft_check"] = run_fft_check(args)
    if args.single_steps > 0:
        legs["single"] = run_single(args)
    if args.precision_leg:
        legs["precision"] = run_precision(args, peak)
    if args.survey_leg:
        legs["survey"] = run_survey(args, peak)
    if legs:
        res["configs"] = legs
    res["summary"] = summary(res)
    return res


def summary(res):
    """The figures the metric names, repeated in a short object at the end of
    the line: batched / plain, serving p50 / p99 per rate, accuracy against
    the oracle, config 3's subsample check."""
    out = {}
    if res.get("plain"):
        out["batched_over_plain"] = round(res["batched_over_plain"], 2)
        out["plain_per_s"] = round(res["plain"]["value"])
    if res.get("e2e"):
        out["e2e_per_s"] = round(res["e2e"]["value"])
    acc = res.get("accuracy")
    if acc:
        out["max_abs_dP"] = float(f"{acc['max_abs_dP']:.3g}")
        out["peak_bins_equal"] = f"{acc['peak_bin_equal_to_oracle']}/{acc['curves_checked']}"
        out["injected_exact"] = f"{acc['injected_bin_recovered']}/{acc['injected_in_band']}"
    sv = res.get("serve")
    if sv and sv.get("rates"):
        out["serve_p50_p99_ms"] = {str(int(r["rate_req_s"])): [round(r["p50_ms"], 2),
                                                          round(r["p99_ms"], 2)]
                                   for r in sv["rates"]}
        out["serve_host_pause_max_ms"] = {
            str(int(r["rate_req_s"])): round(r.get("host_pauses", {}).get("max_ms", 0.0), 1)
            for r in sv["rates"]}
    pr = res.get("configs", {}).get("precision")
    if pr:
        out["cfg3"] = {"bins_checked": pr.get("bins_checked"),
                       "mixed_max_abs_dP": float(f"{pr['mixed']['max_abs_dP']:.3g}"),
                       "fp32_max_abs_dP": float(f"{pr['fp32']['max_abs_dP']:.3g}"),
                       "peak_bin_exact": pr["mixed"]["peak_bin_exact"]}
    sg = res.get("configs", {}).get("single")
    if sg:
        out["cfg1_ms"] = {"api": round(sg["api_ms_per_periodogram"], 3),
                          "device": round(sg["device_ms_per_periodogram"], 3),
                          "max_abs_dP": float(f"{sg['max_abs_dP_device']:.3g}")}
    sv = res.get("configs", {}).get("survey")
    if sv:
        out["cfg5_per_s"] = round(sv["periodograms_per_s"])
    return out


_WATCHDOG = """
import sys, time
out = open(sys.argv[1], "w")
prev = time.perf_counter()
while True:
    time.sleep(0.001)
    now = time.perf_counter()
    if now - prev > 0.005:
        out.write("%.4f %.2f\\n" % (time.time(), 1000.0 * (now - prev)))
        out.flush()
    prev = now
"""


def _steal_ticks():
    """Host CPU time stolen from this machine (the steal column of /proc/stat)."""
    try:
        with open("/proc/stat") as f:
            fields = f.readline().split()
        return int(fields[8]) if fields[0] == "cpu" and len(fields) > 8 else None
    except (OSError, ValueError, IndexError):
        return None


class HostPauses:
    """A separate process that sleeps 1 ms at a time and logs every
    oversleep above 5 ms: pauses of the whole host (or VM), which stall the
    server's threads and this process alike, show up in it at the same
    moments.  Windows of the run are then checked against the log."""

    def __init__(self):
        import tempfile
        self.path = tempfile.mktemp(prefix="cuvgls_watchdog_")
        self.proc = subprocess.Popen([sys.executable, "-c", _WATCHDOG, self.path])
        self.steal0 = _steal_ticks()

    def stop(self):
        self.proc.kill()
        self.proc.wait()
        ev = []
        try:
            with open(self.path) as f:
                ev = [tuple(map(float, line.split())) for line in f if line.strip()]
            os.unlink(self.path)
        except (OSError, ValueError):
            pass
        s1 = _steal_ticks()
        steal = None if self.steal0 is None or s1 is None else s1 - self.steal0
        return ev, steal

    @staticmethod
    def window(ev, t0, t1):
        w = [ms for t, ms in ev if t0 <= t <= t1 + 0.5]
        return {"count": len(w), "max_ms": max(w) if w else 0.0}


def run_serve(args):
    """Serving loop (continuous batching): Poisson arrivals, N log-uniform in
    [100, 20000], nf log-uniform in [1e4, 1e6], 80 GB budget; p50 / p99
    latency and throughput per arrival rate, and the plain path (one request
    at a time, no batching) on a sample of the same requests."""
    from cuvarbase_gb300.serve import GLSServer, poisson_workload, run_poisson
    out = {"budget_gb": 80, "client_threads": args.serve_threads,
           "inflight": args.serve_inflight, "rates": []}
    sink = lambda f, P: None  # noqa: E731  (results are produced, then dropped)
    pauses = HostPauses()
    windows = []
    for rate, dur in zip(args.serve_rates, args.serve_seconds):
        wl = poisson_workload(rate, dur, seed=int(rate), with_freqs=False)
        with GLSServer(sigma=args.sigma if args.sigma == "auto" else float(args.sigma),
                       hbm_budget=80 << 30, warm=(10_000, 1_000_000),
                       inflight=args.serve_inflight) as srv:
            # warm-up: plans and workspaces
            [f.result() for f in run_poisson(srv, wl[:min(20, len(wl))], on_result=sink)]
            srv.reset_stats()
            # Python's collector stops every thread (the delivery thread too)
            # to scan what earlier legs left behind: collect and freeze that
            # first, and hold collection during the replay (~10k requests)
            gc.collect()
            gc.freeze()
            gc.disable()
            t0 = time.perf_counter()
            w0 = time.time()
            futs = run_poisson(srv, wl, on_result=sink, threads=args.serve_threads)
            for f in futs:
                f.result()
            el = time.perf_counter() - t0
            windows.append((w0, time.time()))
            gc.enable()
            gc.unfreeze()
            st = srv.stats()
        nfs = sum(fr[0] for *_, fr in wl)
        out["rates"].append({"rate_req_s": rate, "requests": len(wl), "p50_ms": st["p50_ms"],
                             "p99_ms": st["p99_ms"], "max_ms": st["max_ms"],
                             "ready_p50_ms": st["ready_p50_ms"],
                             "ready_p99_ms": st["ready_p99_ms"],
                             "lib_p99_ms": st["lib_p99_ms"], "lib_max_ms": st["lib_max_ms"],
                             "lag_p99_ms": st["lag_p99_ms"], "lag_max_ms": st["lag_max_ms"],
                             "throughput_req_s": len(wl) / el,
                             "lc_freq_per_s": nfs / el, "mean_batch": st["mean_batch"]})
    ev, steal = pauses.stop()
    for r, (w0, w1) in zip(out["rates"], windows):
        r["host_pauses"] = HostPauses.window(ev, w0, w1)
    out["host_pauses_note"] = ("oversleeps > 5 ms of a separate 1-ms sleeper process during "
                               "each rate's replay (host or VM pauses)")
    out["host_steal_ticks"] = steal
    # plain path: the same kind of requests one at a time, no overlap
    wl = poisson_workload(100.0, 1.0, seed=5, with_freqs=False)[:60]
    with GLSServer(sigma=args.sigma if args.sigma == "auto" else float(args.sigma),
                   hbm_budget=80 << 30, inflight=1, max_batch=1,
                   warm=(10_000, 1_000_000)) as srv:
        for _, t, y, dy, fr in wl[:5]:
            srv.submit(t, y, dy, nf=fr[0], df=fr[1], on_result=sink).result()
        srv.reset_stats()
        t0 = time.perf_counter()
        for _, t, y, dy, fr in wl:
            srv.submit(t, y, dy, nf=fr[0], df=fr[1], on_result=sink).result()
        el = time.perf_counter() - t0
        st = srv.stats()
    out["plain"] = {"requests": len(wl), "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                    "throughput_req_s": len(wl) / el,
                    "lc_freq_per_s": sum(fr[0] for *_, fr in wl) / el}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--curves", type=int, default=10000)
    ap.add_argument("--nf", type=int, default=100000)
    ap.add_argument("--seed", type=int, default=1002)
    ap.add_argument("--plain-curves", type=int, default=200)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-curves", type=int, default=4)
    ap.add_argument("--check", type=int, default=16,
                    help="curves whose whole band is checked against the FP64 oracle")
    ap.add_argument("--check-misses", type=int, default=8,
                    help="missed injected periods whose peak is checked against the oracle")
    ap.add_argument("--workspace-gb", type=int, default=16)
    ap.add_argument("--sigma", default="auto", help="oversampling, or 'auto' (autotuned)")
    ap.add_argument("--chunk-mb", type=int, default=0, help="per-chunk workspace (0: library default)")
    ap.add_argument("--m", type=int, default=8)
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--no-serve", dest="serve", action="store_false")
    ap.add_argument("--serve-rates", type=float, nargs="+",
                    default=[100.0, 1000.0, 5000.0, 10000.0, 20000.0])
    ap.add_argument("--serve-seconds", type=float, nargs="+", default=[4.0, 2.0, 1.0, 1.0, 0.5])
    ap.add_argument("--serve-threads", type=int, default=4, help="client threads submitting")
    ap.add_argument("--serve-inflight", type=int, default=4, help="batches in flight")
    ap.add_argument("--api-curves", type=int, default=1000,
                    help="curves of the Python-API leg (0: skip)")
    ap.add_argument("--api-steps", type=int, default=3)
    ap.add_argument("--plan-curves", type=int, nargs="*", default=[16, 256],
                    help="curves per batch of the captured-plan leg (none: skip)")
    ap.add_argument("--plan-nf", type=int, default=20000)
    ap.add_argument("--fft-curves", type=int, default=1000,
                    help="curves of the cuFFT cross-check of the NFFT (0: skip)")
    ap.add_argument("--fft-nf", type=int, default=100000)
    ap.add_argument("--fft-steps", type=int, default=5)
    ap.add_argument("--fft-check-curves", type=int, default=4)
    ap.add_argument("--plan-iters", type=int, default=200)
    ap.add_argument("--no-precision", dest="precision_leg", action="store_false",
                    help="skip the precision-stress leg (8 x 1e6 points, nf = 1.8e7)")
    ap.add_argument("--single-steps", type=int, default=5,
                    help="timed calls of the single-curve leg (N = 1000, nf = 50,000); 0 skips it")
    ap.add_argument("--prec-curves", type=int, default=8)
    ap.add_argument("--prec-n", type=int, default=1_000_000)
    ap.add_argument("--prec-steps", type=int, default=2)
    ap.add_argument("--prec-warmup", type=int, default=3)
    ap.add_argument("--prec-blocks", type=int, default=100,
                    help="1000-bin oracle blocks of the precision check (100 = 1e5 bins)")
    ap.add_argument("--no-survey", dest="survey_leg", action="store_false",
                    help="skip the survey leg (200,000 short curves, nf = 20,000)")
    ap.add_argument("--survey-curves", type=int, default=200_000)
    ap.add_argument("--survey-nf", type=int, default=20_000)
    ap.add_argument("--survey-steps", type=int, default=3)
    ap.add_argument("--survey-warmup", type=int, default=3)
    ap.add_argument("--survey-check", type=int, default=150)
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        res = run_reference(args, rank)
    else:
        if world > 1:
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
            torch.distributed.init_process_group("nccl")
        res = run_ours(args, rank, world)
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
