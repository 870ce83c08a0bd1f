"""Raw (t, y, dy) input prepared on the GPU (cuvgls_gls_raw): the same powers
as the host-prepared cuvgls_gls_batch, against the FP64 oracle, in every
mode, with best-frequency output, with a non-finite point, and through
LombScargleAsyncProcess.run (which takes this path without preallocated
memory)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _curves(seed, n=24, nmin=40, nmax=900):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        N = int(rng.integers(nmin, nmax))
        T = rng.uniform(100, 2000)
        t = np.sort(rng.uniform(0, T, N)) + rng.uniform(-1e3, 1e3)   # arbitrary offsets
        y = 3.0 + rng.uniform(0.05, 0.5) * np.sin(2 * np.pi * t / rng.uniform(0.3, 30)) \
            + rng.normal(0, 0.1, N)
        dy = np.exp(rng.normal(np.log(0.05), 0.3, N))
        out.append((t, y, dy, 1.0 / (5 * T)))
    return out


def _on_device(arrays):
    """Device copies of host arrays (torch tensors) and their pointers."""
    import torch
    ts = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]
    torch.cuda.synchronize()
    return ts, [x.data_ptr() for x in ts]


def _raw(h, curves, nf, mode=1, lam=0.0, best=False, device=False):
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    t = np.concatenate([c[0] for c in curves])
    y = np.concatenate([c[1] for c in curves])
    dy = np.concatenate([c[2] for c in curves])
    if device:   # inputs and powers resident on the device
        import torch
        keep, (pt, py, pdy) = _on_device([t, y, dy])
    cv = (_lib.RawCurve * len(curves))()
    o = 0
    for i, c in enumerate(curves):
        a = cv[i]
        a.pt_off, a.n, a.nf, a.k0, a.df, a.out_off = o, len(c[0]), nf, 1, c[3], i * nf
        o += len(c[0])
    inp = _lib.RawInput()
    inp.n_curves, inp.mode = len(curves), mode
    inp.curves = ctypes.cast(cv, ctypes.c_void_p)
    inp.t, inp.y, inp.dy = t.ctypes.data, y.ctypes.data, dy.ctypes.data
    inp.reg[0], inp.reg[1], inp.reg[2] = lam, lam, 0.0
    inp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
    inp.n_points_total, inp.n_out_total = o, len(curves) * nf
    if best:
        bk = np.empty(len(curves), np.int64)
        bp = np.empty(len(curves), np.float32)
        h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(inp), None, bk.ctypes.data,
                                 bp.ctypes.data, None), "raw best")
        h.sync(None, -1)
        return bk, bp
    if device:
        inp.t, inp.y, inp.dy = pt, py, pdy
        inp.flags = 0
        out = torch.empty(len(curves) * nf, dtype=torch.float32, device="cuda")
        h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(inp), out.data_ptr(), None, None, None),
                "raw")
        h.sync(None, -1)
        return out.cpu().numpy().reshape(len(curves), nf)
    P = np.empty(len(curves) * nf, np.float32)
    h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(inp), P.ctypes.data, None, None, None), "raw")
    h.sync(None, -1)
    return P.reshape(len(curves), nf)


def _prepared(h, curves, nf, mode=1, lam=0.0, device=False):
    """The host-prepared path (LombScargleMemory.setdata + cuvgls_gls_batch)."""
    from cuvarbase_gb300 import _lib
    from cuvarbase_gb300.lombscargle import LombScargleMemory
    from cuvarbase_gb300.utils import normalize_light_curves
    L = _lib.load()
    data = normalize_light_curves([c[:3] for c in curves])
    mems = [LombScargleMemory(2, None, 8).setdata(t=t, y=y, dy=dy) for t, y, dy in data]
    t = np.concatenate([m.t for m in mems])
    yw = np.concatenate([m.yw for m in mems]).astype(np.float32)
    w = np.concatenate([m.w for m in mems]).astype(np.float32)
    cv = (_lib.Curve * len(curves))()
    o = 0
    for i, (m, c) in enumerate(zip(mems, curves)):
        a = cv[i]
        a.pt_off, a.n, a.nf, a.k0, a.df = o, len(m.t), nf, 1, c[3]
        a.yy, a.ybar, a.yw_sum, a.w_sum = float(m.yy), float(m.ybar), m.yw_sum, m.w_sum
        a.out_off = i * nf
        o += len(m.t)
    inp = _lib.GlsInput()
    inp.n_curves, inp.mode = len(curves), mode
    inp.curves = ctypes.cast(cv, ctypes.c_void_p)
    inp.t, inp.yw, inp.w = t.ctypes.data, yw.ctypes.data, w.ctypes.data
    inp.reg[0], inp.reg[1], inp.reg[2] = lam, lam, 0.0
    inp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
    inp.n_points_total, inp.n_out_total = o, len(curves) * nf
    if device:   # inputs and powers resident on the device
        import torch
        keep, (pt, pyw, pw) = _on_device([t, yw, w])
        inp.t, inp.yw, inp.w = pt, pyw, pw
        inp.flags = 0
        out = torch.empty(len(curves) * nf, dtype=torch.float32, device="cuda")
        h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(inp), out.data_ptr(), None), "batch")
        h.sync(None, -1)
        return out.cpu().numpy().reshape(len(curves), nf)
    P = np.empty(len(curves) * nf, np.float32)
    h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(inp), P.ctypes.data, None), "batch")
    h.sync(None, -1)
    return P.reshape(len(curves), nf)


@pytest.fixture(scope="module")
def h():
    from cuvarbase_gb300 import _lib
    hh = _lib.Handle(sigma=2.0, m=8)
    yield hh
    hh.close()


@pytest.mark.parametrize("mode,lam", [(1, 0.0), (0, 0.0), (2, 0.0), (1, 4.0)])
def test_raw_equals_host_prepared(h, mode, lam):
    curves = _curves(31)
    nf = 8000
    Pr = _raw(h, curves, nf, mode, lam)
    Pp = _prepared(h, curves, nf, mode, lam)
    # same arithmetic after the preparation; sum(yw) differs in its last bits
    assert np.abs(Pr - Pp).max() <= 1e-5


def test_raw_against_oracle_config1(h, oracle):
    from test_gpu_gls import cfg1_curve
    t, y, dy = cfg1_curve()
    df = 1.0 / (5 * 3650.0)
    nf = 50000
    P = _raw(h, [(t, y, dy, df)], nf)[0]
    Pref = oracle.gls_flmean(*oracle.prepare_curve(t, y, dy)[:3], df * (1 + np.arange(nf)),
                             oracle.prepare_curve(t, y, dy)[3])
    assert np.abs(P - Pref).max() <= 1e-4
    assert int(np.argmax(P)) == int(np.argmax(Pref))


def test_raw_best_frequency(h):
    curves = _curves(32)
    nf = 12000
    P = _raw(h, curves, nf)
    bk, bp = _raw(h, curves, nf, best=True)
    for i in range(len(curves)):
        j = int(np.argmax(P[i]))
        assert P[i][bk[i]] >= P[i][j] - 1e-6
        assert abs(float(bp[i]) - float(P[i][j])) <= 1e-6


def test_raw_non_finite_point_invalidates_only_its_curve(h):
    curves = _curves(33, n=4)
    bad = list(curves[1])
    y = bad[1].copy()
    y[5] = np.nan
    bad[1] = y
    curves[1] = tuple(bad)
    P = _raw(h, curves, 4000)
    assert np.all(P[1] == -1.0)
    good = _raw(h, [curves[0], curves[2], curves[3]], 4000)
    np.testing.assert_array_equal(P[[0, 2, 3]] >= 0, good >= 0)
    assert np.abs(P[[0, 2, 3]] - good).max() <= 1e-6


def test_run_api_raw_path_equals_memory_path():
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    curves = _curves(34, n=12)
    data = [c[:3] for c in curves]
    freqs = [c[3] * (1 + np.arange(6000)) for c in curves]
    p = LombScargleAsyncProcess(sigma=2)
    res = p.run(data, freqs=freqs)
    p.finish()                                  # powers are valid after finish()
    fast = [(f, np.copy(P)) for f, P in res]
    mem = p.preallocate(1000, nlcs=len(data), nf=6000, k0=1)
    slow = p.run(data, freqs=freqs, memory=mem)
    p.finish()
    for (f1, P1), (f2, P2) in zip(fast, slow):
        np.testing.assert_array_equal(f1, f2)
        assert np.abs(P1 - P2).max() <= 1e-5


@pytest.mark.parametrize("nmax", [900, 3000])
def test_host_input_in_two_phases_equals_device_input(h, nmax):
    """With host input and several FFT chunks the points of the first chunk
    are copied first and that chunk runs while the rest is copied on the
    copy stream; the powers equal those of the same batch resident on the
    device (one phase), for raw and host-prepared input, with curves of one
    and of several preparation segments."""
    curves = _curves(61 + nmax, n=40, nmin=40, nmax=nmax)
    nf = 3000
    for fn in (_raw, _prepared):
        Ph = fn(h, curves, nf)
        Pd = fn(h, curves, nf, device=True)
        np.testing.assert_array_equal(Ph >= 0, Pd >= 0)
        # (the spreading's float atomics sum in a run-dependent order)
        assert np.abs(Ph - Pd).max() <= 1e-5


def test_host_input_in_two_phases_with_sub_bands(h):
    """Host-prepared input whose bands are wider than one grid: each curve
    runs as two sub-bands over the same points, and the two input phases
    split the batch between bands of one curve; the powers equal those of
    the same batch resident on the device."""
    curves = _curves(71, n=10, nmin=100, nmax=600)
    nf = 5_000_000                      # sigma = 2: two sub-bands per curve
    Ph = _prepared(h, curves, nf)
    Pd = _prepared(h, curves, nf, device=True)
    np.testing.assert_array_equal(Ph >= 0, Pd >= 0)
    assert np.abs(Ph - Pd).max() <= 1e-5
