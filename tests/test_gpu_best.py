"""Per-curve best frequency reduced on the GPU (cuvgls_gls_best) against the
argmax of the full periodogram, through the C ABI and through
batched_run_const_nfreq(only_return_best_freqs=True)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(curves, nf, k0=1):
    """Host-prepared GLS input for (t, y, dy, df) curves on nf bins."""
    from cuvarbase_gb300 import _lib
    from cuvarbase_gb300.lombscargle import LombScargleMemory
    mems = [LombScargleMemory(2, None, 8).setdata(t=t - t.mean(), y=y - y.mean(), dy=dy)
            for t, y, dy, _ in curves]
    t_all = np.concatenate([m.t for m in mems])
    yw_all = np.concatenate([m.yw for m in mems]).astype(np.float32)
    w_all = np.concatenate([m.w for m in mems]).astype(np.float32)
    cv = (_lib.Curve * len(mems))()
    o = 0
    for i, (m, c) in enumerate(zip(mems, curves)):
        a = cv[i]
        a.pt_off, a.n, a.nf, a.k0, a.df = o, len(m.t), nf, k0, c[3]
        a.yy, a.ybar, a.yw_sum, a.w_sum = float(m.yy), float(m.ybar), m.yw_sum, m.w_sum
        a.out_off = i * nf
        o += len(m.t)
    inp = _lib.GlsInput()
    inp.n_curves, inp.mode = len(mems), _lib.MODE_FLOATING_MEAN
    inp.curves = ctypes.cast(cv, ctypes.c_void_p)
    inp.t, inp.yw, inp.w = t_all.ctypes.data, yw_all.ctypes.data, w_all.ctypes.data
    inp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
    inp.n_points_total, inp.n_out_total = o, len(mems) * nf
    return inp, (cv, t_all, yw_all, w_all)


def _full_and_best(curves, nf):
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    h = _lib.Handle(sigma=2.0, m=8)
    try:
        inp, keep = _batch(curves, nf)
        P = np.empty(len(curves) * nf, np.float32)
        h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(inp), P.ctypes.data, None), "batch")
        h.sync(None, -1)
        bk = np.empty(len(curves), np.int64)
        bp = np.empty(len(curves), np.float32)
        h.check(L.cuvgls_gls_best(h.ptr, ctypes.byref(inp), bk.ctypes.data, bp.ctypes.data,
                                  None), "best")
        h.sync(None, -1)
    finally:
        h.close()
    return P.reshape(len(curves), nf), bk, bp


def _curve(rng, N, T, freq, amp=0.3, sn=0.1):
    t = np.sort(rng.uniform(0, T, N))
    y = amp * np.sin(2 * np.pi * freq * t + rng.uniform(0, 6.28)) + rng.normal(0, sn, N)
    return t, y, np.full(N, sn), 1.0 / (5 * T)


def test_best_equals_argmax_of_full_periodogram():
    rng = np.random.default_rng(21)
    nf = 20000
    curves = [_curve(rng, int(rng.integers(30, 400)), 500.0, rng.uniform(0.5, 7.0),
                     amp=rng.uniform(0.0, 0.4)) for _ in range(40)]
    P, bk, bp = _full_and_best(curves, nf)
    for i in range(len(curves)):
        j = int(np.argmax(P[i]))
        # same kernels, spreading atomics in another order: ties at ~1e-7
        assert P[i][bk[i]] >= P[i][j] - 1e-6, (i, bk[i], j)
        assert abs(float(bp[i]) - float(P[i][j])) <= 1e-6


def test_best_over_sub_bands_and_invalid_curve():
    rng = np.random.default_rng(22)
    T = 3650.0
    df = 1.0 / (5 * T)
    nf = 6_000_000                       # two sub-bands at sigma = 2
    k_inj = int(0.8 * nf)
    t = np.sort(rng.uniform(0, T, 300))
    y = 0.3 * np.sin(2 * np.pi * df * (1 + k_inj) * t) + rng.normal(0, 0.05, 300)
    flat = np.ones(200)                  # YY = 0: every power invalid
    curves = [(t, y, np.full(300, 0.05), df),
              (np.sort(rng.uniform(0, T, 200)), flat, np.full(200, 0.05), df)]
    P, bk, bp = _full_and_best(curves, nf)
    assert int(bk[0]) == k_inj == int(np.argmax(P[0]))
    assert abs(float(bp[0]) - float(P[0][k_inj])) <= 1e-6
    assert np.all(P[1] == -1.0)
    assert int(bk[1]) == -1 and float(bp[1]) == -1.0


def test_const_nfreq_best_matches_host_argmax():
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    rng = np.random.default_rng(23)
    datas = [_curve(rng, int(rng.integers(50, 200)), 100.0, f)[:3]
             for f in rng.uniform(1, 10, 30)]
    p = LombScargleAsyncProcess(sigma=2)
    kw = dict(samples_per_peak=3, batch_size=30, only_return_best_freqs=True)
    best_dev, sig_dev = p.batched_run_const_nfreq(datas, **kw)
    # the host argmax path (taken whenever a frequency mask is given)
    nf_probe = p.batched_run_const_nfreq(datas, samples_per_peak=3)[0][0]
    best_host, sig_host = p.batched_run_const_nfreq(
        datas, ignore_freq_mask=np.zeros(len(nf_probe), bool), **kw)
    same = np.asarray(best_dev) == np.asarray(best_host)
    assert same.mean() >= 0.95
    np.testing.assert_allclose(np.asarray(sig_dev)[same], np.asarray(sig_host)[same],
                               atol=1e-5)
