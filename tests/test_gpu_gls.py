"""GLS parity on the GPU: libcuvgls (through the reference-style API and the
C ABI) against the FP64 oracle.  Tolerance: max |dP| <= 1e-4 (the accuracy
gate of the path), peak bin equal to the oracle's."""
import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def cfg1_curve(seed=1001, N=1000, T=3650.0):
    rng = np.random.default_rng(seed)
    t = []
    while len(t) < N:
        c = rng.uniform(0, T, 4 * N)
        t.extend(c[(c / 365.25) % 1.0 >= 0.5].tolist())
    t = np.sort(np.array(t[:N]))
    y = 0.1 * np.sin(2 * np.pi * t / 0.73 + rng.uniform(0, 2 * np.pi)) + rng.normal(0, 0.05, N)
    return t, y, 0.05 * np.ones(N)


def cfg2_curve(rng, nmin=50, nmax=5000):
    N = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
    T = rng.uniform(100, 3650)
    t = np.sort(rng.uniform(0, T, N))
    P = np.exp(rng.uniform(np.log(0.1), np.log(100)))
    y = rng.uniform(0.05, 0.5) * np.sin(2 * np.pi * t / P + rng.uniform(0, 2 * np.pi))
    y = y + rng.normal(0, rng.uniform(0.02, 0.2), N)
    dy = np.exp(rng.normal(np.log(0.05), 0.3, N))
    return t, y, dy, P


def proc(**kw):
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    kw.setdefault("sigma", 2)
    kw.setdefault("m", 8)
    return LombScargleAsyncProcess(**kw)


def oracle_P(oracle, t, y, dy, freqs, **kw):
    tt, yw, w, YY, ybar = oracle.prepare_curve(t, y, dy)
    return oracle.gls_flmean(tt, yw, w, freqs, YY, **kw)


def assert_peak(P, Pref, tol=TOL):
    i, j = int(np.argmax(P)), int(np.argmax(Pref))
    assert i == j or abs(Pref[i] - Pref[j]) <= tol, (i, j, Pref[i], Pref[j])


def test_config1_full_band_against_oracle(oracle):
    t, y, dy = cfg1_curve()
    df = 1.0 / (5 * 3650.0)
    freqs = df * (1 + np.arange(50000))
    p = proc()
    (f, P), = p.run([(t, y, dy)], freqs=freqs)
    p.finish()
    Pref = oracle_P(oracle, t, y, dy, freqs)
    d = np.abs(P - Pref)
    assert d.max() <= TOL, (d.max(), int(np.argmax(d)))
    assert_peak(P, Pref)
    assert abs(1.0 / f[np.argmax(P)] - 0.73) < 1e-3


def test_reference_test_data_sigma5(golden, oracle):
    """The reference tests' own setting: N=100, sigma=5, spp=3, nyquist 3."""
    p = proc(sigma=5)
    (f, P), = p.run([(golden["ls_t_raw"], golden["ls_y_raw"], golden["ls_dy_raw"])],
                    nyquist_factor=3, samples_per_peak=3)
    p.finish()
    np.testing.assert_array_equal(f, golden["ls_freqs"])
    Pref = oracle_P(oracle, golden["ls_t_raw"], golden["ls_y_raw"], golden["ls_dy_raw"], f)
    assert np.abs(P - Pref).max() <= TOL
    # the reference's own direct sums (float32 t) agree at the same level
    assert np.abs(P - golden["ls_P"]).max() <= 2e-4
    assert_peak(P, golden["ls_P"])


@pytest.mark.parametrize("sigma", [2, "auto"])
def test_config2_shaped_batch_against_oracle(oracle, sigma):
    rng = np.random.default_rng(1002)
    data, freqs, periods = [], [], []
    for _ in range(16):
        t, y, dy, P = cfg2_curve(rng)
        data.append((t, y, dy))
        T = t.max() - t.min()
        freqs.append((1 + np.arange(100000)) / (5 * T))
        periods.append(P)
    p = proc(sigma=sigma)
    res = p.run(data, freqs=freqs)
    p.finish()
    worst = 0.0
    for (t, y, dy), fr, (f, P), per in zip(data, freqs, res, periods):
        idx = np.unique(np.concatenate([np.arange(300), rng.integers(0, 100000, 300),
                                        np.arange(99000, 100000), [np.argmax(P)]]))
        Pref = oracle_P(oracle, t, y, dy, fr[idx])
        worst = max(worst, np.abs(P[idx] - Pref).max())
    assert worst <= TOL, worst
    if sigma == "auto":
        # the autotuned plan: ES window at sigma 1.28, 10 taps, 320 x 400
        h = next(iter(p._handles.values()))
        G, G1, G2, m = h.plan(100000)
        assert (G, G1, G2, m) == (128000, 320, 400, 5)
        assert h.plan_window(100000) == ("es", 1.28)
        assert worst <= 3e-5


def test_modes_and_prior_against_oracle(oracle):
    rng = np.random.default_rng(11)
    t = np.sort(rng.uniform(0, 200, 300))
    y = 0.3 * np.sin(2 * np.pi * t / 2.7) + 0.1 * rng.normal(size=300) + 1.0
    dy = 0.1 * np.exp(0.2 * rng.normal(size=300))
    freqs = (1 + np.arange(3000)) / (5 * (t.max() - t.min()))
    tt, yw, w, YY, ybar = oracle.prepare_curve(t, y, dy)
    p = proc()
    for kw, ref in [
        (dict(floating_mean=False), oracle.gls_tau(tt, yw, w, freqs, YY, ybar, mode=0)),
        (dict(window=True), oracle.gls_tau(tt, yw, w, freqs, YY, ybar, mode=2)),
        (dict(amplitude_prior=0.5), oracle.gls_flmean(tt, yw, w, freqs, YY, amplitude_prior=0.5)),
    ]:
        (f, P), = p.run([(t, y, dy)], freqs=freqs, **kw)
        p.finish()
        scale = max(1.0, float(np.abs(ref).max()))
        assert np.abs(P - ref).max() <= TOL * scale, (kw, np.abs(P - ref).max())


def test_same_alone_and_in_the_mix(oracle):
    """Each curve's result in a ragged batch equals its result alone."""
    rng = np.random.default_rng(5)
    data, freqs = [], []
    for nf in (3000, 20000, 5000, 45000, 700):
        t, y, dy, _ = cfg2_curve(rng, 40, 2000)
        data.append((t, y, dy))
        freqs.append((1 + np.arange(nf)) / (5 * (t.max() - t.min())))
    p = proc()
    res = p.run(data, freqs=freqs)
    p.finish()
    mix = [np.copy(P) for _, P in res]
    for d, fr, Pm in zip(data, freqs, mix):
        (_, Pa), = p.run([d], freqs=fr)
        p.finish()
        assert np.abs(Pa - Pm).max() <= 1e-5


def test_batched_run_and_const_nfreq():
    """Reference test designs test_batched_run / test_batched_run_const_nfreq
    (cuvarbase/tests/test_lombscargle.py:177-247) with their tolerances."""
    rng = np.random.RandomState(100)

    def data(ndata, freq):
        t = np.sort(rng.rand(ndata))
        y = np.cos(2 * np.pi * freq * t) + 0.1 * rng.randn(ndata)
        return t, y, 0.1 * np.ones_like(y)

    datas = [data(rng.randint(50, 100), 3.0) for _ in range(5)]
    p = proc(sigma=5)
    kw = dict(nyquist_factor=3, samples_per_peak=3)
    batched = [(f, np.copy(P)) for f, P in p.batched_run(datas, **kw)]
    for d, (fb, pb) in zip(datas, batched):
        (fn, pn), = p.run([d], **kw)
        p.finish()
        np.testing.assert_allclose(pn, pb, rtol=1e-2, atol=1e-2)
        np.testing.assert_allclose(fn, fb, rtol=1e-2, atol=1e-2)
    freqs_true = 10 + rng.rand(27) * 100.
    datas = [data(rng.randint(50, 100), fr) for fr in freqs_true]
    res = p.batched_run_const_nfreq(datas, batch_size=5, samples_per_peak=3)
    p2 = proc(sigma=5)
    for d, (frq, pb) in zip(datas, res):
        (fn, pn), = p2.run([d], freqs=frq)
        p2.finish()
        np.testing.assert_allclose(pn, pb, rtol=1e-2, atol=1e-2)
    best, sig = p.batched_run_const_nfreq(datas, batch_size=27, samples_per_peak=3,
                                          only_return_best_freqs=True)
    assert len(best) == 27
    assert np.mean(np.abs(np.asarray(best) - freqs_true) < 0.5) > 0.8
    assert all(0 <= s <= 1 for s in sig)


def test_preallocated_memory_is_reused():
    rng = np.random.default_rng(3)
    p = proc()
    t, y, dy, _ = cfg2_curve(rng, 100, 300)
    freqs = (1 + np.arange(4000)) / (5 * (t.max() - t.min()))
    mem = p.preallocate(400, nlcs=2, freqs=freqs)
    r1 = p.run([(t, y, dy), (t, -y, dy)], freqs=freqs)
    p.finish()
    a = np.copy(r1[0][1])
    np.testing.assert_allclose(r1[0][1], r1[1][1], atol=1e-5)
    r2 = p.run([(t, 2 * y + 1, dy)], freqs=freqs)
    p.finish()
    assert r2[0][1].base is not None
    np.testing.assert_allclose(r2[0][1], a, atol=1e-5)  # GLS is scale / offset invariant
    assert mem[0].lsp_c is r1[0][1] or np.shares_memory(mem[0].lsp_c, r2[0][1])


def test_direct_sums_on_gpu(golden, oracle):
    from cuvarbase_gb300.lombscargle import lomb_scargle_direct_sums
    g = golden
    P = lomb_scargle_direct_sums(g["ls_t32"], g["ls_yw"], g["ls_w"], g["ls_freqs"], float(g["ls_yy"]))
    np.testing.assert_allclose(P, g["ls_P"], rtol=0, atol=2e-6)
    P = lomb_scargle_direct_sums(g["ls_t32"], g["ls_yw"], g["ls_w"], g["ls_freqs"],
                                 float(g["ls_yy"]), amplitude_priors=0.5)
    np.testing.assert_allclose(P, g["ls_P_prior"], rtol=0, atol=2e-6)
    # use_fft=False through the process API equals the NFFT path
    t, y, dy = g["ls_t_raw"], g["ls_y_raw"], g["ls_dy_raw"]
    p = proc(sigma=5)
    (f, Pd), = p.run([(t, y, dy)], use_fft=False, nyquist_factor=3, samples_per_peak=3)
    p.finish()
    Pd = np.copy(Pd)
    (f, Pn), = p.run([(t, y, dy)], nyquist_factor=3, samples_per_peak=3)
    p.finish()
    assert np.abs(Pd - Pn).max() <= TOL


def test_fp32_variant_is_less_accurate_at_long_baselines(oracle):
    t, y, dy = cfg1_curve(seed=77)
    df = 1.0 / (5 * 3650.0)
    freqs = df * (1 + np.arange(50000))
    Pref = oracle_P(oracle, t, y, dy, freqs)
    pm, pf = proc(), proc(precision="fp32")
    (_, Pm), = pm.run([(t, y, dy)], freqs=freqs)
    pm.finish()
    (_, Pf), = pf.run([(t, y, dy)], freqs=freqs)
    pf.finish()
    em, ef = np.abs(Pm - Pref).max(), np.abs(Pf - Pref).max()
    assert em <= TOL
    assert ef >= em


def test_julian_date_times(oracle):
    """Times given as Julian dates (t ~ 2.46e6 d, where FP32 keeps no
    fraction of a day): the powers still match the FP64 oracle."""
    t, y, dy = cfg1_curve(seed=78, N=800)
    t = t + 2458123.25
    df = 1.0 / (5 * 3650.0)
    freqs = df * (1 + np.arange(20000))
    Pref = oracle_P(oracle, t, y, dy, freqs)
    for kw in ({}, {"use_memory": True}):
        p = proc()
        if kw:
            mem = p.preallocate(len(t), nlcs=1, nf=len(freqs), k0=1)
            (_, P), = p.run([(t, y, dy)], freqs=freqs, memory=mem)
        else:
            (_, P), = p.run([(t, y, dy)], freqs=freqs)
        p.finish()
        assert np.abs(P - Pref).max() <= TOL
        assert_peak(P, Pref)


def test_edge_cases(oracle):
    p = proc()
    assert p.run([]) == []
    rng = np.random.default_rng(9)
    # two points: GLS with a floating mean is degenerate but must not crash
    t = np.array([0.0, 1.3])
    (f, P), = p.run([(t, np.array([1.0, 2.0]), np.ones(2))], freqs=0.1 * (1 + np.arange(16)))
    p.finish()
    assert np.all(np.isfinite(P))
    # three points, tiny band
    t = np.array([0.0, 0.7, 2.9])
    y = np.array([1.0, -0.5, 0.2])
    fr = 0.05 * (1 + np.arange(3))
    (f, P), = p.run([(t, y, np.ones(3))], freqs=fr)
    p.finish()
    Pref = oracle_P(oracle, t, y, np.ones(3), fr)
    ok = np.isfinite(Pref)
    assert np.abs(P[ok] - Pref[ok]).max() <= 1e-3
    # a large first frequency index (k0 >> nf): band far from zero
    t, y, dy, _ = cfg2_curve(rng, 200, 400)
    T = t.max() - t.min()
    df = 1.0 / (5 * T)
    fr = df * (200000 + np.arange(2000))
    (f, P), = p.run([(t, y, dy)], freqs=fr)
    p.finish()
    assert np.abs(P - oracle_P(oracle, t, y, dy, fr)).max() <= TOL


def test_undefined_power_is_reported_as_minus_one(oracle):
    """A curve whose GLS is undefined (one point, or constant y: YY = 0; the
    oracle gives NaN) has power -1 at every frequency, the reference's mark
    for an invalid power, on both preparation paths; its neighbour in the
    batch is unaffected."""
    rng = np.random.default_rng(12)
    fr = 0.1 * (1 + np.arange(64))
    t2, y2, dy2, _ = cfg2_curve(rng, 200, 400)
    cases = [(np.array([3.0]), np.array([1.0]), np.array([1.0])),
             (np.linspace(0, 10, 30), np.full(30, 2.5), np.ones(30)),
             (t2, y2, dy2)]
    for o in cases[:2]:
        with np.errstate(all="ignore"):
            assert np.all(np.isnan(oracle_P(oracle, *o, fr)))
    Pref = oracle_P(oracle, *cases[2], fr)
    for use_memory in (False, True):
        p = proc()
        if use_memory:   # host preparation into preallocated memory
            mem = p.preallocate(400, nlcs=len(cases), nf=len(fr), k0=1)
            res = p.run(cases, freqs=fr, memory=mem)
        else:            # raw input, prepared on the device
            res = p.run(cases, freqs=fr)
        p.finish()
        for (f, P) in res[:2]:
            assert np.all(P == -1.0)
        assert np.abs(res[2][1] - Pref).max() <= TOL


def test_invalid_arguments_raise(handle):
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    inp = _lib.GlsInput()
    inp.n_curves = 1
    inp.mode = 7
    curves = (_lib.Curve * 1)()
    curves[0].n, curves[0].nf, curves[0].df = 10, 10, 0.1
    t = np.zeros(10)
    yw = np.zeros(10, np.float32)
    out = np.zeros(10, np.float32)
    inp.curves = ctypes.cast(curves, ctypes.c_void_p)
    inp.t, inp.yw, inp.w = t.ctypes.data, yw.ctypes.data, yw.ctypes.data
    inp.flags = 3
    inp.n_points_total, inp.n_out_total = 10, 10
    with pytest.raises(ValueError):
        handle.check(L.cuvgls_gls_batch(handle.ptr, ctypes.byref(inp), out.ctypes.data, None))
    inp.mode = 1
    curves[0].nf = 11  # output range outside the array
    with pytest.raises(ValueError):
        handle.check(L.cuvgls_gls_batch(handle.ptr, ctypes.byref(inp), out.ctypes.data, None))
    curves[0].nf = 10
    inp.reg[0], inp.reg[1] = 1.0, 2.0  # anisotropic prior: not what the API builds
    with pytest.raises(ValueError):
        handle.check(L.cuvgls_gls_batch(handle.ptr, ctypes.byref(inp), out.ctypes.data, None))


def test_budget_is_reported():
    """Over-budget batches raise MemoryError before anything is launched."""
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    rng = np.random.default_rng(4)
    t, y, dy, _ = cfg2_curve(rng, 500, 600)
    big = (1 + np.arange(400000)) / (5 * (t.max() - t.min()))
    small = LombScargleAsyncProcess(sigma=2, workspace_bytes=16 << 20)
    with pytest.raises(MemoryError):   # one grid set alone is ~20 MB
        small.run([(t, y, dy)] * 2, freqs=big)


def test_sync_deadline_returns_timeout_then_completes():
    """cuvgls_sync with a 1 ms deadline on a stream kept busy for ~0.3 s (a
    bounded clock-count kernel, no wait on anything) returns ETIMEOUT at the
    deadline; an unbounded sync afterwards returns OK."""
    torch = pytest.importorskip("torch")
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    h = _lib.Handle(sigma=2.0, m=8)
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    # nothing queued: a short deadline is met
    assert L.cuvgls_sync(h.ptr, sp, 100) == _lib.OK
    with torch.cuda.stream(s):
        torch.cuda._sleep(600_000_000)    # ~0.3 s at 2 GHz
    t0 = time.perf_counter()
    rc = L.cuvgls_sync(h.ptr, sp, 1)
    waited = time.perf_counter() - t0
    assert rc == _lib.ETIMEOUT, rc
    assert b"deadline" in L.cuvgls_last_error(h.ptr)
    assert waited < 0.25, waited          # returned at the deadline, not at the end
    assert L.cuvgls_sync(h.ptr, sp, -1) == _lib.OK
    h.close()


def test_nonfinite_input_is_flagged_not_fatal():
    from cuvarbase_gb300 import _lib
    rng = np.random.default_rng(6)
    t, y, dy, _ = cfg2_curve(rng, 100, 200)
    y = y.copy()
    y[5] = np.nan
    p = proc()
    fr = (1 + np.arange(1000)) / (5 * (t.max() - t.min()))
    # normalize_light_curves uses nanmean, weights stay finite; the NaN y
    # makes ybar NaN as in the reference, so the powers come back invalid
    (f, P), = p.run([(t, y, dy)], freqs=fr)
    p.finish()
    h = next(iter(p._handles.values()))
    assert h.device_flags() & _lib.DEVERR_NONFINITE
    assert np.all(P == -1.0)
