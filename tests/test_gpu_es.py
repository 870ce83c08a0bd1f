"""The ES ("exponential of semicircle") spreading window that the autotuner
picks (sigma='auto'): sigma 1.28, m = 5 (10 taps), its Fourier transform
tabulated per plan for the deconvolution.  Checked against the FP64 oracle
through the reference-style API: config-2 curves over the whole band, the GLS
modes and the amplitude prior, the adjoint NFFT against direct sums, bands
wider than one grid, raw input and best-frequency output.  Tolerance: max
|dP| <= 3e-5 (the autotuner's accuracy budget with margin; the gate of the
path is 1e-4)."""
import numpy as np
import pytest

from test_gpu_gls import cfg2_curve, oracle_P

pytestmark = pytest.mark.gpu

TOL_ES = 3e-5


def ls_auto(**kw):
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    return LombScargleAsyncProcess(sigma="auto", **kw)


def test_autotuned_plans_use_the_es_window():
    from cuvarbase_gb300 import _lib
    h = _lib.Handle(sigma=-1.0, m=8)
    try:
        for nf, shape in [(10000, (160, 80)), (20000, (160, 160)), (50000, (160, 400)),
                          (100000, (320, 400)), (200000, (640, 400))]:
            G, G1, G2, m = h.plan(nf)
            assert (G1, G2) == shape and m == 5 and G >= 1.28 * nf, (nf, G1, G2, m)
            assert h.plan_window(nf) == ("es", 1.28)
    finally:
        h.close()
    # explicit sigma and m keep the reference's Gaussian
    h = _lib.Handle(sigma=2.0, m=8)
    try:
        assert h.plan_window(100000) == ("gauss", 2.0)
    finally:
        h.close()


def test_es_config2_whole_band_against_oracle(oracle):
    rng = np.random.default_rng(2024)
    data, freqs = [], []
    for _ in range(12):
        t, y, dy, _ = cfg2_curve(rng)
        data.append((t, y, dy))
        freqs.append((1 + np.arange(100000)) / (5 * (t.max() - t.min())))
    p = ls_auto()
    res = p.run(data, freqs=freqs)
    p.finish()
    worst = 0.0
    for (t, y, dy), fr, (f, P) in zip(data, freqs, res):
        Pref = oracle_P(oracle, t, y, dy, fr)
        worst = max(worst, float(np.abs(P - Pref).max()))
        assert int(np.argmax(P)) == int(np.argmax(Pref))
    assert worst <= TOL_ES, worst


def test_es_modes_and_prior_against_oracle(oracle):
    rng = np.random.default_rng(12)
    t = np.sort(rng.uniform(0, 200, 300))
    y = 0.3 * np.sin(2 * np.pi * t / 2.7) + 0.1 * rng.normal(size=300) + 1.0
    dy = 0.1 * np.exp(0.2 * rng.normal(size=300))
    freqs = (1 + np.arange(30000)) / (5 * (t.max() - t.min()))
    tt, yw, w, YY, ybar = oracle.prepare_curve(t, y, dy)
    p = ls_auto()
    for kw, ref in [
        (dict(floating_mean=False), oracle.gls_tau(tt, yw, w, freqs, YY, ybar, mode=0)),
        (dict(window=True), oracle.gls_tau(tt, yw, w, freqs, YY, ybar, mode=2)),
        (dict(amplitude_prior=0.5), oracle.gls_flmean(tt, yw, w, freqs, YY, amplitude_prior=0.5)),
    ]:
        (f, P), = p.run([(t, y, dy)], freqs=freqs, **kw)
        p.finish()
        scale = max(1.0, float(np.abs(ref).max()))
        assert np.abs(P - ref).max() <= TOL_ES * scale, (kw, np.abs(P - ref).max())


@pytest.mark.parametrize("n,nf,f0", [(100, 500, None), (2000, 40000, 10.0), (300, 100000, 0.0)])
def test_es_nfft_against_direct_sums(oracle, n, nf, f0):
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess
    rng = np.random.RandomState(n)
    t = np.sort(rng.rand(n)) * 30.0
    y = np.cos(2 * np.pi * 3.0 * t) + 0.1 * rng.randn(n)
    df = 1.0 / (t.max() - t.min())
    k0 = -nf // 2 if f0 is None else int(f0 / df)   # first frequency k0 df
    proc = NFFTAsyncProcess(sigma="auto", autoset_m=False)
    out, = proc.run([(t, y, nf)], minimum_frequency=k0 * df, samples_per_peak=1)
    proc.finish()
    ref = oracle.nfft_direct(t, y, (k0 + np.arange(nf)) * df)
    assert np.abs(out - ref).max() <= 1e-5 * np.abs(y).sum()


def test_es_band_wider_than_one_grid(oracle):
    """nf = 8e6: two sub-bands (one ES grid of 2048 x 4096 cells holds at
    most 6.5e6 frequencies), bins around the split, the edges and the peak."""
    rng = np.random.default_rng(1004)
    N, T = 400, 3650.0
    df = 1.0 / (5 * T)
    nf = 8_000_000
    k_inj = int(0.7 * nf)
    t = np.sort(rng.uniform(0, T, N))
    y = 0.3 * np.sin(2 * np.pi * df * (1 + k_inj) * t + 0.4) + rng.normal(0, 0.05, N)
    dy = np.full(N, 0.05)
    freqs = df * (1 + np.arange(nf))
    p = ls_auto()
    (f, P), = p.run([(t, y, dy)], freqs=freqs)
    p.finish()
    assert int(np.argmax(P)) == k_inj
    w = -(-nf // 2)
    idx = np.unique(np.concatenate([np.arange(200), np.arange(nf - 200, nf),
                                    np.arange(w - 300, w + 300), rng.integers(0, nf, 2000),
                                    [k_inj]]))
    tt, yw, ww, YY, _ = oracle.prepare_curve(t, y, dy)
    Pref = oracle.gls_flmean(tt, yw, ww, freqs[idx], YY)
    assert np.abs(P[idx] - Pref).max() <= TOL_ES


def test_es_raw_input_and_best_frequency(oracle):
    from cuvarbase_gb300 import _lib
    from test_gpu_raw import _curves, _prepared, _raw
    h = _lib.Handle(sigma=-1.0, m=8)
    try:
        curves = _curves(77, n=20)
        nf = 60000
        Pr = _raw(h, curves, nf)
        Pp = _prepared(h, curves, nf)
        assert np.abs(Pr - Pp).max() <= 1e-5
        bk, bp = _raw(h, curves, nf, best=True)
        for i, (t, y, dy, df) in enumerate(curves[:6]):
            tt, yw, w, YY, _ = oracle.prepare_curve(t, y, dy)
            ref = oracle.gls_flmean(tt, yw, w, df * (1 + np.arange(nf)), YY)
            assert np.abs(Pr[i] - ref).max() <= TOL_ES
            assert abs(float(bp[i]) - float(ref.max())) <= TOL_ES
            assert ref[bk[i]] >= ref.max() - TOL_ES
    finally:
        h.close()
