"""Bands wider than the largest grid (2048 x 4096 cells): the library runs
them as consecutive sub-bands of the same points, each centred on its own
grid.  Checked against the FP64 oracle on bins around every sub-band
boundary, the band edges, random bins and the peak."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def sample_bins(nf, n_sub, rng, extra=()):
    w = -(-nf // n_sub)
    parts = [np.arange(0, 200), np.arange(nf - 200, nf), rng.integers(0, nf, 2000)]
    for s in range(1, n_sub):
        parts.append(np.arange(s * w - 200, s * w + 200))
    parts.append(np.asarray(extra, dtype=np.int64))
    return np.unique(np.concatenate(parts))


def test_gls_band_wider_than_one_grid(oracle):
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    rng = np.random.default_rng(1003)
    N, T = 400, 3650.0
    df = 1.0 / (5 * T)
    nf = 6_000_000                      # sigma = 2: one grid holds at most 4.19e6
    k_inj = int(0.8 * nf)
    t = np.sort(rng.uniform(0, T, N))
    y = 0.3 * np.sin(2 * np.pi * df * (1 + k_inj) * t + 0.4) + rng.normal(0, 0.05, N)
    dy = np.full(N, 0.05)
    freqs = df * (1 + np.arange(nf))
    proc = LombScargleAsyncProcess(sigma=2, m=8)
    (f, P), = proc.run([(t, y, dy)], freqs=freqs)
    proc.finish()
    assert P.shape == (nf,)
    assert int(np.argmax(P)) == k_inj
    idx = sample_bins(nf, 2, rng, [k_inj])
    tt, yw, w, YY, _ = oracle.prepare_curve(t, y, dy)
    Pref = oracle.gls_flmean(tt, yw, w, freqs[idx], YY)
    d = np.abs(P[idx] - Pref)
    assert d.max() <= TOL, (d.max(), int(idx[np.argmax(d)]))


def test_gls_wide_band_same_as_narrow_pieces():
    """The sub-band split gives the result of calling each slice alone."""
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    rng = np.random.default_rng(5)
    N, T = 200, 1000.0
    df = 1.0 / (3 * T)
    nf = 5_000_000                      # two sub-bands; each half alone is one grid
    t = np.sort(rng.uniform(0, T, N))
    y = np.sin(2 * np.pi * t / 0.37) + rng.normal(0, 0.1, N)
    dy = np.full(N, 0.1)
    proc = LombScargleAsyncProcess(sigma=2, m=8)
    (f, P), = proc.run([(t, y, dy)], freqs=df * (1 + np.arange(nf)))
    proc.finish()
    P = P.copy()
    half = nf // 2
    (f2, P2), = proc.run([(t, y, dy)], freqs=df * (1 + half + np.arange(nf - half)))
    proc.finish()
    # different grids (sizes and centres): agreement at the accuracy level
    assert np.abs(P[half:] - P2).max() <= 2e-5


def test_nfft_band_wider_than_one_grid(oracle):
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess
    rng = np.random.default_rng(7)
    N = 150
    t = np.sort(rng.uniform(0, 1, N))
    y = np.cos(2 * np.pi * 3.0 * t) + 0.1 * rng.standard_normal(N)
    nf = 5_000_000                        # two sub-bands at sigma = 2
    df = 1.0 / (t.max() - t.min())        # samples_per_peak = 1
    f0 = -(nf // 2) * df
    proc = NFFTAsyncProcess(sigma=2, m=8, autoset_m=False)
    out, = proc.run([(t, y, nf)], minimum_frequency=f0, samples_per_peak=1)
    proc.finish()
    assert out.shape == (nf,)
    idx = sample_bins(nf, 2, rng)
    ref = oracle.nfft_direct(t, y, f0 + idx.astype(np.float64) * df)
    assert np.abs(out[idx] - ref).max() <= 2e-6 * np.abs(y).sum()
