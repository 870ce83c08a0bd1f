"""Adjoint NFFT on the GPU against FP64 direct sums (the designs of
cuvarbase/tests/test_nfft.py:115-289, on the reference tests' own data)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIGMA, M = 5, 8
RTOL = ATOL = 5e-3      # the reference's NFFT tolerances (test_nfft.py:26-27)


def data(seed=100, ndata=100, spp=1):
    rand = np.random.RandomState(seed)
    t = np.sort(rand.rand(ndata))
    y = np.cos(2 * np.pi * (3. / (max(t) - min(t))) * t)
    tsc = (t - min(t)) / (spp * (max(t) - min(t))) - 0.5
    y += 0.1 * rand.randn(len(t))
    return t, tsc, y


def gpu_nfft(t, y, nf, **kw):
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess
    proc = NFFTAsyncProcess(sigma=kw.pop("sigma", SIGMA), m=M, autoset_m=False)
    res = proc.run([(t, y, nf)], **kw)
    proc.finish()
    return res[0]


def test_grid_matches_reference_scalar_gridding(golden):
    """just_return_gridded_data against the reference's gpu_grid_scalar."""
    g = golden
    nf = int(g["nf_nf"])
    grid = gpu_nfft(g["nf_t"], g["nf_y"], nf, just_return_gridded_data=True,
                    minimum_frequency=-int(nf / 2), samples_per_peak=1)
    np.testing.assert_allclose(grid, g["nf_grid"], rtol=RTOL, atol=1e-5)


@pytest.mark.parametrize("spp,scaled,f0", [(1, True, None), (5, True, None),
                                           (1, True, 10.), (1, False, None),
                                           (5, False, 0.)])
def test_nfft_against_direct_sums(oracle, spp, scaled, f0):
    t, tsc, y = data(spp=spp)
    nf = int(SIGMA * len(t))
    df = 1. / (spp * (max(t) - min(t)))
    if f0 is None:
        f0 = -0.5 * nf * df
    k0 = int(f0 / df)
    f0 = k0 if scaled else k0 * df
    tg = tsc if scaled else t
    out = gpu_nfft(tg, y, nf, minimum_frequency=f0, samples_per_peak=spp)
    freqs = float(k0) + np.arange(nf)
    if not scaled:
        freqs *= df
    ref = oracle.nfft_direct(tg, y, freqs)
    # much tighter than the reference's 5e-3: relative to sum |y|
    scale = np.abs(y).sum()
    assert np.abs(out - ref).max() <= 2e-6 * scale
    np.testing.assert_allclose(out.real, ref.real, rtol=RTOL, atol=ATOL)
    np.testing.assert_allclose(out.imag, ref.imag, rtol=RTOL, atol=ATOL)


def test_fractional_first_frequency(oracle):
    t, tsc, y = data()
    nf = 300
    df = 1. / (max(t) - min(t))
    f0 = 3.37 * df
    out = gpu_nfft(t, y, nf, minimum_frequency=f0, samples_per_peak=1)
    ref = oracle.nfft_direct(t, y, f0 + df * np.arange(nf))
    assert np.abs(out - ref).max() <= 2e-6 * np.abs(y).sum()


def test_absolute_time_phase(oracle):
    """Times far from zero (MJD-like): the output phase exp(2 pi i f t) is
    kept with FP64 range reduction."""
    rng = np.random.default_rng(2)
    t = 58000.0 + np.sort(rng.uniform(0, 300, 500))
    y = rng.normal(size=500)
    nf = 20000
    df = 1. / (2 * (t.max() - t.min()))
    out = gpu_nfft(t, y, nf, minimum_frequency=0.0, samples_per_peak=2, sigma=2)
    idx = np.concatenate([np.arange(200), np.arange(nf - 200, nf)])
    ref = oracle.nfft_direct(t, y, df * idx)
    assert np.abs(out[idx] - ref).max() <= 1e-5 * np.abs(y).sum()


def test_single_multi_batched_agree():
    """test_nfft_adjoint_async design: single vs multi vs batched runs."""
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess
    datas = []
    for i in range(10):
        t, tsc, y = data(seed=100 + i)
        datas.append((t, y, int(SIGMA * len(t))))
    kw = dict(minimum_frequency=0., samples_per_peak=1)
    singles = [np.copy(gpu_nfft(t, y, nf, **kw)) for t, y, nf in datas]
    proc = NFFTAsyncProcess(sigma=SIGMA, m=M, autoset_m=False)
    res = proc.run(datas, **kw)
    proc.finish()
    multi = [np.copy(x) for x in res]
    batched = [np.copy(x) for x in proc.batched_run(datas, batch_size=3, **kw)]
    for s, mu, b in zip(singles, multi, batched):
        np.testing.assert_allclose(s, mu, rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(s, b, rtol=1e-5, atol=1e-5)


def test_autoset_m():
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess
    p = NFFTAsyncProcess(sigma=2, autoset_m=True, tol=1e-8)
    assert p.get_m(1000) == p.m_from_C(1e-8 / 1000, 2)
    t, tsc, y = data()
    out = p.run([(t, y, 200)])
    p.finish()
    assert out[0].shape == (200,)


def test_use_double_is_fp64_direct_sums(oracle):
    """use_double=True: FP64 direct sums, exact up to FP64 rounding."""
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess
    rng = np.random.default_rng(7)
    data_ = []
    for N, nf in ((300, 2000), (2500, 5000), (40, 777)):
        t = np.sort(rng.uniform(0, 3000, N))          # f t up to ~1e4 cycles
        y = np.cos(2 * np.pi * t / 1.7) + 0.1 * rng.standard_normal(N)
        data_.append((t, y, nf))
    proc = NFFTAsyncProcess(sigma=2, m=8, use_double=True)
    res = proc.run(data_, minimum_frequency=0.25, samples_per_peak=3)
    proc.finish()
    for (t, y, nf), got in zip(data_, res):
        assert got.dtype == np.complex128
        df = 1.0 / (3 * (t.max() - t.min()))
        ref = oracle.nfft_direct(t, y, 0.25 + np.arange(nf) * df)
        assert np.abs(got - ref).max() <= 1e-10 * np.abs(y).sum()


def test_use_grid_matches_reference_steps(oracle):
    """use_grid: shift, inverse FFT and deconvolution of a given grid."""
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess
    t, tsc, y = data()
    nf = 400
    proc = NFFTAsyncProcess(sigma=SIGMA, m=M)
    ng = int(SIGMA * nf)
    rng = np.random.default_rng(8)
    grid = rng.standard_normal(ng) + 1j * rng.standard_normal(ng)
    b = 2 * SIGMA * M / ((2 * SIGMA - 1) * np.pi)
    for f0 in (0.0, -37.5):
        got = proc.run([(t, y, nf)], use_grid=grid, minimum_frequency=f0,
                       samples_per_peak=2)[0]
        ref = oracle.nfft_from_grid_np(grid, nf, t.min(), t.max(), 2.0, f0, b)
        assert got.dtype == np.complex64
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


def test_use_grid_of_the_gridded_data_is_the_nfft(oracle):
    """The reference-convention grid of the data, finished through use_grid,
    is the adjoint NFFT within the reference's tolerances (the pipeline of
    cuvarbase/cunfft.py:163-308 in two calls)."""
    t, tsc, y = data()
    nf = int(SIGMA * len(t))
    k0 = int(-0.5 * nf)
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess
    proc = NFFTAsyncProcess(sigma=SIGMA, m=M)
    grid = proc.run([(tsc, y, nf)], just_return_gridded_data=True,
                    minimum_frequency=float(k0), samples_per_peak=1)[0]
    got = proc.run([(tsc, y, nf)], use_grid=grid, minimum_frequency=float(k0),
                   samples_per_peak=1)[0]
    ref = oracle.nfft_direct(tsc, y, float(k0) + np.arange(nf))
    np.testing.assert_allclose(got.real, ref.real, rtol=RTOL, atol=ATOL)
    np.testing.assert_allclose(got.imag, ref.imag, rtol=RTOL, atol=ATOL)
