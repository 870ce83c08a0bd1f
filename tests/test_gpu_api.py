"""The reference's lower-level entry points against the FP64 oracle:
lomb_scargle_async (cuvarbase/lombscargle.py:579-689), nfft_adjoint_async
(cuvarbase/cunfft.py:163-308), lomb_scargle_simple
(cuvarbase/lombscargle.py:1187-1204) and
LombScargleAsyncProcess.memory_requirement (cuvarbase/lombscargle.py:752-796).
Tolerances: max |dP| <= 1e-4 for the FP32 GLS path, 1e-9 for the FP64
direct sums, 2e-6 sum|y| for the FP32 NFFT (the reference allows 5e-3)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def curve(seed, n=700, T=400.0, period=3.3):
    rng = np.random.default_rng(seed)
    t = np.sort(rng.uniform(0, T, n))
    y = 0.2 * np.sin(2 * np.pi * t / period + 0.4) + rng.normal(0, 0.08, n)
    dy = np.exp(rng.normal(np.log(0.08), 0.25, n))
    return t, y, dy


def grid(t, nf, k0=1, spp=5):
    df = 1.0 / (spp * (t.max() - t.min()))
    return df * (k0 + np.arange(nf))


def oracle_P(oracle, t, y, dy, freqs):
    tt, yw, w, YY, _ = oracle.prepare_curve(t, y, dy)
    return oracle.gls_flmean(tt, yw, w, freqs, YY)


def ls_proc(**kw):
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    kw.setdefault("sigma", 2)
    kw.setdefault("m", 8)
    return LombScargleAsyncProcess(**kw)


def _functions(proc, nf):
    """The (handle, stream) pair lomb_scargle_async takes where the reference
    takes its compiled kernels."""
    return proc._gls_handle(nf), proc._stream().ptr


@pytest.mark.parametrize("k0", [1, 37])
def test_lomb_scargle_async_fft_against_oracle(oracle, k0):
    from cuvarbase_gb300.lombscargle import lomb_scargle_async
    t, y, dy = curve(1)
    nf = 30000
    freqs = grid(t, nf, k0)
    p = ls_proc()
    mem = p.allocate_for_single_lc(t, y, dy, nf, k0=k0)
    out = lomb_scargle_async(mem, _functions(p, nf), freqs)
    assert out is mem.lsp_c
    p.finish()
    Pref = oracle_P(oracle, t, y, dy, freqs)
    assert np.abs(mem.lsp_c - Pref).max() <= TOL
    assert int(np.argmax(mem.lsp_c)) == int(np.argmax(Pref))


def test_lomb_scargle_async_direct_sums_against_oracle(oracle):
    """use_fft=False: the direct-sum kernel (FP32 sums of FP64 phases)."""
    from cuvarbase_gb300.lombscargle import lomb_scargle_async
    t, y, dy = curve(2, n=300)
    nf = 4000
    freqs = grid(t, nf)
    p = ls_proc()
    mem = p.allocate_for_single_lc(t, y, dy, nf, k0=1)
    lomb_scargle_async(mem, _functions(p, nf), freqs, use_fft=False)
    p.finish()
    Pref = oracle_P(oracle, t, y, dy, freqs)
    assert np.abs(mem.lsp_c - Pref).max() <= TOL


def test_lomb_scargle_async_python_dir_sums_branch(oracle):
    """python_dir_sums=True returns the FP64 direct sums of the memory's own
    (float32) yw and w, as the reference's branch does."""
    from cuvarbase_gb300.lombscargle import lomb_scargle_async
    t, y, dy = curve(3, n=250)
    nf = 3000
    freqs = grid(t, nf)
    p = ls_proc()
    mem = p.allocate_for_single_lc(t, y, dy, nf, k0=1)
    P = lomb_scargle_async(mem, _functions(p, nf), freqs, python_dir_sums=True)
    Pref = oracle.gls_flmean(mem.t, mem.yw.astype(np.float64), mem.w.astype(np.float64),
                             freqs, mem.yy)
    assert P.shape == (nf,)
    assert np.abs(P - Pref).max() <= 1e-9


def test_lomb_scargle_async_checks_k0():
    from cuvarbase_gb300.lombscargle import lomb_scargle_async
    t, y, dy = curve(4, n=100)
    nf = 1000
    freqs = grid(t, nf, k0=5)
    p = ls_proc()
    mem = p.allocate_for_single_lc(t, y, dy, nf, k0=4)   # memory for another grid
    with pytest.raises(AssertionError):
        lomb_scargle_async(mem, _functions(p, nf), freqs)


def test_lomb_scargle_simple_against_oracle(oracle):
    from cuvarbase_gb300.lombscargle import lomb_scargle_simple
    from cuvarbase_gb300.utils import autofrequency
    t, y, dy = curve(5, n=400, T=200.0)
    freqs = grid(t, 20000)
    f, P = lomb_scargle_simple(t, y, dy, freqs=freqs)
    assert np.array_equal(f, freqs)
    Pref = oracle_P(oracle, t, y, dy, freqs)
    assert np.abs(P - Pref).max() <= TOL
    # default grid: the reference's autofrequency
    f, P = lomb_scargle_simple(t, y, dy)
    np.testing.assert_array_equal(f, autofrequency(t))
    Pref = oracle_P(oracle, t, y, dy, f)
    assert np.abs(P - Pref).max() <= TOL
    assert int(np.argmax(P)) == int(np.argmax(Pref))


def test_memory_requirement_is_enough_to_run_the_batch(oracle):
    """A process whose workspace is exactly memory_requirement(n0, nf, k0,
    nbatch) runs nbatch curves of n0 points and nf frequencies, through the
    run() path (raw host input, host output)."""
    n0, nf, k0, nbatch = 3000, 100000, 1, 8
    p0 = ls_proc(sigma=4)
    req = p0.memory_requirement(n0, nf, k0, nbatch=nbatch)
    G = p0._gls_handle(nf).plan(nf)[0]
    assert req >= nbatch * (3 * G * 8 + 40 * n0)       # grids and records at least
    assert req <= 2 * nbatch * (3 * G * 8 + 64 * n0 + 4 * nf) + (1 << 20)
    data = [curve(100 + i, n=n0, T=1000.0) for i in range(nbatch)]
    freqs = grid(data[0][0], nf, k0)
    p = ls_proc(sigma=4, workspace_bytes=req)
    res = p.run(data, freqs=freqs)
    p.finish()
    for (t, y, dy), (f, P) in zip(data[:3], res[:3]):
        Pref = oracle_P(oracle, t, y, dy, f)
        assert np.abs(P - Pref).max() <= TOL


# ---- nfft_adjoint_async --------------------------------------------------

def _nfft_setup(use_double=False, sigma=2, m=8):
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess, NFFTMemory
    proc = NFFTAsyncProcess(sigma=sigma, m=m, use_double=use_double)
    rng = np.random.default_rng(11)
    t = np.sort(rng.uniform(0, 250, 900))
    y = np.cos(2 * np.pi * t / 2.1) + 0.2 * rng.standard_normal(len(t))
    nf = 6000
    mem = NFFTMemory(sigma, proc._stream(), m, use_double=use_double)
    mem.fromdata(t, y, nf=nf, allocate=True)
    functions = (proc._handle(proc._lib_sigma(), m), proc._stream().ptr)
    return proc, mem, functions, t, y, nf


@pytest.mark.parametrize("f0", [0.0, 1.37])
def test_nfft_adjoint_async_against_direct_sums(oracle, f0):
    from cuvarbase_gb300.cunfft import nfft_adjoint_async
    proc, mem, fn, t, y, nf = _nfft_setup()
    spp = 3
    out = nfft_adjoint_async(mem, fn, minimum_frequency=f0, samples_per_peak=spp)
    assert out is mem.ghat_c
    proc.finish()
    df = 1.0 / (spp * (t.max() - t.min()))
    ref = oracle.nfft_direct(t, y, f0 + df * np.arange(nf))
    assert mem.ghat_c.dtype == np.complex64
    assert np.abs(mem.ghat_c - ref).max() <= 2e-6 * np.abs(y).sum()


def test_nfft_adjoint_async_use_double(oracle):
    from cuvarbase_gb300.cunfft import nfft_adjoint_async
    proc, mem, fn, t, y, nf = _nfft_setup(use_double=True)
    nfft_adjoint_async(mem, fn, minimum_frequency=0.5, samples_per_peak=2)
    proc.finish()
    df = 1.0 / (2 * (t.max() - t.min()))
    ref = oracle.nfft_direct(t, y, 0.5 + df * np.arange(nf))
    assert mem.ghat_c.dtype == np.complex128
    assert np.abs(mem.ghat_c - ref).max() <= 1e-10 * np.abs(y).sum()


def test_nfft_adjoint_async_just_return_gridded_data(golden, oracle):
    """The reference-convention real grid, against the reference's own
    gpu_grid_scalar output and the C restatement of its gridding."""
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess, NFFTMemory, nfft_adjoint_async
    g = golden
    nf = int(g["nf_nf"])
    proc = NFFTAsyncProcess(sigma=5, m=8)
    mem = NFFTMemory(5, proc._stream(), 8).fromdata(g["nf_t"], g["nf_y"], nf=nf)
    grid_ = nfft_adjoint_async(mem, (proc._handle(5.0, 8), proc._stream().ptr),
                               just_return_gridded_data=True,
                               minimum_frequency=-int(nf / 2), samples_per_peak=1)
    np.testing.assert_allclose(grid_, g["nf_grid"], rtol=5e-3, atol=1e-5)
    ref = oracle.grid_ref(g["nf_t"], g["nf_y"], 5 * nf, 8, 5.0)
    assert np.abs(grid_ - ref).max() <= 1e-5 * np.abs(g["nf_y"]).sum()
