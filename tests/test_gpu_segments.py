"""Curves longer than one preparation segment (1024 points): binning counted
per segment, scanned per curve and scattered per segment, and raw-input
statistics reduced from per-segment partial sums.  Checked against the FP64
oracle and against the host-prepared path, around the segment boundary
(1023, 1024, 1025, 2048 points), in every GLS mode, with sub-bands, with
best-frequency output, with a non-finite point, through the no-alloc entry
point and for the adjoint NFFT."""
import ctypes

import numpy as np
import pytest

from test_gpu_raw import _prepared, _raw

pytestmark = pytest.mark.gpu


def _curves(seed, sizes, T=1500.0):
    rng = np.random.default_rng(seed)
    out = []
    for N in sizes:
        t = np.sort(rng.uniform(0, T, N)) + rng.uniform(-500, 500)
        y = 2.0 + 0.3 * np.sin(2 * np.pi * t / rng.uniform(0.3, 30)) + rng.normal(0, 0.1, N)
        dy = np.exp(rng.normal(np.log(0.05), 0.3, N))
        out.append((t, y, dy, 1.0 / (5 * T)))
    return out


SIZES = [1023, 1024, 1025, 2048, 2049, 5000, 12000, 300, 60]


@pytest.fixture(scope="module")
def h():
    from cuvarbase_gb300 import _lib
    hh = _lib.Handle(sigma=2.0, m=8)
    yield hh
    hh.close()


@pytest.mark.parametrize("mode,lam", [(1, 0.0), (0, 0.0), (2, 0.0), (1, 3.0)])
def test_raw_long_curves_equal_host_prepared(h, mode, lam):
    curves = _curves(41, SIZES)
    nf = 6000
    Pr = _raw(h, curves, nf, mode, lam)
    Pp = _prepared(h, curves, nf, mode, lam)
    assert np.abs(Pr - Pp).max() <= 1e-5


def test_long_curves_against_oracle(h, oracle):
    curves = _curves(42, [1025, 4096, 20000])
    nf = 20000
    P = _raw(h, curves, nf)
    rng = np.random.default_rng(0)
    for i, (t, y, dy, df) in enumerate(curves):
        tt, yw, w, YY, _ = oracle.prepare_curve(t, y, dy)
        idx = np.unique(np.concatenate([np.arange(100), rng.integers(0, nf, 300),
                                        [int(np.argmax(P[i]))]]))
        ref = oracle.gls_flmean(tt, yw, w, df * (1 + idx), YY)
        assert np.abs(P[i][idx] - ref).max() <= 1e-4
        full = oracle.gls_flmean(tt, yw, w, df * (1 + np.arange(nf)), YY)
        assert int(np.argmax(P[i])) == int(np.argmax(full))


def test_raw_long_curves_sub_bands_and_best(h):
    curves = _curves(43, [3000, 500])
    nf = 6_000_000                      # two sub-bands at sigma = 2
    Pr = _raw(h, curves, nf)
    Pp = _prepared(h, curves, nf)
    assert np.abs(Pr - Pp).max() <= 1e-5
    bk, bp = _raw(h, curves, nf, best=True)
    for i in range(len(curves)):
        j = int(np.argmax(Pr[i]))
        assert Pr[i][bk[i]] >= Pr[i][j] - 1e-6
        assert abs(float(bp[i]) - float(Pr[i][j])) <= 1e-6


def test_non_finite_point_in_a_long_curve(h):
    curves = _curves(44, [3000, 2500, 700])
    t, y, dy, df = curves[1]
    y = y.copy()
    y[2100] = np.nan                     # third segment of the curve
    curves[1] = (t, y, dy, df)
    P = _raw(h, curves, 4000)
    assert np.all(P[1] == -1.0)
    good = _raw(h, [curves[0], curves[2]], 4000)
    assert np.abs(P[[0, 2]] - good).max() <= 1e-6


def test_no_alloc_long_curves(h):
    torch = pytest.importorskip("torch")
    from cuvarbase_gb300 import _lib
    from oracle import oracle as O
    L = _lib.load()
    curves = _curves(45, [3000, 1025, 200])
    nf = 20000
    ts, yws, ws, rows, off = [], [], [], [], 0
    for i, (t, y, dy, df) in enumerate(curves):
        tt, yw, w, YY, ybar = O.prepare_curve(t, y, dy)
        ts.append(tt)
        yws.append(yw)
        ws.append(w)
        rows.append((off, len(tt), nf, 1, df, YY, ybar,
                     float(np.cumsum(yw, dtype=np.float32)[-1]), float(w.sum()), i * nf))
        off += len(tt)
    t_d = torch.from_numpy(np.concatenate(ts)).cuda()
    yw_d = torch.from_numpy(np.concatenate(yws)).cuda()
    w_d = torch.from_numpy(np.concatenate(ws)).cuda()
    cv = (_lib.Curve * len(rows))()
    for c, r in zip(cv, rows):
        (c.pt_off, c.n, c.nf, c.k0, c.df, c.yy, c.ybar, c.yw_sum, c.w_sum, c.out_off) = r
    inp = _lib.GlsInput()
    inp.n_curves, inp.mode = len(rows), _lib.MODE_FLOATING_MEAN
    inp.curves = ctypes.cast(cv, ctypes.c_void_p)
    inp.t, inp.yw, inp.w = t_d.data_ptr(), yw_d.data_ptr(), w_d.data_ptr()
    inp.n_points_total, inp.n_out_total = t_d.numel(), len(rows) * nf
    ref = torch.full((len(rows) * nf,), -7.0, dtype=torch.float32, device="cuda")
    out = torch.full((len(rows) * nf,), -7.0, dtype=torch.float32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(inp), ctypes.c_void_p(ref.data_ptr()),
                               stream), "gls batch")
    err = ctypes.create_string_buffer(256)
    rc = L.cuvgls_gls_noalloc(2.0, 8, ctypes.byref(inp), ctypes.c_void_p(out.data_ptr()),
                              None, stream, err, len(err))
    assert rc == 0, (rc, err.value)
    torch.cuda.synchronize()
    assert torch.abs(out - ref).max().item() <= 1e-4


def test_nfft_long_curve(oracle):
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess
    rng = np.random.default_rng(46)
    out = []
    for N in (3000, 1025, 40):
        t = np.sort(rng.uniform(0, 100, N))
        y = np.cos(2 * np.pi * t / 3.0) + 0.1 * rng.standard_normal(N)
        out.append((t, y, 4000))
    proc = NFFTAsyncProcess(sigma=2, m=8, autoset_m=False)
    res = proc.run(out, minimum_frequency=-200.0, samples_per_peak=1)
    proc.finish()
    for (t, y, nf), got in zip(out, res):
        df = 1.0 / (t.max() - t.min())
        ref = oracle.nfft_direct(t, y, -200.0 + np.arange(nf) * df)
        assert np.abs(got - ref).max() <= 2e-6 * np.abs(y).sum()


@pytest.mark.parametrize("N,nf", [(200_000, 2_000_000), (120_000, 409_600)])
def test_dense_column_blocks_against_oracle(h, oracle, N, nf):
    """Curves dense enough that pass 1 spreads by gather (long column tiles
    of 2048 and 1280 cells, thousands of records per column block)."""
    rng = np.random.default_rng(N)
    T = 1000.0
    df = 1.0 / (5 * T)
    k_inj = int(0.37 * nf)
    t = np.sort(rng.uniform(0, T, N))
    y = 0.05 * np.sin(2 * np.pi * df * (1 + k_inj) * t) + rng.normal(0, 0.2, N)
    dy = np.full(N, 0.2)
    P = _raw(h, [(t, y, dy, df)], nf)[0]
    assert int(np.argmax(P)) == k_inj
    tt, yw, w, YY, _ = oracle.prepare_curve(t, y, dy)
    idx = np.unique(np.concatenate([np.arange(200), np.arange(nf - 200, nf),
                                    rng.integers(0, nf, 1500), [k_inj]]))
    ref = oracle.gls_flmean(tt, yw, w, df * (1 + idx), YY)
    assert np.abs(P[idx] - ref).max() <= 1e-4


def test_dense_nfft_against_direct_sums(oracle):
    from cuvarbase_gb300.cunfft import NFFTAsyncProcess
    rng = np.random.default_rng(47)
    N, nf = 100_000, 2_000_000
    t = np.sort(rng.uniform(0, 100, N))
    y = np.cos(2 * np.pi * t / 3.0) + 0.1 * rng.standard_normal(N)
    proc = NFFTAsyncProcess(sigma=2, m=8, autoset_m=False)
    got, = proc.run([(t, y, nf)], minimum_frequency=-1000.0, samples_per_peak=1)
    proc.finish()
    df = 1.0 / (t.max() - t.min())
    idx = np.unique(np.concatenate([np.arange(100), rng.integers(0, nf, 1000)]))
    ref = oracle.nfft_direct(t, y, -1000.0 + idx * df)
    assert np.abs(got[idx] - ref).max() <= 2e-6 * np.abs(y).sum()
