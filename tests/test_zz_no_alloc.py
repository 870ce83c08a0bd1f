"""cuvgls_gls_noalloc: the GLS batch for callers that cannot allocate memory
(code inside a framework whose memory pool owns every device allocation, or a
real-time loop that may not touch the allocator once it runs).

The entry point takes device inputs and outputs and keeps every temporary in
one fixed static device array.  These tests call it through the C ABI, twice
in a row on different batches (the second mixing two nf values, so the plan
of the larger band also serves the smaller one), and check each result
against the FP64 oracle and against cuvgls_gls_batch, the allocating entry
point, within the GLS tolerance of the test suite (max |dP| <= 1e-4).  They
also check the device error word the call hands back and its size limits.
They need nothing from the other test files, so they run the same alone in a
fresh process and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _batch(seed, nfs):
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    ts, yws, ws, rows, ref = [], [], [], [], []
    off = oo = 0
    for i, nf in enumerate(nfs):
        n = int(rng.integers(40, 900))
        T = rng.uniform(50, 1500)
        t = np.sort(rng.uniform(0, T, n))
        y = 0.3 * np.sin(2 * np.pi * t / rng.uniform(0.3, 20)) + rng.normal(0, 0.1, n)
        dy = np.exp(rng.normal(np.log(0.1), 0.2, n))
        tt, yw, w, YY, ybar = O.prepare_curve(t, y, dy)
        df = 1.0 / (5 * (tt.max() - tt.min()))
        ts.append(tt)
        yws.append(yw)
        ws.append(w)
        rows.append((off, n, nf, 1, df, YY, ybar,
                     float(np.cumsum(yw, dtype=np.float32)[-1]), float(w.sum()), oo))
        ref.append((oo, nf, (tt, yw, w, df * (1 + np.arange(nf)), YY)))
        off += n
        oo += nf
    return np.concatenate(ts), np.concatenate(yws), np.concatenate(ws), rows, ref, oo


def _input(_lib, rows, t_d, yw_d, w_d, n_out):
    curves = (_lib.Curve * len(rows))()
    for c, r in zip(curves, rows):
        (c.pt_off, c.n, c.nf, c.k0, c.df, c.yy, c.ybar, c.yw_sum, c.w_sum, c.out_off) = r
    inp = _lib.GlsInput()
    inp.n_curves, inp.mode = len(rows), _lib.MODE_FLOATING_MEAN
    inp.curves = ctypes.cast(curves, ctypes.c_void_p)
    inp.t, inp.yw, inp.w = t_d.data_ptr(), yw_d.data_ptr(), w_d.data_ptr()
    inp.flags = 0
    inp.n_points_total, inp.n_out_total = t_d.numel(), n_out
    return inp, curves


def _device(torch, t, yw, w):
    return (torch.from_numpy(t).cuda(), torch.from_numpy(yw).cuda(),
            torch.from_numpy(w).cuda())


def test_no_alloc_entry_point_matches_oracle_and_batch_twice_in_a_row():
    torch = pytest.importorskip("torch")
    from cuvarbase_gb300 import _lib
    from cuvarbase_gb300 import build as B
    from oracle import oracle as O
    B.build()
    L = _lib.load()
    h = _lib.Handle(sigma=2.0, m=8)
    err = ctypes.create_string_buffer(256)
    flags = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    for seed, nfs in ((21, [30000] * 6), (22, [20000, 70000, 20000])):
        t, yw, w, rows, ref, n_out = _batch(seed, nfs)
        t_d, yw_d, w_d = _device(torch, t, yw, w)
        Pbat = torch.full((n_out,), -7.0, dtype=torch.float32, device="cuda")
        out = torch.full((n_out,), -7.0, dtype=torch.float32, device="cuda")
        inp, keep = _input(_lib, rows, t_d, yw_d, w_d, n_out)
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(inp), ctypes.c_void_p(Pbat.data_ptr()),
                                   stream), "gls batch")
        flags.fill_(-1)
        rc = L.cuvgls_gls_noalloc(2.0, 8, ctypes.byref(inp), ctypes.c_void_p(out.data_ptr()),
                                  ctypes.c_void_p(flags.data_ptr()), stream, err, len(err))
        assert rc == 0, (rc, err.value)
        torch.cuda.synchronize()
        assert int(flags.item()) == 0
        P, Pb = out.cpu().numpy(), Pbat.cpu().numpy()
        assert np.all(P != -7.0)
        assert np.abs(P - Pb).max() <= TOL, np.abs(P - Pb).max()
        for oo, nf, (tt, ywc, wc, fr, YY) in ref:
            Pref = O.gls_flmean(tt, ywc, wc, fr, YY)
            Pc = P[oo:oo + nf]
            assert np.abs(Pc - Pref).max() <= TOL, (nf, np.abs(Pc - Pref).max())
            assert int(np.argmax(Pc)) == int(np.argmax(Pref))
    h.close()


def test_no_alloc_reports_nonfinite_input_in_its_flags_word():
    torch = pytest.importorskip("torch")
    from cuvarbase_gb300 import _lib
    from oracle import oracle as O
    L = _lib.load()
    t, yw, w, rows, ref, n_out = _batch(23, [5000, 5000])
    t = t.copy()
    t[rows[1][0] + 7] = np.nan        # one bad time in the second curve
    t_d, yw_d, w_d = _device(torch, t, yw, w)
    out = torch.full((n_out,), -7.0, dtype=torch.float32, device="cuda")
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    inp, keep = _input(_lib, rows, t_d, yw_d, w_d, n_out)
    err = ctypes.create_string_buffer(256)
    rc = L.cuvgls_gls_noalloc(2.0, 8, ctypes.byref(inp), ctypes.c_void_p(out.data_ptr()),
                              ctypes.c_void_p(flags.data_ptr()), None, err, len(err))
    assert rc == 0, (rc, err.value)
    torch.cuda.synchronize()
    f = int(flags.item())
    assert f & _lib.DEVERR_NONFINITE
    assert f & _lib.DEVERR_BINNING == 0
    # the clean curve is unaffected
    oo, nf, (tt, ywc, wc, fr, YY) = ref[0]
    Pref = O.gls_flmean(tt, ywc, wc, fr, YY)
    assert np.abs(out.cpu().numpy()[oo:oo + nf] - Pref).max() <= TOL


def test_no_alloc_rejects_batches_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    t, yw, w, rows, _, n_out = _batch(5, [400000] * 8)   # 8 x 3 x 819200 x 8 B > 32 MiB
    t_d, yw_d, w_d = _device(torch, t, yw, w)
    out = torch.empty(n_out, dtype=torch.float32, device="cuda")
    inp, keep = _input(_lib, rows, t_d, yw_d, w_d, out.numel())
    err = ctypes.create_string_buffer(256)
    rc = L.cuvgls_gls_noalloc(2.0, 8, ctypes.byref(inp), ctypes.c_void_p(out.data_ptr()),
                              None, None, err, len(err))
    assert rc == _lib.EBUDGET
    assert b"scratch" in err.value


def test_no_alloc_rejects_bands_wider_than_one_grid():
    torch = pytest.importorskip("torch")
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    nf = 5_000_000                      # above the largest single grid at sigma 2
    t, yw, w, rows, _, n_out = _batch(6, [nf])
    t_d, yw_d, w_d = _device(torch, t, yw, w)
    out = torch.empty(n_out, dtype=torch.float32, device="cuda")
    inp, keep = _input(_lib, rows, t_d, yw_d, w_d, out.numel())
    err = ctypes.create_string_buffer(256)
    rc = L.cuvgls_gls_noalloc(2.0, 8, ctypes.byref(inp), ctypes.c_void_p(out.data_ptr()),
                              None, None, err, len(err))
    assert rc == _lib.ENOTSUP
    assert b"plan" in err.value
