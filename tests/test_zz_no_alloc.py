"""cuvgls_gls_noalloc: the GLS batch for callers that cannot allocate memory
(code inside a framework that owns every device allocation, code running
under stream capture, real-time loops that may not touch the allocator).

The entry point takes device inputs and outputs and keeps every temporary in
one fixed static device array.  This test calls it through the C ABI twice in
a row on different batches and checks each result against cuvgls_gls_batch,
the allocating entry point, within the GLS tolerance of the test suite
(max |dP| <= 1e-4).  It needs nothing from the other test files, so it runs
the same alone in a fresh process and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _batch(seed, n_curves, nf):
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    ts, yws, ws, rows = [], [], [], []
    off = 0
    for i in range(n_curves):
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
                     float(np.cumsum(yw, dtype=np.float32)[-1]), float(w.sum()), i * nf))
        off += n
    return np.concatenate(ts), np.concatenate(yws), np.concatenate(ws), rows


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


def test_no_alloc_entry_point_matches_batch_twice_in_a_row():
    torch = pytest.importorskip("torch")
    from cuvarbase_gb300 import _lib
    from cuvarbase_gb300 import build as B
    B.build()
    L = _lib.load()
    h = _lib.Handle(sigma=2.0, m=8)
    err = ctypes.create_string_buffer(256)
    for seed, n_curves, nf in ((21, 6, 30000), (22, 3, 70000)):
        t, yw, w, rows = _batch(seed, n_curves, nf)
        t_d = torch.from_numpy(t).cuda()
        yw_d = torch.from_numpy(yw).cuda()
        w_d = torch.from_numpy(w).cuda()
        n_out = n_curves * nf
        ref = torch.full((n_out,), -7.0, dtype=torch.float32, device="cuda")
        out = torch.full((n_out,), -7.0, dtype=torch.float32, device="cuda")
        inp, keep = _input(_lib, rows, t_d, yw_d, w_d, n_out)
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        h.check(L.cuvgls_gls_batch(h.ptr, ctypes.byref(inp), ctypes.c_void_p(ref.data_ptr()),
                                   stream), "gls batch")
        rc = L.cuvgls_gls_noalloc(2.0, 8, ctypes.byref(inp), ctypes.c_void_p(out.data_ptr()),
                                  stream, err, len(err))
        assert rc == 0, (rc, err.value)
        torch.cuda.synchronize()
        P, Pref = out.cpu().numpy(), ref.cpu().numpy()
        assert np.all(P != -7.0)
        assert np.abs(P - Pref).max() <= TOL, np.abs(P - Pref).max()
    h.close()


def test_no_alloc_rejects_batches_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    t, yw, w, rows = _batch(5, 8, 400000)   # 8 x 3 x 819200 x 8 B > 32 MiB
    t_d = torch.from_numpy(t).cuda()
    yw_d = torch.from_numpy(yw).cuda()
    w_d = torch.from_numpy(w).cuda()
    out = torch.empty(8 * 400000, dtype=torch.float32, device="cuda")
    inp, keep = _input(_lib, rows, t_d, yw_d, w_d, out.numel())
    err = ctypes.create_string_buffer(256)
    rc = L.cuvgls_gls_noalloc(2.0, 8, ctypes.byref(inp), ctypes.c_void_p(out.data_ptr()),
                              None, err, len(err))
    assert rc == _lib.EBUDGET
    assert b"scratch" in err.value
