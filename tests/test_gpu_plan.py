"""Captured batch plans (cuvgls_gls_plan_*): a batch over fixed device buffers
replayed as one CUDA graph gives the results of the ordinary call on the
data the buffers hold at each launch."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _layout(curves, nf):
    from cuvarbase_gb300 import _lib
    cv = (_lib.RawCurve * len(curves))()
    o = 0
    for i, c in enumerate(curves):
        a = cv[i]
        a.pt_off, a.n, a.nf, a.k0, a.df, a.out_off = o, len(c[0]), nf, 1, c[3], i * nf
        o += len(c[0])
    return cv, o


def _input(cv, n_curves, npts, nout, t, y, dy, flags):
    from cuvarbase_gb300 import _lib
    inp = _lib.RawInput()
    inp.n_curves, inp.mode = n_curves, _lib.MODE_FLOATING_MEAN
    inp.curves = ctypes.cast(cv, ctypes.c_void_p)
    inp.t, inp.y, inp.dy = t, y, dy
    inp.flags = flags
    inp.n_points_total, inp.n_out_total = npts, nout
    return inp


def _data(seed, n=10):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        N = int(rng.integers(50, 600))
        T = rng.uniform(100, 1000)
        t = np.sort(rng.uniform(0, T, N))
        y = 0.3 * np.sin(2 * np.pi * t / rng.uniform(0.5, 20)) + rng.normal(0, 0.1, N)
        out.append((t, y, np.full(N, 0.1), 1.0 / (5 * T)))
    return out


def test_plan_replays_on_new_data():
    import torch
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    h = _lib.Handle(sigma=2.0, m=8)
    nf = 5000
    first = _data(1)
    second = [(t, y[::-1].copy() * 2.0 + 0.5, dy * 1.5, df) for t, y, dy, df in first]
    cv, npts = _layout(first, nf)             # same layout for both data sets
    t_d = torch.empty(npts, dtype=torch.float64, device="cuda")
    y_d = torch.empty(npts, dtype=torch.float64, device="cuda")
    dy_d = torch.empty(npts, dtype=torch.float64, device="cuda")
    out_d = torch.empty(len(first) * nf, dtype=torch.float32, device="cuda")

    def fill(curves):
        t_d.copy_(torch.from_numpy(np.concatenate([c[0] for c in curves])))
        y_d.copy_(torch.from_numpy(np.concatenate([c[1] for c in curves])))
        dy_d.copy_(torch.from_numpy(np.concatenate([c[2] for c in curves])))
        torch.cuda.synchronize()

    def direct(curves):
        P = np.empty(len(curves) * nf, np.float32)
        t = np.concatenate([c[0] for c in curves])
        y = np.concatenate([c[1] for c in curves])
        dy = np.concatenate([c[2] for c in curves])
        inp = _input(cv, len(curves), npts, len(curves) * nf, t.ctypes.data, y.ctypes.data,
                     dy.ctypes.data, _lib.HOST_INPUT | _lib.HOST_OUTPUT)
        h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(inp), P.ctypes.data, None, None, None),
                "raw")
        h.sync(None, -1)
        return P

    fill(first)
    dinp = _input(cv, len(first), npts, len(first) * nf, t_d.data_ptr(), y_d.data_ptr(),
                  dy_d.data_ptr(), 0)
    plan = ctypes.c_void_p()
    h.check(L.cuvgls_gls_plan_create(h.ptr, ctypes.byref(dinp), ctypes.c_void_p(out_d.data_ptr()),
                                     None, None, ctypes.byref(plan)), "plan create")
    try:
        for curves in (first, second, first):
            fill(curves)
            out_d.zero_()
            assert L.cuvgls_gls_plan_launch(plan, None) == 0
            torch.cuda.synchronize()
            got = out_d.cpu().numpy()
            assert np.abs(got - direct(curves)).max() <= 1e-5
    finally:
        L.cuvgls_gls_plan_destroy(plan)
        h.close()


def test_plan_best_frequencies_and_host_flags_rejected():
    import torch
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    h = _lib.Handle(sigma=2.0, m=8)
    nf = 4000
    curves = _data(2)
    cv, npts = _layout(curves, nf)
    t_d = torch.from_numpy(np.concatenate([c[0] for c in curves])).cuda()
    y_d = torch.from_numpy(np.concatenate([c[1] for c in curves])).cuda()
    dy_d = torch.from_numpy(np.concatenate([c[2] for c in curves])).cuda()
    bk_d = torch.empty(len(curves), dtype=torch.int64, device="cuda")
    bp_d = torch.empty(len(curves), dtype=torch.float32, device="cuda")
    P_d = torch.empty(len(curves) * nf, dtype=torch.float32, device="cuda")
    dinp = _input(cv, len(curves), npts, len(curves) * nf, t_d.data_ptr(), y_d.data_ptr(),
                  dy_d.data_ptr(), 0)
    try:
        h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(dinp), ctypes.c_void_p(P_d.data_ptr()),
                                 None, None, None), "raw")
        h.sync(None, -1)
        P = P_d.cpu().numpy().reshape(len(curves), nf)
        plan = ctypes.c_void_p()
        h.check(L.cuvgls_gls_plan_create(h.ptr, ctypes.byref(dinp), None,
                                         ctypes.c_void_p(bk_d.data_ptr()),
                                         ctypes.c_void_p(bp_d.data_ptr()), ctypes.byref(plan)),
                "plan create")
        bk_d.fill_(-7)
        assert L.cuvgls_gls_plan_launch(plan, None) == 0
        torch.cuda.synchronize()
        L.cuvgls_gls_plan_destroy(plan)
        bk = bk_d.cpu().numpy()
        bp = bp_d.cpu().numpy()
        for i in range(len(curves)):
            j = int(np.argmax(P[i]))
            assert P[i][bk[i]] >= P[i][j] - 1e-6
            assert abs(float(bp[i]) - float(P[i][j])) <= 1e-6
        hinp = _input(cv, len(curves), npts, len(curves) * nf, t_d.data_ptr(), y_d.data_ptr(),
                      dy_d.data_ptr(), _lib.HOST_INPUT)
        bad = ctypes.c_void_p()
        rc = L.cuvgls_gls_plan_create(h.ptr, ctypes.byref(hinp), ctypes.c_void_p(P_d.data_ptr()),
                                      None, None, ctypes.byref(bad))
        assert rc == _lib.EINVAL and not bad.value
    finally:
        h.close()
