"""Host input in phases: with several FFT chunks (a small chunk_mb here) each
chunk's points are copied, prepared and binned just before its passes, or,
when the chunks' point ranges are not disjoint and in order, the first
chunk's range is copied first and the rest after.  Every layout must give the
powers of the same curves run one per call (one chunk, one phase) within
1e-5: points in input order, points stored in reverse curve order, two plan
classes interleaved, raw and prepared input, best-frequency output."""
import ctypes

import numpy as np
import pytest

from test_gpu_raw import _prepared, _raw

pytestmark = pytest.mark.gpu


def _curves(seed, n, nfs):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        N = int(round(np.exp(rng.uniform(np.log(50), np.log(3000)))))
        T = rng.uniform(100, 3650)
        t = np.sort(rng.uniform(0, T, N)) + rng.uniform(-500, 500)
        y = 1.0 + 0.3 * np.sin(2 * np.pi * t / rng.uniform(0.2, 50)) + rng.normal(0, 0.1, N)
        dy = np.exp(rng.normal(np.log(0.05), 0.3, N))
        out.append((t, y, dy, 1.0 / (5 * T), nfs[i % len(nfs)]))
    return out


def _handle(chunk_mb=0):
    from cuvarbase_gb300 import _lib
    return _lib.Handle(sigma=-1.0, m=8, chunk_mb=chunk_mb)


@pytest.fixture(scope="module")
def hs():
    h = _handle(16)     # 16 MiB of intermediate: a few curves per chunk
    yield h
    h.close()


@pytest.fixture(scope="module")
def h1():
    h = _handle()
    yield h
    h.close()


def _raw_placed(h, curves, place, best=False):
    """cuvgls_gls_raw with host input and output, curve i's points stored as
    block place[i] of the concatenated arrays (descriptors in curve order)."""
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    n = [len(c[0]) for c in curves]
    blocks = sorted(range(len(curves)), key=lambda i: place[i])
    off = {}
    o = 0
    for i in blocks:
        off[i] = o
        o += n[i]
    t = np.empty(o); y = np.empty(o); dy = np.empty(o)
    for i, c in enumerate(curves):
        t[off[i]:off[i] + n[i]], y[off[i]:off[i] + n[i]], dy[off[i]:off[i] + n[i]] = c[:3]
    cv = (_lib.RawCurve * len(curves))()
    oo = 0
    outs = []
    for i, c in enumerate(curves):
        a = cv[i]
        a.pt_off, a.n, a.nf, a.k0, a.df, a.out_off = off[i], n[i], c[4], 1, c[3], oo
        outs.append((oo, c[4]))
        oo += c[4]
    inp = _lib.RawInput()
    inp.n_curves, inp.mode = len(curves), 1
    inp.curves = ctypes.cast(cv, ctypes.c_void_p)
    inp.t, inp.y, inp.dy = t.ctypes.data, y.ctypes.data, dy.ctypes.data
    inp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
    inp.n_points_total, inp.n_out_total = o, oo
    if best:
        bk = np.empty(len(curves), np.int64)
        bp = np.empty(len(curves), np.float32)
        h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(inp), None, bk.ctypes.data,
                                 bp.ctypes.data, None), "raw best")
        h.sync(None, -1)
        return bk, bp
    P = np.empty(oo, np.float32)
    h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(inp), P.ctypes.data, None, None, None), "raw")
    h.sync(None, -1)
    return [P[a:a + k] for a, k in outs]


def _one_per_call(h, curves):
    return [_raw_placed(h, [c], [0])[0] for c in curves]


@pytest.mark.parametrize("layout", ["in_order", "reversed"])
def test_phases_raw_input_match_one_per_call(hs, h1, layout):
    curves = _curves(61, 22, [100_000])
    place = list(range(len(curves)))
    if layout == "reversed":      # chunk point ranges out of order: two-phase fallback
        place = place[::-1]
    P = _raw_placed(hs, curves, place)
    ref = _one_per_call(h1, curves)
    for a, b in zip(P, ref):
        assert np.abs(a - b).max() <= 1e-5


def test_phases_two_classes_interleaved(hs, h1):
    # two frequency counts alternate: the classes are reordered into two
    # groups, so chunk point ranges interleave and the fallback splits
    curves = _curves(62, 20, [100_000, 20_000])
    P = _raw_placed(hs, curves, list(range(len(curves))))
    ref = _one_per_call(h1, curves)
    for a, b in zip(P, ref):
        assert np.abs(a - b).max() <= 1e-5


def test_phases_prepared_input_and_best(hs, h1):
    curves = [c[:4] for c in _curves(63, 22, [100_000])]
    P = _prepared(hs, curves, 100_000)
    ref = np.stack([_prepared(h1, [c], 100_000)[0] for c in curves])
    assert np.abs(P - ref).max() <= 1e-5
    bk, bp = _raw(hs, curves, 100_000, best=True)
    for i in range(len(curves)):
        j = int(np.argmax(ref[i]))
        assert ref[i][bk[i]] >= ref[i][j] - 1e-5
        assert abs(float(bp[i]) - float(ref[i][j])) <= 1e-5
