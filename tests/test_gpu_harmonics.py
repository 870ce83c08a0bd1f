"""Multi-harmonic floating-mean GLS by FP64 direct sums on the GPU
(lomb_scargle_direct_sums with nharms, cuvarbase/lombscargle.py:337-576)
against the reference's own outputs and the FP64 restatement."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_reference_vectors(golden):
    from cuvarbase_gb300.lombscargle import lomb_scargle_direct_sums
    g = golden
    args = (g["ls_t32"], g["ls_yw"], g["ls_w"], g["ls_freqs"], float(g["ls_yy"]))
    np.testing.assert_allclose(lomb_scargle_direct_sums(*args), g["ls_P"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(lomb_scargle_direct_sums(*args, amplitude_priors=0.5),
                               g["ls_P_prior"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(lomb_scargle_direct_sums(*args, nharms=2), g["ls_P_h2"],
                               rtol=0, atol=1e-10)
    P3 = lomb_scargle_direct_sums(*args, nharms=3, amplitude_priors=np.array([0.5, 0.8, 1.5]),
                                  cn0=np.array([0.01, -0.02, 0.0]),
                                  sn0=np.array([0.0, 0.015, -0.01]))
    np.testing.assert_allclose(P3, g["ls_P_h3_prior"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("H", [1, 4, 6, 8])
def test_against_restatement_nonuniform_freqs(oracle, H):
    from cuvarbase_gb300.lombscargle import lomb_scargle_direct_sums
    rng = np.random.default_rng(50 + H)
    N = 700
    t = np.sort(rng.uniform(0, 2000, N))
    y = 0.2 * np.sign(np.sin(2 * np.pi * t / 3.3)) + rng.normal(0, 0.05, N)   # square wave
    dy = np.full(N, 0.05)
    tt, yw, w, YY, _ = oracle.prepare_curve(t, y, dy)
    freqs = np.sort(rng.uniform(0.01, 2.0, 300))          # any values, not a grid
    freqs[0] = 1 / 3.3
    P = lomb_scargle_direct_sums(tt, yw, w, freqs, YY, nharms=H, amplitude_priors=3.0)
    ref = oracle.mhgls_np(tt, yw, w, freqs, YY, nharms=H, amplitude_priors=3.0)
    assert np.abs(P - ref).max() <= 1e-9


def test_argument_checks():
    from cuvarbase_gb300.lombscargle import lomb_scargle_direct_sums
    t = np.linspace(0, 10, 20)
    w = np.full(20, 0.05)
    yw = w * np.sin(t)
    with pytest.raises(ValueError):
        lomb_scargle_direct_sums(t, yw, w, [0.1, 0.2], 1.0, nharms=9)
    with pytest.raises(ValueError):
        lomb_scargle_direct_sums(t, yw, w, [0.1, 0.2], 1.0, nharms=2,
                                 amplitude_priors=np.array([1.0, 2.0, 3.0]))


def test_entry_point_argument_errors():
    """The FP64 entry points reject bad sizes and pointers before any launch."""
    import ctypes
    from cuvarbase_gb300 import _lib
    L = _lib.load()
    h = _lib.Handle(sigma=2.0, m=8)
    try:
        t = np.linspace(0, 1, 10)
        fr = np.linspace(0.1, 1, 5)
        out = np.empty(5)
        flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
        for H in (0, 9):
            assert L.cuvgls_mhgls_direct(h.ptr, H, t.ctypes.data, t.ctypes.data, t.ctypes.data,
                                         10, fr.ctypes.data, 5, 1.0, 0.0, None, None, None,
                                         flags, out.ctypes.data, None) == _lib.EINVAL
        assert L.cuvgls_mhgls_direct(h.ptr, 1, None, t.ctypes.data, t.ctypes.data, 10,
                                     fr.ctypes.data, 5, 1.0, 0.0, None, None, None, flags,
                                     out.ctypes.data, None) == _lib.EINVAL
        c = (_lib.GridFinCurve * 1)()
        c[0].grid_off, c[0].ng, c[0].nf, c[0].out_off = 0, 20, 5, 0
        c[0].tmin, c[0].tmax, c[0].spp, c[0].f0, c[0].b = 1.0, 1.0, 1.0, 0.0, 1.0  # tmax == tmin
        g = np.zeros(40)
        assert L.cuvgls_nfft_from_grid(h.ptr, 1, ctypes.cast(c, ctypes.c_void_p), g.ctypes.data,
                                       20, 5, flags, out.ctypes.data, None) == _lib.EINVAL
        c[0].tmax = 2.0
        c[0].ng = 30                                        # beyond the 20 cells given
        assert L.cuvgls_nfft_from_grid(h.ptr, 1, ctypes.cast(c, ctypes.c_void_p), g.ctypes.data,
                                       20, 5, flags, out.ctypes.data, None) == _lib.EINVAL
        nc = (_lib.NfftCurve * 1)()
        nc[0].pt_off, nc[0].n, nc[0].nf, nc[0].f0, nc[0].df, nc[0].out_off = 0, 10, 5, 0.0, 0.0, 0
        inp = _lib.NfftInput()
        inp.n_curves, inp.flags = 1, flags
        inp.curves = ctypes.cast(nc, ctypes.c_void_p)
        inp.t, inp.n_points_total, inp.n_out_total = t.ctypes.data, 10, 5
        assert L.cuvgls_nfft_adjoint_fp64(h.ptr, ctypes.byref(inp), t.ctypes.data,
                                          out.ctypes.data, None) == _lib.EINVAL   # df = 0
    finally:
        h.close()
