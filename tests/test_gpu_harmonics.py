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
