"""The FP64 oracle against the reference's own outputs (golden fixtures made
by tests/golden/make_golden.py from cuvarbase's CPU functions)."""
import numpy as np
import pytest


def test_gls_flmean_matches_reference(golden, oracle):
    g = golden
    P = oracle.gls_flmean(g["ls_t32"], g["ls_yw"], g["ls_w"], g["ls_freqs"], float(g["ls_yy"]))
    np.testing.assert_allclose(P, g["ls_P"], rtol=0, atol=1e-12)


def test_gls_flmean_numpy_matches_reference(golden, oracle):
    g = golden
    P = oracle.gls_flmean_np(g["ls_t32"], g["ls_yw"], g["ls_w"], g["ls_freqs"], float(g["ls_yy"]))
    np.testing.assert_allclose(P, g["ls_P"], rtol=0, atol=1e-12)


def test_gls_amplitude_prior_matches_reference(golden, oracle):
    g = golden
    P = oracle.gls_flmean(g["ls_t32"], g["ls_yw"], g["ls_w"], g["ls_freqs"], float(g["ls_yy"]),
                          amplitude_prior=0.5)
    np.testing.assert_allclose(P, g["ls_P_prior"], rtol=0, atol=1e-12)


def test_multi_harmonic_matches_reference(golden, oracle):
    """mhdirect_sums -> add_regularization -> mhgls_from_sums restated: H=1
    with a prior, H=2, and H=3 with per-harmonic priors and centres."""
    g = golden
    args = (g["ls_t32"], g["ls_yw"], g["ls_w"], g["ls_freqs"], float(g["ls_yy"]))
    np.testing.assert_allclose(oracle.mhgls_np(*args, nharms=1, amplitude_priors=0.5),
                               g["ls_P_prior"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(oracle.mhgls_np(*args, nharms=2), g["ls_P_h2"],
                               rtol=0, atol=1e-12)
    P3 = oracle.mhgls_np(*args, nharms=3, amplitude_priors=np.array([0.5, 0.8, 1.5]),
                         cn0=np.array([0.01, -0.02, 0.0]), sn0=np.array([0.0, 0.015, -0.01]))
    np.testing.assert_allclose(P3, g["ls_P_h3_prior"], rtol=0, atol=1e-12)


def test_tau_form_equals_solve_form(golden, oracle):
    """lomb.cu's rotated closed form and mhgls_from_sums agree in FP64
    (up to the float32 sum(yw) term the direct sums subtract)."""
    g = golden
    P = oracle.gls_tau(g["ls_t32"], g["ls_yw"], g["ls_w"], g["ls_freqs"], float(g["ls_yy"]),
                       float(g["ls_ybar"]), mode=1)
    np.testing.assert_allclose(P, g["ls_P"], rtol=0, atol=1e-7)
    Pr = oracle.gls_tau(g["ls_t32"], g["ls_yw"], g["ls_w"], g["ls_freqs"], float(g["ls_yy"]),
                        float(g["ls_ybar"]), mode=1, reg=[4.0, 4.0, 0.0])
    np.testing.assert_allclose(Pr, g["ls_P_prior"], rtol=0, atol=1e-7)


def test_benchmark_shaped_curves_match_reference(golden, oracle):
    g = golden
    t, yw, w, YY, ybar = oracle.prepare_curve(g["c1_t"], g["c1_y"], g["c1_dy"])
    P = oracle.gls_flmean(t.astype(np.float32), yw, w, g["c1_df"] * (1 + g["c1_k"]), YY)
    np.testing.assert_allclose(P, g["c1_P"], rtol=0, atol=1e-12)
    for i in range(3):
        t, yw, w, YY, ybar = oracle.prepare_curve(g[f"c2_{i}_t"], g[f"c2_{i}_y"], g[f"c2_{i}_dy"])
        P = oracle.gls_flmean(t.astype(np.float32), yw, w,
                              g[f"c2_{i}_df"] * (1 + g[f"c2_{i}_k"]), YY)
        np.testing.assert_allclose(P, g[f"c2_{i}_P"], rtol=0, atol=1e-12)


def test_prepare_curve_matches_reference_normalisation(golden, oracle):
    g = golden
    t, yw, w, YY, ybar = oracle.prepare_curve(g["ls_t_raw"], g["ls_y_raw"], g["ls_dy_raw"])
    np.testing.assert_array_equal(t, g["ls_t_norm"])
    np.testing.assert_array_equal(yw, g["ls_yw"])
    np.testing.assert_array_equal(w, g["ls_w"])
    assert YY == pytest.approx(float(g["ls_yy"]), rel=1e-15)


def test_grid_matches_reference_scalar_gridding(golden, oracle):
    g = golden
    ng = int(g["nf_sigma"]) * int(g["nf_nf"])
    for fn in (oracle.grid_ref, oracle.grid_ref_np):
        grid = fn(g["nf_tsc"], g["nf_y"], ng, int(g["nf_m"]), float(g["nf_sigma"]))
        np.testing.assert_allclose(grid, g["nf_grid"], rtol=0, atol=1e-12)


def test_nfft_direct_matches_reference(golden, oracle):
    g = golden
    k0, nf = int(g["nf_k0"]), int(g["nf_nf"])
    d = oracle.nfft_direct(g["nf_tsc"], g["nf_y"], k0 + np.arange(nf))
    np.testing.assert_allclose(d, g["nf_dft_scaled"], rtol=0, atol=1e-10)
    t = g["nf_t"]
    d = oracle.nfft_direct(t, g["nf_y"], (k0 + np.arange(nf)) / (t.max() - t.min()))
    np.testing.assert_allclose(d, g["nf_dft_unscaled"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(oracle.nfft_direct_np(t, g["nf_y"], (k0 + np.arange(nf)) /
                                                     (t.max() - t.min())),
                               g["nf_dft_unscaled"], rtol=0, atol=1e-10)


def test_oracle_mode0_and_window_against_numpy():
    """Standard LS (mode 0) and the window mode restated independently."""
    from oracle import oracle as O
    rng = np.random.default_rng(7)
    t = np.sort(rng.uniform(0, 50, 80))
    y = np.sin(2 * np.pi * t / 3.1) + 0.2 * rng.normal(size=80) + 0.3
    dy = 0.2 + 0.05 * rng.uniform(size=80)
    tt, yw, w, YY, ybar = O.prepare_curve(t, y, dy)
    f = (1 + np.arange(300)) / (5 * 50.0)
    ph = 2 * np.pi * np.outer(f, tt)
    C, S = np.cos(ph) @ w.astype(float), np.sin(ph) @ w.astype(float)
    C2, S2 = np.cos(2 * ph) @ w.astype(float), np.sin(2 * ph) @ w.astype(float)
    YC = np.cos(ph) @ yw.astype(float) + ybar * C
    YS = np.sin(ph) @ yw.astype(float) + ybar * S
    CC, SS, CS = 0.5 * (1 + C2), 0.5 * (1 - C2), 0.5 * S2
    det = CC * SS - CS * CS
    P0 = (YC ** 2 * SS - 2 * YC * YS * CS + YS ** 2 * CC) / det / (YY + ybar ** 2)
    np.testing.assert_allclose(O.gls_tau(tt, yw, w, f, YY, ybar, mode=0), P0, rtol=1e-9, atol=1e-12)
    YC, YS = 2 * C, 2 * S
    P2 = (YC ** 2 * SS - 2 * YC * YS * CS + YS ** 2 * CC) / det
    np.testing.assert_allclose(O.gls_tau(tt, yw, w, f, YY, ybar, mode=2), P2, rtol=1e-9, atol=1e-12)


def test_block_oracle_equals_direct_sums(oracle):
    """The phasor-recurrence block form of the oracle (for N ~ 1e6 curves)
    against the one-sin/cos-per-term direct sums, across re-seed points."""
    rng = np.random.default_rng(3)
    N, T = 3001, 3650.0
    t = np.sort(rng.uniform(0, T, N))
    y = 0.1 * np.sin(2 * np.pi * 7.3 * t) + rng.normal(0, 0.1, N)
    tt, yw, w, YY, _ = oracle.prepare_curve(t, y, np.full(N, 0.1))
    df = 1.0 / (5 * T)
    f_start = np.array([1.0, 7.3 - 50 * df, 999.0])
    blk = 150  # crosses the 64-bin re-seed twice
    P = oracle.gls_flmean_blocks(tt, yw, w, f_start, df, blk, YY)
    freqs = (f_start[:, None] + df * np.arange(blk)[None, :]).ravel()
    ref = oracle.gls_flmean(tt, yw, w, freqs, YY).reshape(3, blk)
    assert np.abs(P - ref).max() <= 1e-9
