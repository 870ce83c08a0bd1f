"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Run in a container that has the cuvarbase source tree (read-only), with
REFERENCE_ROOT naming its root (the directory that holds `cuvarbase/`):

    REFERENCE_ROOT=<path to the cuvarbase tree> python tests/golden/make_golden.py

The reference's CPU functions are importable once empty stub modules stand in
for pycuda / scikit-cuda (GPU-only imports) and for nfft / astropy (test-only
imports).  Nothing here calls GPU code.  The script records the reference's
outputs of

  * cuvarbase/lombscargle.py:539-576  lomb_scargle_direct_sums (H=1 and H=2,
    with and without amplitude prior; H=3 with per-harmonic priors and prior
    centres cn0 / sn0),
  * cuvarbase/lombscargle.py:1115-1184 fap_baluev,
  * cuvarbase/utils.py:10-13 weights, :46-97 autofrequency,
    :113-146 normalize_light_curves,
  * cuvarbase/tests/test_nfft.py:31-87 direct_sums, precomp_psi,
    gpu_grid_scalar on the reference test data (test_nfft.py:41-54),

on the reference tests' own data generators and on seeded synthetic curves of
the benchmark shapes.  The fixtures are plain npz files; the GPU machine never
needs the reference tree.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

REF = os.environ.get("REFERENCE_ROOT", "")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")


def _stub_imports():
    names = ["pycuda", "pycuda.driver", "pycuda.gpuarray", "pycuda.compiler",
             "pycuda.autoprimaryctx", "pycuda.tools", "skcuda", "skcuda.fft",
             "nfft", "nfft.utils", "nfft.kernels", "astropy",
             "astropy.timeseries"]
    for n in names:
        sys.modules.setdefault(n, types.ModuleType(n))
    sys.modules["pycuda.compiler"].SourceModule = object
    sys.modules["pycuda.tools"].mark_cuda_test = lambda f: f
    sys.modules["nfft"].nfft_adjoint = None
    sys.modules["nfft.utils"].nfft_matrix = None
    sys.modules["nfft.kernels"].KERNELS = {}
    sys.modules["astropy.timeseries"].LombScargle = None
    sys.path.insert(0, REF)


def cfg1_curve(seed=1001, N=1000, T=3650.0):
    """N times uniform over T days with the half-year seasonal gap, sorted;
    y = 0.1 sin(2 pi t / 0.73 + phi) + N(0, 0.05^2); dy = 0.05."""
    rng = np.random.default_rng(seed)
    t = []
    while len(t) < N:
        c = rng.uniform(0, T, 4 * N)
        t.extend(c[(c / 365.25) % 1.0 >= 0.5].tolist())
    t = np.sort(np.array(t[:N]))
    y = 0.1 * np.sin(2 * np.pi * t / 0.73 + rng.uniform(0, 2 * np.pi))
    y = y + rng.normal(0, 0.05, N)
    return t, y, 0.05 * np.ones(N)


def cfg2_curve(rng):
    N = int(round(np.exp(rng.uniform(np.log(50), np.log(5000)))))
    T = rng.uniform(100, 3650)
    t = np.sort(rng.uniform(0, T, N))
    P = np.exp(rng.uniform(np.log(0.1), np.log(100)))
    A = rng.uniform(0.05, 0.5)
    sn = rng.uniform(0.02, 0.2)
    dy = np.exp(rng.normal(np.log(0.05), 0.3, N))
    y = A * np.sin(2 * np.pi * t / P + rng.uniform(0, 2 * np.pi))
    y = y + rng.normal(0, sn, N)
    return t, y, dy


def setdata(t, y, dy):
    """LombScargleMemory.setdata (lombscargle.py:235-261) without the GPU
    container: FP64 weights / mean / YY, then float32 casts."""
    from cuvarbase.utils import weights
    w = weights(dy)
    ybar = np.dot(y, w)
    yw = np.multiply(w, y - ybar)
    yy = np.dot(w, np.power(y - ybar, 2))
    return (np.asarray(t).astype(np.float32), yw.astype(np.float32),
            w.astype(np.float32), float(yy), float(ybar))


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "cuvarbase")):
        sys.exit("set REFERENCE_ROOT to the root of the cuvarbase source tree")
    _stub_imports()
    import cuvarbase.lombscargle as ls
    import cuvarbase.utils as ut
    import cuvarbase.tests.test_nfft as tn
    import cuvarbase.tests.test_lombscargle as tl

    g = {}

    # --- LS on the reference tests' own data (test_lombscargle.py:24-35) ---
    t, y, err = tl.data()                   # RandomState(100), N=100, freq=3
    g["ls_t_raw"], g["ls_y_raw"], g["ls_dy_raw"] = t, y, err
    (tn_, yn_, dyn_), = ut.normalize_light_curves([(t, y, err)])
    g["ls_t_norm"], g["ls_y_norm"] = tn_, yn_
    freqs = ut.autofrequency(tn_, nyquist_factor=3, samples_per_peak=3)
    g["ls_freqs"] = freqs
    t32, yw, w, yy, ybar = setdata(tn_, yn_, dyn_)
    g["ls_t32"], g["ls_yw"], g["ls_w"] = t32, yw, w
    g["ls_yy"], g["ls_ybar"] = yy, ybar
    g["ls_P"] = ls.lomb_scargle_direct_sums(t32, yw, w, freqs, yy)
    g["ls_P_prior"] = ls.lomb_scargle_direct_sums(t32, yw, w, freqs, yy,
                                                  amplitude_priors=0.5)
    g["ls_P_h2"] = ls.lomb_scargle_direct_sums(t32, yw, w, freqs, yy,
                                               nharms=2)
    g["ls_P_h3_prior"] = ls.lomb_scargle_direct_sums(
        t32, yw, w, freqs, yy, nharms=3, amplitude_priors=np.array([0.5, 0.8, 1.5]),
        cn0=np.array([0.01, -0.02, 0.0]), sn0=np.array([0.0, 0.015, -0.01]))
    g["ls_weights"] = ut.weights(err)

    # --- autofrequency variants (utils.py:46-97) ---
    g["af_default"] = ut.autofrequency(tn_)
    g["af_minmax"] = ut.autofrequency(tn_, minimum_frequency=2.0,
                                      maximum_frequency=40.0,
                                      samples_per_peak=5)
    g["af_spp1"] = ut.autofrequency(tn_, samples_per_peak=1,
                                    nyquist_factor=2)

    # --- fap_baluev (lombscargle.py:1115-1184) ---
    z = np.linspace(0.01, 0.6, 25)
    g["fap_z"] = z
    g["fap"] = ls.fap_baluev(t, err, z, float(freqs.max()))

    # --- benchmark-shaped curves on a frequency subsample ---
    t, y, dy = cfg1_curve()
    (tn_, yn_, dyn_), = ut.normalize_light_curves([(t, y, dy)])
    t32, yw, w, yy, ybar = setdata(tn_, yn_, dyn_)
    df = 1.0 / (5 * 3650.0)
    kk = np.unique(np.concatenate([np.arange(0, 300), np.arange(24800, 25200),
                                   np.arange(49700, 50000)]))
    g["c1_t"], g["c1_y"], g["c1_dy"] = t, y, dy
    g["c1_df"], g["c1_k"] = df, kk
    g["c1_P"] = ls.lomb_scargle_direct_sums(t32, yw, w, df * (1 + kk), yy)

    rng = np.random.default_rng(1002)
    for i in range(3):
        t, y, dy = cfg2_curve(rng)
        (tn_, yn_, dyn_), = ut.normalize_light_curves([(t, y, dy)])
        t32, yw, w, yy, ybar = setdata(tn_, yn_, dyn_)
        dfc = 1.0 / (5 * (tn_.max() - tn_.min()))
        kk = np.unique(np.concatenate([np.arange(0, 100),
                                       rng.integers(0, 100000, 200)]))
        g[f"c2_{i}_t"], g[f"c2_{i}_y"], g[f"c2_{i}_dy"] = t, y, dy
        g[f"c2_{i}_df"], g[f"c2_{i}_k"] = dfc, kk
        g[f"c2_{i}_P"] = ls.lomb_scargle_direct_sums(t32, yw, w,
                                                     dfc * (1 + kk), yy)

    # --- NFFT pins from the reference tests (test_nfft.py:31-87) ---
    t, tsc, y, err = tn.data()              # RandomState(100), N=100
    g["nf_t"], g["nf_tsc"], g["nf_y"] = t, tsc, y
    nf = int(tn.nfft_sigma * len(t))        # 500
    g["nf_grid"] = tn.gpu_grid_scalar(tsc, y, tn.nfft_sigma, tn.nfft_m, nf)
    g["nf_sigma"], g["nf_m"], g["nf_nf"] = tn.nfft_sigma, tn.nfft_m, nf
    k0 = int(-0.5 * nf)
    g["nf_k0"] = k0
    g["nf_dft_scaled"] = tn.direct_sums(tsc, y, float(k0) + np.arange(nf))
    dfu = 1.0 / (t.max() - t.min())
    g["nf_dft_unscaled"] = tn.direct_sums(t, y, (k0 + np.arange(nf)) * dfu)

    np.savez_compressed(OUT, **{k: np.asarray(v) for k, v in g.items()})
    print("wrote", OUT, sum(np.asarray(v).nbytes for v in g.values()), "bytes")


if __name__ == "__main__":
    main()
