"""FP64 CPU oracle for the GLS / adjoint-NFFT path (TEST INFRASTRUCTURE ONLY).

This module is the checker the CUDA path is compared with.  The product
package (``cuvarbase_gb300``) never imports it; only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (CPU baseline and reference arm)
do.

Two layers:

* ``liboracle.so`` (``gls_oracle.c``, built by ``oracle/Makefile``): FP64
  OpenMP direct sums restating cuvarbase/lombscargle.py:337-576 and
  cuvarbase/kernels/lomb.cu:36-165, used for anything larger than a toy.
* small pure-numpy restatements (``*_np``) of the same reference functions,
  used to cross-check the C code and for tiny cases.

Host-side preparation (``prepare_curve``) restates what the reference does on
the host before any kernel runs: cuvarbase/utils.py:113-146
(normalize_light_curves), :10-13 (weights) and
cuvarbase/lombscargle.py:235-261 (LombScargleMemory.setdata).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (when stale)."""
    src = os.path.join(_HERE, "gls_oracle.c")
    if (force or not os.path.exists(_LIB_PATH)
            or os.path.getmtime(src) > os.path.getmtime(_LIB_PATH)):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        i64 = ctypes.c_int64
        L.oracle_gls_flmean.argtypes = [_dp, _dp, _dp, i64, _dp, i64,
                                        ctypes.c_double, ctypes.c_double, _dp,
                                        ctypes.c_int]
        L.oracle_gls_tau.argtypes = [_dp, _dp, _dp, i64, _dp, i64,
                                     ctypes.c_double, ctypes.c_double, _dp,
                                     ctypes.c_int, _dp, ctypes.c_int]
        L.oracle_gls_flmean_blocks.argtypes = [_dp, _dp, _dp, i64, _dp, i64,
                                               ctypes.c_double, i64, ctypes.c_double,
                                               _dp, ctypes.c_int]
        L.oracle_nfft_direct.argtypes = [_dp, _dp, i64, _dp, i64, _dp,
                                         ctypes.c_int]
        L.oracle_grid_ref.argtypes = [_dp, _dp, i64, i64, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, _dp]
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _c(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def max_threads() -> int:
    return int(lib().oracle_max_threads())


# ----------------------------------------------------------------------------
# host-side preparation (what the reference does before the GPU)
# ----------------------------------------------------------------------------
def prepare_curve(t, y, dy, normalize=True):
    """Return (t, yw, w, YY, ybar) as the reference computes them.

    normalize_light_curves subtracts the unweighted nanmean of t and y
    (utils.py:113-146); setdata computes w = dy^-2 / sum(dy^-2), the weighted
    mean ybar, yw = w (y - ybar) and YY = sum w (y - ybar)^2 in FP64 and then
    casts t, yw, w to float32 (lombscargle.py:246-261).  t is returned in FP64
    and as the float32 the reference would use.
    """
    t = np.asarray(t, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    dy = np.asarray(dy, dtype=np.float64)
    if normalize:
        t = t - np.nanmean(t)
        y = y - np.nanmean(y)
    w = np.power(dy, -2)
    w = w / sum(w)
    ybar = np.dot(y, w)
    yw = np.multiply(w, y - ybar)
    YY = np.dot(w, np.power(y - ybar, 2))
    return t, yw.astype(np.float32), w.astype(np.float32), float(YY), float(ybar)


# ----------------------------------------------------------------------------
# C oracle wrappers
# ----------------------------------------------------------------------------
def gls_flmean(t, yw, w, freqs, YY, amplitude_prior=None, nthreads=0):
    """FP64 floating-mean GLS (lomb_scargle_direct_sums, H=1)."""
    t, tp = _c(t); yw, ywp = _c(yw); w, wp = _c(w); f, fp = _c(freqs)
    P = np.empty(len(f))
    lib().oracle_gls_flmean(tp, ywp, wp, len(t), fp, len(f), float(YY),
                            float(amplitude_prior or 0.0),
                            P.ctypes.data_as(_dp), int(nthreads))
    return P


def gls_flmean_blocks(t, yw, w, f_start, df, block_len, YY, nthreads=0):
    """FP64 floating-mean GLS on blocks of contiguous bins f_start[b] + k df
    (phasor recurrence, re-seeded every 64 bins); returns (nblocks, block_len)."""
    t, tp = _c(t); yw, ywp = _c(yw); w, wp = _c(w); f0, f0p = _c(f_start)
    P = np.empty(len(f0) * int(block_len))
    lib().oracle_gls_flmean_blocks(tp, ywp, wp, len(t), f0p, len(f0), float(df),
                                   int(block_len), float(YY), P.ctypes.data_as(_dp),
                                   int(nthreads))
    return P.reshape(len(f0), int(block_len))


def gls_tau(t, yw, w, freqs, YY, ybar, mode=1, reg=None, nthreads=0):
    """FP64 closed-form GLS of lomb.cu (mode 0 standard, 1 floating mean, 2 window)."""
    t, tp = _c(t); yw, ywp = _c(yw); w, wp = _c(w); f, fp = _c(freqs)
    P = np.empty(len(f))
    if reg is None:
        regp = None
    else:
        reg, regp = _c(reg)
    lib().oracle_gls_tau(tp, ywp, wp, len(t), fp, len(f), float(YY),
                         float(ybar), regp, int(mode),
                         P.ctypes.data_as(_dp), int(nthreads))
    return P


def nfft_direct(t, y, freqs, nthreads=0):
    """sum_j y_j exp(+2 pi i f t_j) in FP64 (tests/test_nfft.py:31-34)."""
    t, tp = _c(t); y, yp = _c(y); f, fp = _c(freqs)
    out = np.empty(2 * len(f))
    lib().oracle_nfft_direct(tp, yp, len(t), fp, len(f),
                             out.ctypes.data_as(_dp), int(nthreads))
    return out[0::2] + 1j * out[1::2]


def grid_ref(t, y, ng, m, sigma, spp=1.0, tmin=None, tmax=None):
    """Reference-convention real Gaussian grid (cunfft.cu:84-163)."""
    t, tp = _c(t); y, yp = _c(y)
    tmin = float(np.min(t)) if tmin is None else float(tmin)
    tmax = float(np.max(t)) if tmax is None else float(tmax)
    g = np.empty(int(ng))
    lib().oracle_grid_ref(tp, yp, len(t), int(ng), int(m), float(sigma), tmin,
                          tmax, float(spp), g.ctypes.data_as(_dp))
    return g


# ----------------------------------------------------------------------------
# pure-numpy restatements (small cases; cross-check of the C code)
# ----------------------------------------------------------------------------
def gls_flmean_np(t, yw, w, freqs, YY, amplitude_prior=None):
    """Vectorised restatement of lomb_scargle_direct_sums (H=1)."""
    t = np.asarray(t, np.float64); yw = np.asarray(yw, np.float64)
    w = np.asarray(w, np.float64); freqs = np.asarray(freqs, np.float64)
    ph = 2 * np.pi * (np.outer(freqs, t) % 1.0)
    c, s = np.cos(ph), np.sin(ph)
    c2, s2 = np.cos(2 * ph), np.sin(2 * ph)
    W = w.sum()
    C, S, C2, S2 = c @ w, s @ w, c2 @ w, s2 @ w
    ybar = float(np.cumsum(yw.astype(np.float32), dtype=np.float32)[-1])
    YC = c @ yw - ybar * C
    YS = s @ yw - ybar * S
    D = 0.0 if amplitude_prior is None else amplitude_prior ** -2
    CC = 0.5 * (C2 + W) - C * C + D
    SS = 0.5 * (W - C2) - S * S + D
    CS = 0.5 * S2 - C * S
    det = CC * SS - CS * CS
    cn = (SS * YC - CS * YS) / det
    sn = (CC * YS - CS * YC) / det
    XX = cn * cn * CC + 2 * cn * sn * CS + sn * sn * SS
    return (2 * (cn * YC + sn * YS) - XX) / YY


def nfft_direct_np(t, y, freqs):
    t = np.asarray(t, np.float64); y = np.asarray(y, np.float64)
    ph = 2 * np.pi * (np.outer(freqs, t) % 1.0)
    return np.cos(ph) @ y + 1j * (np.sin(ph) @ y)


def mhgls_np(t, yw, w, freqs, YY, nharms=1, amplitude_priors=None, cn0=None, sn0=None):
    """Multi-harmonic floating-mean GLS by direct sums in FP64, restating
    cuvarbase/lombscargle.py:337-400 (mhdirect_sums), :403-447
    (add_regularization), :450-494 (mhgls_params_from_sums) and :497-536
    (mhgls_from_sums); ybar = sum(yw) as a sequential sum in yw's own type,
    as the reference's Python sum() forms it."""
    yw_in = np.asarray(yw)
    ybar = float(np.cumsum(yw_in, dtype=yw_in.dtype)[-1])
    t = np.asarray(t, np.float64)
    yw = np.asarray(yw, np.float64)
    w = np.asarray(w, np.float64)
    H = int(nharms)
    D = np.zeros(H) if amplitude_priors is None else \
        np.ones(H) * np.power(amplitude_priors, -2.0)
    cn0 = np.zeros(H) if cn0 is None else np.asarray(cn0, np.float64)
    sn0 = np.zeros(H) if sn0 is None else np.asarray(sn0, np.float64)
    ns = np.arange(2 * H + 1)
    hs = ns[1:H + 1]
    out = np.empty(len(freqs))
    for i, f in enumerate(np.asarray(freqs, np.float64)):
        ph = 2 * np.pi * ((t * f) % 1.0)
        c = np.array([np.dot(w, np.cos(n * ph)) for n in ns])
        s = np.array([np.dot(w, np.sin(n * ph)) for n in ns])
        yc = np.array([np.dot(yw, np.cos(n * ph)) for n in hs])
        ys = np.array([np.dot(yw, np.sin(n * ph)) for n in hs])
        cc = np.array([[0.5 * (c[n + m] + c[abs(n - m)]) for m in hs] for n in hs])
        cs = np.array([[0.5 * (s[n + m] - (1 if n == m else np.sign(n - m)) * s[abs(n - m)])
                        for m in hs] for n in hs])
        ss = np.array([[0.5 * (c[abs(n - m)] - c[n + m]) for m in hs] for n in hs])
        C, S = c[1:H + 1], s[1:H + 1]
        YC, YS = yc - ybar * C, ys - ybar * S
        CC = cc - np.outer(C, C) + np.diag(D)
        CS = cs - np.outer(C, S)
        SS = ss - np.outer(S, S) + np.diag(D)
        YC, YS = YC + D * cn0, YS + D * sn0
        A = np.block([[CC, CS], [CS.T, SS]])
        th = np.linalg.solve(A, np.concatenate((YC, YS)))
        cn, sn = th[:H], th[H:]
        XX = np.outer(cn, cn) * CC + 2 * np.outer(cn, sn) * CS + np.outer(sn, sn) * SS
        out[i] = (2 * (np.dot(cn, YC) + np.dot(sn, YS)) - np.sum(XX)) / YY
    return out


def nfft_from_grid_np(grid, nf, tmin, tmax, spp, f0, b):
    """The steps of nfft_adjoint_async after gridding, on a given grid (its
    use_grid branch, cuvarbase/cunfft.py:270-301), in FP64: kernel nfft_shift
    (cuvarbase/kernels/cunfft.cu:59-82) when |f0| > 1e-9, the unnormalised
    inverse FFT (cuFFT ifft, cunfft.py:288), then kernel normalize
    (cunfft.cu:214-248) on the first nf bins."""
    g = np.asarray(grid, np.complex128).reshape(-1)
    ng = len(g)
    sT = spp * (tmax - tmin)
    k0 = f0 * sT
    if abs(f0) > 1e-9:
        g = g * np.exp(2j * np.pi * np.arange(ng) * k0 / ng)
    G = np.fft.ifft(g) * ng
    kk = k0 + np.arange(nf)
    n0 = tmin / sT * ng
    return G[:nf] * np.exp(2j * np.pi * n0 * kk / ng) * np.exp(b * (np.pi * kk / ng) ** 2)


def grid_ref_np(t, y, ng, m, sigma, spp=1.0):
    """tests/test_nfft.py:57-87 (precomp_psi + gpu_grid_scalar) restated,
    on the scaled positions x = (t - tmin) / (spp (tmax - tmin))."""
    t = np.asarray(t, np.float64)
    x = (t - t.min()) / (spp * (t.max() - t.min()))
    b = (2.0 * sigma * m) / ((2 * sigma - 1) * np.pi)
    xg = m + ng * x - np.floor(ng * x)
    q1 = np.exp(-xg ** 2 / b) / np.sqrt(np.pi * b)
    q2 = np.exp(2 * xg / b)
    q3 = np.exp(-np.arange(2 * m + 1) ** 2 / b)
    u = np.floor(ng * x - m).astype(np.int64)
    grid = np.zeros(int(ng))
    inds = np.arange(2 * m + 1)
    for i in range(len(t)):
        grid[(u[i] + inds) % ng] += y[i] * q1[i] * q2[i] ** inds * q3
    return grid
