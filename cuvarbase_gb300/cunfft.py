"""Adjoint non-equispaced FFT on GB300 (drop-in for cuvarbase/cunfft.py).

``NFFTAsyncProcess(...).run([(t, y, nf), ...])`` returns, per light curve,
the complex64 array

    out[k] = sum_j y_j exp(+2 pi i (f0 + k df) t_j),   k = 0 .. nf-1,
    df = 1 / (samples_per_peak (max t - min t)),  f0 = minimum_frequency,

the semantics pinned by cuvarbase/tests/test_nfft.py:202-239.  All curves of
one call run in one batched libcuvgls call.  ``just_return_gridded_data``
returns the reference-convention real Gaussian grid
(cuvarbase/cunfft.py:266-268).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .core import GPUAsyncProcess


class NFFTMemory:
    """Per-curve state of an adjoint NFFT (mirrors cuvarbase/cunfft.py:23-160):
    the data, sizes and the page-locked result ``ghat_c``."""

    def __init__(self, sigma, stream, m, use_double=False, precomp_psi=True,
                 **kwargs):
        self.sigma = sigma
        self.stream = stream
        self.m = m
        self.use_double = use_double
        self.precomp_psi = precomp_psi
        self.real_type = np.float64 if use_double else np.float32
        self.complex_type = np.complex128 if use_double else np.complex64
        self.other_settings = dict(kwargs)
        self.t = kwargs.get('t', None)
        self.y = kwargs.get('y', None)
        self.f0 = kwargs.get('f0', 0.)
        self.n0 = kwargs.get('n0', None)
        self.nf = kwargs.get('nf', None)
        self.ghat_c = kwargs.get('ghat_c', None)
        sig = 2.0 if self.sigma == 'auto' else float(self.sigma)
        D = (2 * sig - 1) * np.pi
        self.b = float(2 * sig * self.m) / D
        self._buf = None

    def allocate_pinned_cpu(self, **kwargs):
        self.nf = kwargs.get('nf', self.nf)
        assert self.nf is not None
        self._buf = _lib.PinnedBuffer(self.nf * np.dtype(self.complex_type).itemsize)
        self.ghat_c = self._buf.view(self.complex_type, self.nf)
        return self

    def allocate(self, **kwargs):
        self.n0 = kwargs.get('n0', self.n0)
        self.nf = kwargs.get('nf', self.nf)
        assert self.n0 is not None and self.nf is not None
        self.n = int((2.0 if self.sigma == 'auto' else self.sigma) * self.nf)
        if self._buf is None:
            self.allocate_pinned_cpu(**kwargs)
        return self

    def fromdata(self, t, y, allocate=True, **kwargs):
        self.tmin = float(np.min(t))
        self.tmax = float(np.max(t))
        self.t = np.ascontiguousarray(t, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=self.real_type)
        self.n0 = kwargs.get('n0', len(t))
        self.nf = kwargs.get('nf', self.nf)
        if self.nf is not None and allocate:
            self.allocate(**kwargs)
        return self


def _freq_grid(mem, minimum_frequency, samples_per_peak):
    df = 1.0 / (samples_per_peak * (mem.tmax - mem.tmin))
    return float(minimum_frequency), df


def nfft_adjoint_async(memory, functions, minimum_frequency=0., block_size=256,
                       just_return_gridded_data=False, use_grid=None,
                       fast_grid=True, transfer_to_device=True,
                       transfer_to_host=True, precomp_psi=True,
                       samples_per_peak=1, **kwargs):
    """Enqueue the adjoint NFFT of one curve (cuvarbase/cunfft.py:163-308).

    ``functions`` is the (handle, stream) pair of the calling process.
    Returns ``memory.ghat_c`` (valid after finish()), or the real grid when
    ``just_return_gridded_data`` is set (synchronously, as the reference).
    """
    handle, stream = functions
    if just_return_gridded_data:
        return _grids(handle, stream, [memory], samples_per_peak)[0]
    if use_grid is not None:
        return _finish_grid(handle, stream, memory, use_grid, minimum_frequency,
                            samples_per_peak)
    if memory.use_double:
        _launch_nfft64(handle, stream, [memory], minimum_frequency, samples_per_peak)
    else:
        _launch_nfft(handle, stream, [memory], minimum_frequency, samples_per_peak)
    return memory.ghat_c


def _launch_nfft(handle, stream, mems, minimum_frequency, samples_per_peak):
    n_tot = sum(len(m.t) for m in mems)
    nf_tot = sum(m.nf for m in mems)
    t = np.empty(n_tot, np.float64)
    y = np.empty(n_tot, np.float32)
    curves = (_lib.NfftCurve * len(mems))()
    out = _lib.PinnedBuffer(nf_tot * 8)
    o, fo = 0, 0
    for i, m in enumerate(mems):
        n = len(m.t)
        t[o:o + n] = m.t
        y[o:o + n] = m.y
        f0, df = _freq_grid(m, minimum_frequency, samples_per_peak)
        c = curves[i]
        c.pt_off, c.n, c.nf, c.f0, c.df, c.out_off = o, n, m.nf, f0, df, fo
        m._buf = out
        m.ghat_c = out.view(np.complex64, m.nf, fo * 8)
        o += n
        fo += m.nf
    inp = _lib.NfftInput()
    inp.n_curves = len(mems)
    inp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
    inp.curves = ctypes.cast(curves, ctypes.c_void_p)
    inp.t = t.ctypes.data
    inp.y = y.ctypes.data
    inp.n_points_total = n_tot
    inp.n_out_total = nf_tot
    handle.check(_lib.load().cuvgls_nfft_adjoint_batch(handle.ptr, ctypes.byref(inp),
                                                       out.ptr, stream), "nfft batch")


def _launch_nfft64(handle, stream, mems, minimum_frequency, samples_per_peak):
    """use_double: FP64 direct sums (cuvgls_nfft_adjoint_fp64), results as
    complex128 in each memory's ``ghat_c`` (valid after finish())."""
    n_tot = sum(len(m.t) for m in mems)
    nf_tot = sum(m.nf for m in mems)
    t = np.empty(n_tot, np.float64)
    y = np.empty(n_tot, np.float64)
    curves = (_lib.NfftCurve * len(mems))()
    out = _lib.PinnedBuffer(nf_tot * 16)
    o, fo = 0, 0
    for i, m in enumerate(mems):
        n = len(m.t)
        t[o:o + n] = m.t
        y[o:o + n] = m.y
        f0, df = _freq_grid(m, minimum_frequency, samples_per_peak)
        c = curves[i]
        c.pt_off, c.n, c.nf, c.f0, c.df, c.out_off = o, n, m.nf, f0, df, fo
        m._buf = out
        m.ghat_c = out.view(np.complex128, m.nf, fo * 16)
        o += n
        fo += m.nf
    inp = _lib.NfftInput()
    inp.n_curves = len(mems)
    inp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
    inp.curves = ctypes.cast(curves, ctypes.c_void_p)
    inp.t = t.ctypes.data
    inp.n_points_total = n_tot
    inp.n_out_total = nf_tot
    handle.check(_lib.load().cuvgls_nfft_adjoint_fp64(handle.ptr, ctypes.byref(inp),
                                                      y.ctypes.data, out.ptr, stream),
                 "nfft fp64")


def _finish_grid(handle, stream, mem, grid, minimum_frequency, samples_per_peak):
    """use_grid: the reference's steps after gridding (shift, inverse FFT,
    deconvolution; cuvarbase/cunfft.py:270-301) applied to ``grid`` instead
    of the gridded data, in FP64 on the device (cuvgls_nfft_from_grid).
    Returned synchronously in the memory's complex type."""
    g = np.ascontiguousarray(np.asarray(grid).reshape(-1), dtype=np.complex128)
    ng = int(mem.n)
    if len(g) != ng:
        raise ValueError("use_grid needs %d grid cells (sigma * nf), got %d" % (ng, len(g)))
    c = (_lib.GridFinCurve * 1)()
    c[0].grid_off, c[0].ng, c[0].nf, c[0].out_off = 0, ng, mem.nf, 0
    c[0].tmin, c[0].tmax = mem.tmin, mem.tmax
    c[0].spp, c[0].f0, c[0].b = float(samples_per_peak), float(minimum_frequency), mem.b
    out = np.empty(mem.nf, np.complex128)
    handle.check(_lib.load().cuvgls_nfft_from_grid(
        handle.ptr, 1, ctypes.cast(c, ctypes.c_void_p), g.ctypes.data, ng, mem.nf,
        _lib.HOST_INPUT | _lib.HOST_OUTPUT, out.ctypes.data, stream), "nfft from grid")
    handle.sync(stream)
    return out.astype(mem.complex_type)


def _grids(handle, stream, mems, samples_per_peak):
    """Reference-convention grids, returned synchronously as float arrays."""
    n_tot = sum(len(m.t) for m in mems)
    ngs = [int((2.0 if m.sigma == 'auto' else m.sigma) * m.nf) for m in mems]
    t = np.empty(n_tot, np.float64)
    y = np.empty(n_tot, np.float32)
    curves = (_lib.GridCurve * len(mems))()
    out = np.zeros(sum(ngs), np.float32)
    o, go = 0, 0
    for i, (m, ng) in enumerate(zip(mems, ngs)):
        n = len(m.t)
        t[o:o + n] = m.t
        y[o:o + n] = m.y
        c = curves[i]
        c.pt_off, c.n, c.ng = o, n, ng
        c.tmin, c.tmax, c.spp, c.out_off = m.tmin, m.tmax, float(samples_per_peak), go
        o += n
        go += ng
    handle.check(_lib.load().cuvgls_spread_ref(
        handle.ptr, len(mems), ctypes.cast(curves, ctypes.c_void_p), t.ctypes.data,
        y.ctypes.data, n_tot, len(out), _lib.HOST_INPUT | _lib.HOST_OUTPUT,
        out.ctypes.data, stream), "spread_ref")
    handle.sync(stream)
    res, go = [], 0
    for ng in ngs:
        res.append(out[go:go + ng].astype(np.float64))
        go += ng
    return res


class NFFTAsyncProcess(GPUAsyncProcess):
    """Adjoint NFFT of batches of light curves (mirrors cuvarbase/cunfft.py:311-542).

    Parameters as in the reference: ``sigma=4``, ``m=8``, ``autoset_m=False``,
    ``tol=1e-8``, ``block_size=256``, ``use_double=False``,
    ``use_fast_math=True``.  ``sigma='auto'`` lets the library choose the
    window, oversampling and window width per frequency count (the
    "exponential of semicircle" window at sigma 1.28, m = 5; the GLS budget
    is max |dP| <= 2e-5).  The NFFT kernels keep FP64 for time offsets and phase
    reduction; ``use_double=True`` computes FP64 direct sums instead
    (exact, cost N x nf) and returns complex128.  ``use_grid`` (the
    reference's debug input of a grid of sigma * nf cells) applies the
    shift, inverse FFT and deconvolution of the reference to that grid.
    """

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.sigma = kwargs.get('sigma', 4)
        if self.sigma is None or self.sigma == 'auto':
            self.sigma = 'auto'
        self.m = kwargs.get('m', 8)
        self.autoset_m = kwargs.get('autoset_m', False)
        self.block_size = kwargs.get('block_size', 256)
        self.use_double = kwargs.get('use_double', False)
        self.m_tol = kwargs.get('tol', 1E-8)
        self.real_type = np.float64 if self.use_double else np.float32
        self.complex_type = np.complex128 if self.use_double else np.complex64
        self.function_names = ['nfft_adjoint']
        self.allocated_memory = []

    def _lib_sigma(self):
        """sigma as the library takes it (negative = autotune)."""
        return -1.0 if self.sigma == 'auto' else float(self.sigma)

    def m_from_C(self, C, sigma):
        """m for an error constant C ~ tol / N (cuvarbase/cunfft.py:378-388)."""
        sigma = 2.0 if sigma == 'auto' else sigma
        D = (np.pi * (1. - 1. / (2. * sigma - 1.)))
        return int(np.ceil(-np.log(0.25 * C) / D))

    def estimate_m(self, N):
        """m for the tolerance ``tol`` and N frequencies (cunfft.py:390-411)."""
        return self.m_from_C(self.m_tol / N, self.sigma)

    def get_m(self, N=None):
        """The window half-width for N frequencies (cunfft.py:414-431)."""
        if self.autoset_m:
            return self.estimate_m(N)
        return self.m

    def allocate(self, data, **kwargs):
        """NFFTMemory objects for [(t, y, nf), ...] (cunfft.py:468-505)."""
        stream = self._stream()  # one stream serves the whole batched call
        mems = []
        for i, (t, y, nf) in enumerate(data):
            m = self.get_m(nf)
            mem = NFFTMemory(self.sigma, stream, m,
                             use_double=self.use_double, **kwargs)
            mems.append(mem.fromdata(t, y, nf=nf, allocate=True, **kwargs))
        return mems

    def run(self, data, memory=None, **kwargs):
        """Adjoint NFFTs of [(t, y, nf), ...] (cunfft.py:507-542)."""
        self._compile_and_prepare_functions()
        if memory is None:
            memory = self.allocate(data, **kwargs)
        spp = kwargs.get('samples_per_peak', 1)
        f0 = kwargs.get('minimum_frequency', 0.)
        by_m = {}
        for mem in memory:
            by_m.setdefault(mem.m, []).append(mem)
        if kwargs.get('just_return_gridded_data', False):
            res = {}
            for m, mems in by_m.items():
                h = self._handle(2.0 if self.sigma == 'auto' else self.sigma, m)
                for mem, g in zip(mems, _grids(h, self._stream().ptr, mems, spp)):
                    res[id(mem)] = g
            return [res[id(mem)] for mem in memory]
        if kwargs.get('use_grid', None) is not None:
            h = self._handle(self._lib_sigma(), self.m)
            return [_finish_grid(h, self._stream().ptr, mem, kwargs['use_grid'], f0, spp)
                    for mem in memory]
        for m, mems in by_m.items():
            h = self._handle(self._lib_sigma(), m)
            if self.use_double:
                _launch_nfft64(h, self._stream().ptr, mems, f0, spp)
            else:
                _launch_nfft(h, self._stream().ptr, mems, f0, spp)
        return [mem.ghat_c for mem in memory]
