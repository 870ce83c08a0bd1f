"""Generalized Lomb-Scargle periodograms on GB300 (drop-in for
cuvarbase/lombscargle.py).

The public names, arguments, defaults and return types follow the
reference: ``LombScargleAsyncProcess`` with ``run`` / ``batched_run`` /
``batched_run_const_nfreq`` / ``preallocate`` / ``allocate`` /
``memory_requirement``, ``LombScargleMemory``, ``lomb_scargle_async``,
``lomb_scargle_direct_sums``, ``fap_baluev``, ``lomb_scargle_simple``,
``get_k0`` and ``check_k0``.

What differs underneath: every curve of a ``run`` call goes to the GPU in one
batched call of libcuvgls (spreading + two-pass shared-memory FFT + fused GLS
finish, see include/cuvgls.h) instead of nine kernel launches and two cuFFT
plans per curve.  Results are numpy views of page-locked host buffers owned
by the memory objects, valid after ``finish()``, as in the reference.
"""
from __future__ import annotations

import ctypes

import numpy as np
from scipy.special import gammaln

from . import _lib
from .core import GPUAsyncProcess
from .cunfft import NFFTAsyncProcess
from .utils import autofrequency as utils_autofreq
from .utils import normalize_light_curves, weights


def get_k0(freqs):
    """Index of the first frequency, freqs[0] / df (cuvarbase/lombscargle.py:25-26)."""
    return max([1, int(round(freqs[0] / (freqs[1] - freqs[0])))])


def _grid_df(freqs):
    """Spacing of a linear frequency grid for the kernels, (f[-1] - f[0]) /
    (nf - 1): on a grid of many bins far from zero, f[1] - f[0] (two close
    large numbers) loses ~1e-10 of df, which over millions of bins moves
    the evaluated frequencies by ~1e-3 bin.  Equal to f[1] - f[0] on an exact
    grid."""
    return float((freqs[-1] - freqs[0]) / (len(freqs) - 1))


def check_k0(freqs, k0=None, rtol=1E-2, atol=1E-7):
    """Assert freqs[0] == k0 * df (cuvarbase/lombscargle.py:29-33)."""
    k0 = k0 if k0 is not None else get_k0(freqs)
    df = freqs[1] - freqs[0]
    f0 = k0 * df
    assert abs(f0 - freqs[0]) < rtol * df + atol


def _mode(floating_mean=True, window=False):
    return _lib.MODE_WINDOW if window else (
        _lib.MODE_FLOATING_MEAN if floating_mean else _lib.MODE_STANDARD)


class _Arena:
    """One page-locked float32 buffer shared by the results of several curves."""

    def __init__(self, nfloats, dtype=np.float32):
        self.dtype = np.dtype(dtype)
        self.n = int(nfloats)
        self.buf = _lib.PinnedBuffer(max(self.n, 1) * self.dtype.itemsize)

    def view(self, off, count):
        return self.buf.view(self.dtype, count, off * self.dtype.itemsize)

    @property
    def ptr(self):
        return self.buf.ptr


class LombScargleMemory:
    """Per-light-curve state (mirrors cuvarbase/lombscargle.py:36-334).

    Holds the host-prepared data (t in FP64; yw, w in float32, as the
    reference casts them; YY, ybar) and the page-locked result buffer
    ``lsp_c``.  Device buffers belong to the library handle, which reuses
    them across calls, so there is no per-curve device allocation.
    """

    def __init__(self, sigma, stream, m, **kwargs):
        self.sigma = sigma
        self.stream = stream
        self.m = m
        self.k0 = kwargs.get('k0', 0)
        self.precomp_psi = kwargs.get('precomp_psi', True)
        self.amplitude_prior = kwargs.get('amplitude_prior', None)
        self.window = kwargs.get('window', False)
        self.nharmonics = kwargs.get('nharmonics', 1)
        self.use_fft = kwargs.get('use_fft', True)
        self.other_settings = dict(kwargs)
        self.floating_mean = kwargs.get('floating_mean', True)
        self.use_double = kwargs.get('use_double', False)
        self.mode = _mode(self.floating_mean, self.window)
        self.n0 = kwargs.get('n0', None)
        self.nf = kwargs.get('nf', None)
        self.buffered_transfer = kwargs.get('buffered_transfer', False)
        self.n0_buffer = kwargs.get('n0_buffer', None)
        self.real_type = np.float32
        self.reg = np.zeros(2 * self.nharmonics + 1, dtype=np.float32)
        if self.amplitude_prior is not None:
            lmbda = np.power(self.amplitude_prior, -2)
            if isinstance(lmbda, float):
                lmbda = lmbda * np.ones(self.nharmonics)
            for i, lam in enumerate(np.atleast_1d(lmbda)):
                self.reg[2 * i] = lam
                self.reg[1 + 2 * i] = lam
        self.lsp_c = kwargs.get('lsp_c', None)
        self._arena = None
        self._off = 0
        self.t = kwargs.get('t', None)
        self.yw = kwargs.get('yw', None)
        self.w = kwargs.get('w', None)
        self.ybar = 0.
        self.yy = kwargs.get('yy', 1.)

    # --- allocation -----------------------------------------------------
    def allocate_pinned_cpu(self, **kwargs):
        nf = kwargs.get('nf', self.nf)
        assert nf is not None
        self._arena = _Arena(nf)
        self._off = 0
        self.lsp_c = self._arena.view(0, nf)
        return self

    def _bind(self, arena, off):
        self._arena, self._off = arena, off
        self.lsp_c = arena.view(off, self.nf)

    def allocate(self, **kwargs):
        """Allocate the result buffer (device memory is the handle's)."""
        self.nf = kwargs.get('nf', self.nf)
        assert self.nf is not None
        if self._arena is None:
            self.allocate_pinned_cpu(**kwargs)
        return self

    # --- data -------------------------------------------------------------
    def setdata(self, **kwargs):
        """Prepare the light curve (cuvarbase/lombscargle.py:235-293):
        w = dy^-2 / sum, ybar = w.y, yw = w (y - ybar), YY = w.(y - ybar)^2
        in FP64; yw and w are then cast to float32 as the reference does.
        t stays FP64 (the kernels use FP64 for t - t0)."""
        t = kwargs.get('t', self.t)
        yw = kwargs.get('yw', self.yw)
        w = kwargs.get('w', self.w)
        y = kwargs.get('y', None)
        dy = kwargs.get('dy', None)
        self.ybar = 0.
        self.yy = kwargs.get('yy', 1.)
        self.n0 = kwargs.get('n0', len(t))
        if dy is not None:
            assert 'w' not in kwargs
            w = weights(dy)
        if y is not None:
            assert 'yw' not in kwargs
            self.ybar = np.dot(y, w)
            yw = np.multiply(w, y - self.ybar)
            self.yy = np.dot(w, np.power(y - self.ybar, 2))
        self.t = np.ascontiguousarray(t, dtype=np.float64)
        self.yw = np.ascontiguousarray(yw, dtype=np.float32)
        self.w = np.ascontiguousarray(w, dtype=np.float32)
        if self.buffered_transfer and self.n0_buffer is not None:
            assert self.n0 <= self.n0_buffer
        # sum(yw) as the reference's direct sums form it (sequential float32)
        self.yw_sum = float(np.cumsum(self.yw, dtype=np.float32)[-1]) if len(self.yw) else 0.
        self.w_sum = float(np.sum(self.w, dtype=np.float64))
        self.tmin = float(np.min(self.t))
        self.tmax = float(np.max(self.t))
        return self

    def fromdata(self, **kwargs):
        self.setdata(**kwargs)
        if kwargs.get('allocate', True):
            self.allocate(**kwargs)
        return self

    def set_gpu_arrays_to_zero(self, **kwargs):
        """Kept for API compatibility: the kernels zero their own tiles."""
        return self

    def transfer_data_to_gpu(self, **kwargs):
        """Kept for API compatibility: data moves inside the batch call."""
        return self

    def transfer_lsp_to_cpu(self, **kwargs):
        """Kept for API compatibility: results land in lsp_c after finish()."""
        return self


def _launch_gls(handle, stream, mems, freqs_list, use_fft=True, mode=None,
                out_f64=False):
    """One libcuvgls call per (arena, mode, prior) group of memory objects."""
    groups = {}
    for mem, fr in zip(mems, freqs_list):
        md = mem.mode if mode is None else mode
        key = (id(mem._arena), md, float(mem.reg[0]))
        groups.setdefault(key, []).append((mem, fr))
    for (_, md, lam), items in groups.items():
        arena = items[0][0]._arena
        n_tot = sum(len(m.t) for m, _ in items)
        t = np.empty(n_tot, np.float64)
        yw = np.empty(n_tot, np.float32)
        w = np.empty(n_tot, np.float32)
        curves = (_lib.Curve * len(items))()
        o = 0
        for i, (m, fr) in enumerate(items):
            n = len(m.t)
            t[o:o + n] = m.t
            yw[o:o + n] = m.yw
            w[o:o + n] = m.w
            df = _grid_df(fr)
            c = curves[i]
            c.pt_off, c.n, c.nf, c.k0, c.df = o, n, m.nf, int(m.k0), df
            c.yy, c.ybar, c.yw_sum, c.w_sum = float(m.yy), float(m.ybar), m.yw_sum, m.w_sum
            c.out_off = m._off
            o += n
        inp = _lib.GlsInput()
        inp.n_curves = len(items)
        inp.mode = md
        inp.curves = ctypes.cast(curves, ctypes.c_void_p)
        inp.t = t.ctypes.data
        inp.yw = yw.ctypes.data
        inp.w = w.ctypes.data
        inp.reg[0], inp.reg[1], inp.reg[2] = lam, lam, 0.0
        inp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
        inp.n_points_total = n_tot
        inp.n_out_total = arena.n
        L = _lib.load()
        fn = L.cuvgls_gls_batch if use_fft else L.cuvgls_gls_direct_batch
        handle.check(fn(handle.ptr, ctypes.byref(inp), arena.ptr, stream),
                     "gls batch" if use_fft else "gls direct")
        # keep the staging arrays alive until the copies are enqueued: the
        # library copies pageable input synchronously, so nothing to hold.


_default_handle = None


def _direct_handle():
    global _default_handle
    if _default_handle is None:
        _default_handle = _lib.Handle(sigma=2.0, m=8)
    return _default_handle


def lomb_scargle_direct_sums(t, yw, w, freqs, YY, nharms=1, **kwargs):
    """Multi-harmonic floating-mean GLS by direct summation
    (cuvarbase/lombscargle.py:539-576, with mhdirect_sums, add_regularization
    and mhgls_from_sums, :337-536), evaluated on the GPU in FP64
    (cuvgls_mhgls_direct) for 1 <= nharms <= 8 and any frequencies.
    ``amplitude_priors`` (a float, or one per harmonic), ``cn0`` and ``sn0``
    are the reference's regulariser arguments; ybar = sum(yw) as the
    reference's Python sum() forms it.  A singular system gives NaN where the
    reference's numpy.linalg.solve raises.
    """
    H = int(nharms)
    if not 1 <= H <= 8:
        raise ValueError("nharms must be 1..8")
    yw_in = np.asarray(yw)
    ybar = float(np.cumsum(yw_in, dtype=yw_in.dtype)[-1])
    t = np.ascontiguousarray(t, dtype=np.float64)
    ywd = np.ascontiguousarray(yw_in, dtype=np.float64)
    wd = np.ascontiguousarray(w, dtype=np.float64)
    freqs = np.ascontiguousarray(freqs, dtype=np.float64).reshape(-1)
    if not (len(t) == len(ywd) == len(wd)) or len(t) < 1 or len(freqs) < 1:
        raise ValueError("t, yw, w need equal, nonzero lengths and freqs at least one value")
    ap = kwargs.get('amplitude_priors', None)
    d = None if ap is None else np.ascontiguousarray(
        np.ones(H) * np.power(np.asarray(ap, dtype=np.float64), -2.0))
    cn0 = kwargs.get('cn0', None)
    sn0 = kwargs.get('sn0', None)
    cn0 = None if cn0 is None else np.ascontiguousarray(cn0, dtype=np.float64)
    sn0 = None if sn0 is None else np.ascontiguousarray(sn0, dtype=np.float64)
    for name, v in (("amplitude_priors", d), ("cn0", cn0), ("sn0", sn0)):
        if v is not None and v.shape != (H,):
            raise ValueError("%s needs one value per harmonic" % name)
    ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
    out = np.empty(len(freqs), np.float64)
    h = _direct_handle()
    h.check(_lib.load().cuvgls_mhgls_direct(
        h.ptr, H, t.ctypes.data, ywd.ctypes.data, wd.ctypes.data, len(t), freqs.ctypes.data,
        len(freqs), float(YY), ybar, ptr(d), ptr(cn0), ptr(sn0),
        _lib.HOST_INPUT | _lib.HOST_OUTPUT, out.ctypes.data, None), "mhgls direct")
    h.sync(None)
    return out

def lomb_scargle_async(memory, functions, freqs, block_size=256, use_fft=True,
                       python_dir_sums=False, transfer_to_device=True,
                       transfer_to_host=True, window=False, **kwargs):
    """Enqueue the periodogram of one light curve (cuvarbase/lombscargle.py:579-689).

    ``functions`` is the (handle, stream) pair of the calling process (the
    reference passes its compiled kernels here).  Returns ``memory.lsp_c``.
    """
    handle, stream = functions
    df = freqs[1] - freqs[0]
    assert get_k0(freqs) == memory.k0
    if python_dir_sums:
        return lomb_scargle_direct_sums(memory.t, memory.yw, memory.w, freqs,
                                        memory.yy)
    _launch_gls(handle, stream, [memory], [freqs], use_fft=use_fft)
    return memory.lsp_c


class LombScargleAsyncProcess(GPUAsyncProcess):
    """GLS periodograms for batches of light curves (mirrors
    cuvarbase/lombscargle.py:692-1112).

    Parameters are those of the reference (``sigma=4``, ``m=8``,
    ``autoset_m=False``, ``tol=1e-8``, ``use_double=False``,
    ``nharmonics=1``, ...).  ``sigma`` is the minimum grid oversampling; the
    band is centred on the grid, so sigma=2 already meets |dP| <= 1e-4.
    ``sigma='auto'`` lets the library pick the window, sigma and m per
    frequency count (the smallest grid within a max |dP| <= 2e-5 budget: the
    "exponential of semicircle" window at sigma 1.28 with 10 taps) and the
    grid shape of least measured cost; explicit sigma and m keep the
    reference's Gaussian.
    ``precision='fp32'`` selects the all-FP32 comparison variant.
    """

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.nfft_proc = NFFTAsyncProcess(*args, **kwargs)
        self.real_type = self.nfft_proc.real_type
        self.complex_type = self.nfft_proc.complex_type
        self.block_size = self.nfft_proc.block_size
        self.use_double = self.nfft_proc.use_double
        self.memory = None
        self.nharmonics = kwargs.get('nharmonics', 1)
        self.precision = (_lib.PREC_FP32 if kwargs.get('precision', 'mixed') == 'fp32'
                          else _lib.PREC_MIXED)
        self.workspace_bytes = int(kwargs.get('workspace_bytes', 0))
        if self.nharmonics > 1:
            raise Exception("Only 1 harmonic is supported right now")

    def _gls_handle(self, nf):
        m = self.nfft_proc.get_m(nf)
        return self._handle(self.nfft_proc._lib_sigma(), m, self.precision,
                            self.workspace_bytes)

    def memory_requirement(self, n0, nf, k0, nbatch=1, **kwargs):
        """Device bytes for nbatch light curves of n0 points and nf
        frequencies (the reference's estimate at lombscargle.py:752-796
        reads `mem` before assigning it; this one asks the library)."""
        h = self._gls_handle(nf)
        n = (ctypes.c_int64 * nbatch)(*([int(n0)] * nbatch))
        f = (ctypes.c_int64 * nbatch)(*([int(nf)] * nbatch))
        out = ctypes.c_int64()
        h.check(_lib.load().cuvgls_batch_bytes(h.ptr, nbatch, n, f, 1,
                                               ctypes.byref(out)), "batch bytes")
        return int(out.value)

    def allocate_for_single_lc(self, t, y, dy, nf, k0=0, stream=None, **kwargs):
        m = self.nfft_proc.get_m(nf)
        kw = dict(use_double=self.use_double, nharmonics=self.nharmonics)
        kw.update(kwargs)
        mem = LombScargleMemory(self.nfft_proc.sigma, stream, m, k0=k0, **kw)
        mem.fromdata(t=t, y=y, dy=dy, nf=nf, allocate=True, **kwargs)
        return mem

    def preallocate(self, max_nobs, nlcs=1, nf=None, k0=None, freqs=None,
                    streams=None, **kwargs):
        """Memory for nlcs curves of up to max_nobs points sharing one
        result arena; later run() calls reuse it (results are overwritten
        by the next run, as in the reference)."""
        if freqs is not None:
            k0 = get_k0(freqs)
            nf = len(freqs)
        if nf is not None:
            assert k0 is not None
        m = self.nfft_proc.get_m(nf)
        arena = _Arena(nlcs * nf)
        self.memory = []
        for i in range(nlcs):
            stream = None if streams is None else streams[i]
            mem = LombScargleMemory(self.nfft_proc.sigma, stream, m, k0=k0,
                                    buffered_transfer=True, n0_buffer=max_nobs,
                                    nf=nf, use_double=self.use_double,
                                    nharmonics=self.nharmonics, **kwargs)
            mem._bind(arena, i * nf)
            self.memory.append(mem)
        return self.memory

    def autofrequency(self, *args, **kwargs):
        return utils_autofreq(*args, **kwargs)

    def _nfreqs(self, *args, **kwargs):
        return len(self.autofrequency(*args, **kwargs))

    def allocate(self, data, nfreqs=None, k0s=None, **kwargs):
        """Memory objects for a list of (t, y, dy) light curves, sharing one
        page-locked result arena."""
        self._stream()  # one stream serves the whole batched call
        nfrqs = nfreqs
        if nfrqs is None:
            nfrqs = [self._nfreqs(t, **kwargs) for (t, y, dy) in data]
        elif isinstance(nfreqs, (int, np.integer)):
            nfrqs = [int(nfreqs)] * len(data)
        if k0s is None:
            k0s = [1] * len(nfrqs)
        elif isinstance(k0s, (int, float, np.integer)):
            k0s = [k0s] * len(nfrqs)
        nfrqs = [int(n) for n in nfrqs]
        arena = _Arena(sum(nfrqs))
        mems, off = [], 0
        for (t, y, dy), nf, k0 in zip(data, nfrqs, k0s):
            m = self.nfft_proc.get_m(nf)
            kw = dict(use_double=self.use_double, nharmonics=self.nharmonics)
            kw.update(kwargs)
            mem = LombScargleMemory(self.nfft_proc.sigma, self._stream(), m,
                                    k0=int(k0), **kw)
            mem.nf = nf
            mem.setdata(t=t, y=y, dy=dy)
            mem._bind(arena, off)
            off += nf
            mems.append(mem)
        return mems

    def run(self, data, use_fft=True, memory=None, freqs=None, **kwargs):
        """Periodograms of a list of (t, y, dy) light curves
        (cuvarbase/lombscargle.py:923-1010).

        Returns [(freqs, powers)] with ``powers`` valid after finish().
        Keyword arguments as in the reference: floating_mean, window,
        amplitude_prior, samples_per_peak, nyquist_factor, minimum_frequency,
        maximum_frequency, python_dir_sums.
        """
        self._compile_and_prepare_functions()
        if len(data) == 0:
            return []
        # without memory objects the preparation runs on the GPU, where the
        # mean removal of normalize_light_curves is not needed (the power
        # does not depend on shifts of t or y)
        raw = (memory is None and self.memory is None and use_fft
               and not kwargs.get('python_dir_sums', False) and self.nharmonics == 1)
        if not raw:
            data = normalize_light_curves(data)
        frqs = freqs
        if frqs is None:
            frqs = [self.autofrequency(d[0], **kwargs) for d in data]
        elif isinstance(frqs[0], (float, np.floating)):
            frqs = [frqs] * len(data)
        assert len(frqs) == len(data)
        k0s = [get_k0(frq) for frq in frqs]
        for frq, k0 in zip(frqs, k0s):
            check_k0(frq, k0=k0)
        if raw:
            # the host preparation (weights, ybar, yw, YY) runs on the GPU
            return _run_raw(self, data, frqs, k0s, **kwargs)
        if memory is None:
            memory = self.memory
        if memory is None:
            nfreqs = [len(frq) for frq in frqs]
            memory = self.allocate(data, nfreqs=nfreqs, k0s=k0s,
                                   use_fft=use_fft, **kwargs)
        else:
            for i, (t, y, dy) in enumerate(data):
                memory[i].set_gpu_arrays_to_zero(**kwargs)
                memory[i].setdata(t=t, y=y, dy=dy, **{k: v for k, v in kwargs.items()
                                                     if k in ('yy', 'n0')})
                memory[i].k0 = k0s[i]
                if memory[i].nf != len(frqs[i]):
                    raise ValueError("memory was allocated for %d frequencies, got %d"
                                     % (memory[i].nf, len(frqs[i])))
        mems = list(memory[:len(data)])
        if kwargs.get('python_dir_sums', False):
            out = []
            for mem, frq in zip(mems, frqs):
                out.append((frq, lomb_scargle_direct_sums(mem.t, mem.yw, mem.w, frq,
                                                          mem.yy)))
            return out
        for mem in mems:
            if 'floating_mean' in kwargs or 'window' in kwargs:
                mem.floating_mean = kwargs.get('floating_mean', mem.floating_mean)
                mem.window = kwargs.get('window', mem.window)
                mem.mode = _mode(mem.floating_mean, mem.window)
            if 'amplitude_prior' in kwargs and kwargs['amplitude_prior'] is not None:
                lam = float(np.power(kwargs['amplitude_prior'], -2))
                mem.reg[:2] = lam
        nf_max = max(m.nf for m in mems)
        h = self._gls_handle(nf_max)
        _launch_gls(h, self._stream().ptr, mems, frqs, use_fft=use_fft)
        return [(f, m.lsp_c) for f, m in zip(frqs, mems)]

    def autotune(self, data, freqs, steps=3, max_shapes=8):
        """Time the grid shapes the planner weighs for ``len(freqs)``
        frequencies on the curves ``data`` and pin the fastest on this
        process's plan, so that later runs with that frequency count use it
        (``cuvarbase_gb300.tune.autotune``; no reference counterpart).
        ``freqs`` is one grid, or a list of one grid per curve, all of the
        same length.  Returns the shapes fastest first."""
        from .tune import autotune
        grids = freqs if isinstance(freqs, (list, tuple)) else [freqs]
        return autotune(self._gls_handle(len(grids[0])), data, freqs, steps=steps,
                        max_shapes=max_shapes)

    def batched_run_const_nfreq(self, data, batch_size=10, use_fft=True,
                                freqs=None, only_return_best_freqs=False,
                                ignore_freq_mask=None, **kwargs):
        """All curves on one shared frequency grid
        (cuvarbase/lombscargle.py:1012-1112).  The grid is built from the
        longest-baseline curve and snapped to df (k0 + arange(nf)).  The
        curves run in batches of ``batch_size`` light curves per library
        call (use a large batch for throughput)."""
        if not use_fft or kwargs.get('python_dir_sums', False):
            data = normalize_light_curves(data)
        if freqs is None:
            longest = max(data, key=lambda d: max(d[0]) - min(d[0]))
            freqs = self.autofrequency(longest[0], **kwargs)
            df = freqs[1] - freqs[0]
            k0 = get_k0(freqs)
            nf = int(round(max(freqs) / df)) - k0
            freqs = df * (k0 + np.arange(nf))
        freqs = np.asarray(freqs)
        df = freqs[1] - freqs[0]
        k0 = get_k0(freqs)
        nf = len(freqs)
        check_k0(freqs, k0=k0)
        if only_return_best_freqs and use_fft and ignore_freq_mask is None:
            return _best_freqs_of(self, data, freqs, batch_size, **kwargs)
        mask = (np.ones(nf, bool) if ignore_freq_mask is None
                else ~np.asarray(ignore_freq_mask))
        bsize = max(1, min(len(data), batch_size))
        kw = {k: v for k, v in kwargs.items() if k not in ('samples_per_peak',
                                                            'nyquist_factor',
                                                            'minimum_frequency',
                                                            'maximum_frequency')}
        # with the FFT path the curves are prepared on the GPU (no memory
        # objects); the direct sums keep the reference's preallocated memory
        raw = use_fft and not kw.get('python_dir_sums', False)
        if not raw:
            self.preallocate(max(len(d[0]) for d in data), nlcs=bsize, nf=nf, k0=k0,
                             **{k: v for k, v in kwargs.items()
                                if k in ('floating_mean', 'window', 'amplitude_prior')})
        lsps, best_freqs, sigs = [], [], []
        for b0 in range(0, len(data), bsize):
            batch = data[b0:b0 + bsize]
            if raw:
                res = _run_raw(self, batch, [freqs] * len(batch), [k0] * len(batch), **kw)
            else:
                res = self.run(batch, memory=self.memory, freqs=freqs,
                               use_fft=use_fft, **kw)
            self.finish()
            for i, (f, p) in enumerate(res):
                if only_return_best_freqs:
                    pm = p[mask]
                    bi = int(np.argmax(pm))
                    fap = fap_baluev(batch[i][0], batch[i][2], pm[bi],
                                     np.max(freqs[mask]))
                    best_freqs.append(freqs[mask][bi])
                    sigs.append(1. - fap)
                else:
                    lsps.append(np.copy(p))
        self.memory = None
        if only_return_best_freqs:
            return best_freqs, sigs
        return [(freqs, lsp) for lsp in lsps]


def _raw_buffer(proc, nbytes):
    """A page-locked result buffer of the process: a pooled one that no
    earlier result views any more, else a new one."""
    import sys
    pool = proc.__dict__.setdefault('_raw_pool', [])
    for buf in pool:
        # references: the pool, the loop variable, getrefcount's argument
        if buf.nbytes >= nbytes and sys.getrefcount(buf) <= 3:
            return buf
    buf = _lib.PinnedBuffer(max(int(nbytes), 1 << 20))
    pool.append(buf)
    return buf


def _run_raw(proc, data, frqs, k0s, best=False, **kwargs):
    """One cuvgls_gls_raw call for a list of (t, y, dy) curves: the weights,
    ybar, yw and YY of every curve are computed on the GPU from the raw FP64
    arrays, so the host only concatenates them.  Returns [(freqs, powers)]
    (powers valid after finish()) or, with best=True, (best_k, best_p)
    arrays after synchronising."""
    n = np.fromiter((len(d[0]) for d in data), np.int64, len(data))
    off = np.zeros(len(data) + 1, np.int64)
    off[1:] = np.cumsum(n)
    t = np.concatenate([np.asarray(d[0], np.float64) for d in data])
    y = np.concatenate([np.asarray(d[1], np.float64) for d in data])
    dy = np.concatenate([np.asarray(d[2], np.float64) for d in data])
    nfs = np.fromiter((len(f) for f in frqs), np.int64, len(frqs))
    oo = np.zeros(len(data) + 1, np.int64)
    oo[1:] = np.cumsum(nfs)
    curves = (_lib.RawCurve * len(data))()
    for i, f in enumerate(frqs):
        c = curves[i]
        c.pt_off, c.n, c.nf, c.k0 = int(off[i]), int(n[i]), int(nfs[i]), int(k0s[i])
        c.df, c.out_off = _grid_df(f), int(oo[i])
    fm, win = kwargs.get('floating_mean', True), kwargs.get('window', False)
    lam = 0.0
    if kwargs.get('amplitude_prior') is not None:
        lam = float(np.power(kwargs['amplitude_prior'], -2))
    inp = _lib.RawInput()
    inp.n_curves, inp.mode = len(data), _mode(fm, win)
    inp.curves = ctypes.cast(curves, ctypes.c_void_p)
    inp.t, inp.y, inp.dy = t.ctypes.data, y.ctypes.data, dy.ctypes.data
    inp.reg[0], inp.reg[1], inp.reg[2] = lam, lam, 0.0
    inp.flags = _lib.HOST_INPUT | _lib.HOST_OUTPUT
    inp.n_points_total, inp.n_out_total = int(off[-1]), int(oo[-1])
    h = proc._gls_handle(int(nfs.max()))
    stream = proc._stream().ptr
    L = _lib.load()
    if best:
        bk = np.empty(len(data), np.int64)
        bp = np.empty(len(data), np.float32)
        h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(inp), None, bk.ctypes.data,
                                 bp.ctypes.data, stream), "gls raw best")
        h.sync(stream, -1)
        return bk, bp
    buf = _raw_buffer(proc, 4 * int(oo[-1]))
    # the library copies pageable inputs before the call returns
    h.check(L.cuvgls_gls_raw(h.ptr, ctypes.byref(inp), buf.ptr, None, None, stream),
            "gls raw")
    return [(f, buf.view(np.float32, int(nfs[i]), 4 * int(oo[i]))) for i, f in enumerate(frqs)]


def _best_freqs_of(proc, data, freqs, batch_size, **kwargs):
    """Best frequency and significance of each curve on one shared grid,
    with the curve preparation and the argmax on the GPU (cuvgls_gls_raw
    with best-frequency output): only the index and power of each curve's
    peak leave the device.  Same result as the host
    argmax of the full periodogram (ties: lowest index); the significance
    1 - fap_baluev(...) is computed on the host as the reference does
    (cuvarbase/lombscargle.py:1094-1105)."""
    freqs = np.asarray(freqs, np.float64)
    k0 = get_k0(freqs)
    fmax = float(np.max(freqs))
    mkw = {k: v for k, v in kwargs.items()
           if k in ('floating_mean', 'window', 'amplitude_prior')}
    best_freqs, sigs = [], []
    bsize = max(1, batch_size)
    for b0 in range(0, len(data), bsize):
        batch = data[b0:b0 + bsize]
        bk, bp = _run_raw(proc, batch, [freqs] * len(batch), [k0] * len(batch), best=True,
                          **mkw)
        for (t, y, dy), k, pw in zip(batch, bk, bp):
            k = int(k) if k >= 0 else 0     # no valid power: as argmax of all -1
            fap = fap_baluev(t, dy, float(pw), fmax)
            best_freqs.append(freqs[k])
            sigs.append(1. - fap)
    return best_freqs, sigs



def fap_baluev(t, dy, z, fmax, d_K=3, d_H=1, use_gamma=True):
    """False-alarm probability of a periodogram peak, Baluev (2008)
    (cuvarbase/lombscargle.py:1115-1184), evaluated on the host."""
    N = len(t)
    d = d_K - d_H
    N_K = N - d_K
    N_H = N - d_H
    g = (0.5 * N_H) ** (0.5 * (d - 1))
    if use_gamma:
        g = np.exp(gammaln(0.5 * N_H) - gammaln(0.5 * (N_K + 1)))
    w = np.power(dy, -2)
    tbar = np.dot(w, t) / sum(w)
    Dt = np.dot(w, np.power(t - tbar, 2)) / sum(w)
    Teff = np.sqrt(4 * np.pi * Dt)
    W = fmax * Teff
    A = (2 * np.pi ** 1.5) * W
    eZ1 = (z / np.pi) ** 0.5 * (d - 1)
    eZ2 = (1 - z) ** (0.5 * (N_K - 1))
    tau = (g * A / (2 * np.pi)) * eZ1 * eZ2
    Psing = 1 - (1 - z) ** (0.5 * N_K)
    return 1 - Psing * np.exp(-tau)


def lomb_scargle_simple(t, y, dy, **kwargs):
    """One light curve, synchronously (cuvarbase/lombscargle.py:1187-1204;
    the reference passes weights where dy is expected, this passes dy)."""
    proc = LombScargleAsyncProcess()
    results = proc.run([(t, y, dy)], **kwargs)
    freqs, powers = results[0]
    proc.finish()
    return freqs, powers
