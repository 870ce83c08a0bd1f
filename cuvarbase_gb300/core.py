"""Asynchronous-process base class (mirrors cuvarbase/core.py:13-56)."""
from __future__ import annotations

from . import _lib


class GPUAsyncProcess:
    """Base of the GPU processes: owns CUDA streams and library handles.

    Keyword arguments as in the reference: ``nstreams``, ``device``,
    ``reader`` and ``function_kwargs``.  Unlike the reference, ``device``
    selects the GPU the handles run on.
    """

    def __init__(self, *args, **kwargs):
        self.reader = kwargs.get('reader', None)
        self.nstreams = kwargs.get('nstreams', None)
        self.function_kwargs = kwargs.get('function_kwargs', {})
        self.device = kwargs.get('device', 0)
        self.streams = []
        self.gpu_data = []
        self.results = []
        self._adjust_nstreams = self.nstreams is None
        self._handles = {}
        if self.nstreams is not None:
            self._create_streams(self.nstreams)
        self.prepared_functions = {}

    def _create_streams(self, n):
        for _ in range(n):
            self.streams.append(_lib.Stream())

    def _stream(self):
        if not self.streams:
            self._create_streams(1)
        return self.streams[0]

    def _handle(self, sigma, m, precision=_lib.PREC_MIXED, workspace_bytes=0):
        key = (float(sigma), int(m), int(precision))
        h = self._handles.get(key)
        if h is None:
            h = _lib.Handle(sigma=sigma, m=m, device=self.device,
                            workspace_bytes=workspace_bytes, precision=precision)
            self._handles[key] = h
        return h

    def _compile_and_prepare_functions(self, **kwargs):
        """Kernels are compiled ahead of time into libcuvgls.so; this only
        loads the library (kept for API compatibility)."""
        _lib.load()

    def run(self, *args, **kwargs):
        raise NotImplementedError()

    def finish(self, timeout_ms=-1):
        """Synchronise every stream this process used (cuvarbase/core.py:37-40).

        With ``timeout_ms >= 0`` a stuck stream raises TimeoutError instead
        of blocking forever.
        """
        for h in self._handles.values():
            for s in (self.streams or [None]):
                h.sync(None if s is None else s.ptr, timeout_ms)

    def batched_run(self, data, batch_size=10, **kwargs):
        """run() on consecutive batches of ``batch_size`` light curves, with a
        finish() after each (cuvarbase/core.py:42-56)."""
        nsubmit = 0
        results = []
        while nsubmit < len(data):
            batch = []
            while len(batch) < batch_size and nsubmit < len(data):
                batch.append(data[nsubmit])
                nsubmit += 1
            res = self.run(batch, **kwargs)
            self.finish()
            results.extend(res)
        return results
