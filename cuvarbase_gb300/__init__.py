"""cuvarbase_gb300 — GB300-native generalized Lomb-Scargle and adjoint NFFT.

Drop-in for the GLS / NFFT path of cuvarbase: the modules ``lombscargle``,
``cunfft``, ``core`` and ``utils`` keep the reference's public names and
arguments.  The compute runs in libcuvgls.so (hand-written sm_103a CUDA,
C ABI in include/cuvgls.h); importing the package does not touch the GPU.
"""
__version__ = "0.3.0+gb300.1"

from . import utils  # noqa: F401
