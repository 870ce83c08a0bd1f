"""ctypes bindings of libcuvgls.so (the C ABI declared in include/cuvgls.h).

The library is built in-tree (``cuvarbase_gb300/build.py``).  There is no
fallback: if the shared library is missing or cannot be loaded, every GPU
entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcuvgls.so")

# status codes
OK = 0
EINVAL = -1
ENOMEM = -2
EBUDGET = -3
ETIMEOUT = -4
ECUDA = -5
ENOTSUP = -6
EDEVICE = -7
ECLOSED = -8

HOST_INPUT = 1
HOST_OUTPUT = 2

MODE_STANDARD = 0
MODE_FLOATING_MEAN = 1
MODE_WINDOW = 2

PREC_MIXED = 0
PREC_FP32 = 1

WIN_GAUSS = 0
WIN_ES = 1

DEVERR_NONFINITE = 1
DEVERR_TIMEOUT = 2
DEVERR_BINNING = 4

STAGES = ("prep", "pass1", "pass2", "direct", "spread")

i32, i64, f64, f32 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_float
vp = ctypes.c_void_p


class Opts(ctypes.Structure):
    _fields_ = [("sigma", f64), ("m", i32), ("device", i32),
                ("workspace_bytes", i64), ("precision", i32), ("chunk_mb", i32)]


class Curve(ctypes.Structure):
    _fields_ = [("pt_off", i64), ("n", i64), ("nf", i64), ("k0", i64),
                ("df", f64), ("yy", f64), ("ybar", f64), ("yw_sum", f64),
                ("w_sum", f64), ("out_off", i64)]


class GlsInput(ctypes.Structure):
    _fields_ = [("n_curves", i32), ("mode", i32), ("curves", vp), ("t", vp),
                ("yw", vp), ("w", vp), ("reg", f32 * 3), ("flags", i32),
                ("n_points_total", i64), ("n_out_total", i64)]


class RawCurve(ctypes.Structure):
    _fields_ = [("pt_off", i64), ("n", i64), ("nf", i64), ("k0", i64),
                ("df", f64), ("out_off", i64)]


class RawInput(ctypes.Structure):
    _fields_ = [("n_curves", i32), ("mode", i32), ("curves", vp), ("t", vp),
                ("y", vp), ("dy", vp), ("reg", f32 * 3), ("flags", i32),
                ("n_points_total", i64), ("n_out_total", i64)]


class NfftCurve(ctypes.Structure):
    _fields_ = [("pt_off", i64), ("n", i64), ("nf", i64), ("f0", f64),
                ("df", f64), ("out_off", i64)]


class NfftInput(ctypes.Structure):
    _fields_ = [("n_curves", i32), ("flags", i32), ("curves", vp), ("t", vp),
                ("y", vp), ("n_points_total", i64), ("n_out_total", i64)]


class GridCurve(ctypes.Structure):
    _fields_ = [("pt_off", i64), ("n", i64), ("ng", i64), ("tmin", f64),
                ("tmax", f64), ("spp", f64), ("out_off", i64)]


class GridFinCurve(ctypes.Structure):
    _fields_ = [("grid_off", i64), ("ng", i64), ("nf", i64), ("tmin", f64), ("tmax", f64),
                ("spp", f64), ("f0", f64), ("b", f64), ("out_off", i64)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("sigma", f64), ("m", i32), ("device", i32), ("hbm_budget", i64),
                ("max_batch", i32), ("inflight", i32), ("precision", i32), ("mode", i32),
                ("reg", f32), ("reserved", i32), ("warm_nf_min", i64), ("warm_nf_max", i64),
                ("stage_points", i64), ("stage_results", i64)]


# name -> (restype, argtypes); every symbol include/cuvgls.h declares
SIGNATURES = {
    "cuvgls_version": (ctypes.c_int, []),
    "cuvgls_create": (ctypes.c_int, [ctypes.POINTER(vp), ctypes.POINTER(Opts)]),
    "cuvgls_destroy": (ctypes.c_int, [vp]),
    "cuvgls_gls_batch": (ctypes.c_int, [vp, ctypes.POINTER(GlsInput), vp, vp]),
    "cuvgls_gls_direct_batch": (ctypes.c_int, [vp, ctypes.POINTER(GlsInput), vp, vp]),
    "cuvgls_gls_best": (ctypes.c_int, [vp, ctypes.POINTER(GlsInput), vp, vp, vp]),
    "cuvgls_gls_raw": (ctypes.c_int, [vp, ctypes.POINTER(RawInput), vp, vp, vp, vp]),
    "cuvgls_gls_plan_create": (ctypes.c_int, [vp, ctypes.POINTER(RawInput), vp, vp, vp,
                                              ctypes.POINTER(vp)]),
    "cuvgls_gls_plan_launch": (ctypes.c_int, [vp, vp]),
    "cuvgls_gls_plan_destroy": (ctypes.c_int, [vp]),
    "cuvgls_nfft_adjoint_batch": (ctypes.c_int, [vp, ctypes.POINTER(NfftInput), vp, vp]),
    "cuvgls_spread_ref": (ctypes.c_int, [vp, i32, vp, vp, vp, i64, i64, i32, vp, vp]),
    "cuvgls_mhgls_direct": (ctypes.c_int, [vp, i32, vp, vp, vp, i64, vp, i64, f64, f64, vp, vp,
                                           vp, i32, vp, vp]),
    "cuvgls_nfft_adjoint_fp64": (ctypes.c_int, [vp, ctypes.POINTER(NfftInput), vp, vp, vp]),
    "cuvgls_nfft_from_grid": (ctypes.c_int, [vp, i32, vp, vp, i64, i64, i32, vp, vp]),
    "cuvgls_sync": (ctypes.c_int, [vp, vp, i32]),
    "cuvgls_device_flags": (ctypes.c_int, [vp, ctypes.POINTER(i32)]),
    "cuvgls_last_error": (ctypes.c_char_p, [vp]),
    "cuvgls_plan": (ctypes.c_int, [vp, i64, ctypes.POINTER(i64), ctypes.POINTER(i32),
                                   ctypes.POINTER(i32), ctypes.POINTER(i32)]),
    "cuvgls_plan_window": (ctypes.c_int, [vp, i64, ctypes.POINTER(i32), ctypes.POINTER(f64)]),
    "cuvgls_plan_shapes": (ctypes.c_int, [vp, i64, i32, ctypes.POINTER(i32), ctypes.POINTER(i32),
                                          ctypes.POINTER(i32)]),
    "cuvgls_plan_pin": (ctypes.c_int, [vp, i64, i32, i32]),
    "cuvgls_plan_nf": (ctypes.c_int, [f64, i32, i64, ctypes.POINTER(i64),
                                      ctypes.POINTER(i32), ctypes.POINTER(i32)]),
    "cuvgls_batch_bytes": (ctypes.c_int, [vp, i32, vp, vp, i32, ctypes.POINTER(i64)]),
    "cuvgls_warm": (ctypes.c_int, [vp, i64, i64, i32]),
    "cuvgls_profile": (ctypes.c_int, [vp, i32]),
    "cuvgls_profile_read": (ctypes.c_int, [vp, ctypes.POINTER(i64), ctypes.POINTER(f64)]),
    "cuvgls_gls_noalloc": (ctypes.c_int, [f64, i32, ctypes.POINTER(GlsInput), vp, vp, vp,
                                          ctypes.c_char_p, i32]),
    "cuvgls_stream_create": (ctypes.c_int, [ctypes.POINTER(vp)]),
    "cuvgls_stream_destroy": (ctypes.c_int, [vp]),
    "cuvgls_host_alloc": (ctypes.c_int, [ctypes.POINTER(vp), i64]),
    "cuvgls_host_free": (ctypes.c_int, [vp]),
    "cuvgls_server_create": (ctypes.c_int, [ctypes.POINTER(vp), ctypes.POINTER(ServerOpts)]),
    "cuvgls_server_submit": (ctypes.c_int, [vp, i64, vp, vp, vp, i64, i64, f64, i64]),
    "cuvgls_server_poll": (ctypes.c_int, [vp, i32, i32, vp, vp, vp, vp, vp]),
    "cuvgls_server_release": (ctypes.c_int, [vp, i64]),
    "cuvgls_server_release_many": (ctypes.c_int, [vp, vp, i32]),
    "cuvgls_server_slot_buffer": (ctypes.c_int, [vp, i32, ctypes.POINTER(vp),
                                                 ctypes.POINTER(i64)]),
    "cuvgls_server_request_bytes": (ctypes.c_int, [vp, i64, i64, ctypes.POINTER(i64)]),
    "cuvgls_server_stats": (ctypes.c_int, [vp, vp]),
    "cuvgls_server_shutdown": (ctypes.c_int, [vp]),
    "cuvgls_server_destroy": (ctypes.c_int, [vp]),
}

_lib = None
_lock = threading.Lock()


class CuvglsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cuvgls error {code}: {msg}")
        self.code = code


def load(path: str = LIB_PATH):
    """Load libcuvgls.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise ImportError(
                    f"{path} is missing: build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'` "
                    "or `python cuvarbase_gb300/build.py`")
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def raise_for(code: int, handle=None, what: str = ""):
    """Map a status code to the exception the reference API would raise."""
    if code == OK:
        return
    msg = what
    if handle is not None:
        try:
            m = load().cuvgls_last_error(handle)
            if m:
                msg = (what + ": " if what else "") + m.decode()
        except Exception:  # pragma: no cover - diagnostics only
            pass
    if code in (EINVAL, ENOTSUP):
        raise ValueError(f"cuvgls: {msg} (status {code})")
    if code in (ENOMEM, EBUDGET):
        raise MemoryError(f"cuvgls: {msg} (status {code})")
    if code == ETIMEOUT:
        raise TimeoutError(f"cuvgls: {msg}")
    raise CuvglsError(code, msg)


class Handle:
    """Owns one cuvgls handle (one device, one sigma / m / precision)."""

    def __init__(self, sigma=2.0, m=8, device=0, workspace_bytes=0,
                 precision=PREC_MIXED, chunk_mb=0):
        L = load()
        o = Opts(float(sigma), int(m), int(device), int(workspace_bytes),
                 int(precision), int(chunk_mb))
        h = vp()
        rc = L.cuvgls_create(ctypes.byref(h), ctypes.byref(o))
        if rc != OK:
            raise_for(rc, None, f"cuvgls_create(sigma={sigma}, m={m}, device={device})")
        self.ptr = h
        self.sigma, self.m, self.device, self.precision = sigma, m, device, precision
        self._lib = L

    def close(self):
        if getattr(self, "ptr", None):
            self._lib.cuvgls_destroy(self.ptr)
            self.ptr = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc, what=""):
        raise_for(rc, self.ptr, what)

    def sync(self, stream=None, timeout_ms=-1):
        self.check(self._lib.cuvgls_sync(self.ptr, stream, int(timeout_ms)), "sync")

    def device_flags(self) -> int:
        f = i32()
        self.check(self._lib.cuvgls_device_flags(self.ptr, ctypes.byref(f)), "flags")
        return int(f.value)

    def profile(self, enable=True):
        self.check(self._lib.cuvgls_profile(self.ptr, 1 if enable else 0), "profile")

    def profile_read(self):
        """{stage: (launches, total ms)} since profile(True); synchronises."""
        n = (i64 * len(STAGES))()
        ms = (f64 * len(STAGES))()
        self.check(self._lib.cuvgls_profile_read(self.ptr, n, ms), "profile read")
        return {s: (int(n[i]), float(ms[i])) for i, s in enumerate(STAGES)}

    def plan(self, nf):
        G, G1, G2, m = i64(), i32(), i32(), i32()
        self.check(self._lib.cuvgls_plan(self.ptr, int(nf), ctypes.byref(G),
                                         ctypes.byref(G1), ctypes.byref(G2),
                                         ctypes.byref(m)), "plan")
        return int(G.value), int(G1.value), int(G2.value), int(m.value)

    def plan_shapes(self, nf, max_shapes=32):
        """[(G1, G2), ...] the planner weighs for nf frequencies, cheapest
        first by the measured pass costs."""
        g1, g2, n = (i32 * max_shapes)(), (i32 * max_shapes)(), i32()
        self.check(self._lib.cuvgls_plan_shapes(self.ptr, int(nf), int(max_shapes), g1, g2,
                                                ctypes.byref(n)), "plan shapes")
        return [(int(g1[i]), int(g2[i])) for i in range(min(n.value, max_shapes))]

    def plan_pin(self, nf, G1=0, G2=0):
        """Pin the grid shape of GLS bands of nf frequencies (0, 0 unpins)."""
        self.check(self._lib.cuvgls_plan_pin(self.ptr, int(nf), int(G1), int(G2)), "plan pin")

    def plan_window(self, nf):
        """("gauss" | "es", nominal sigma) of the plan for nf frequencies."""
        w, s = i32(), f64()
        self.check(self._lib.cuvgls_plan_window(self.ptr, int(nf), ctypes.byref(w),
                                                ctypes.byref(s)), "plan window")
        return ("es" if w.value == WIN_ES else "gauss"), float(s.value)


def plan_nf(nf, sigma=2.0, m=8):
    """(G, G1, G2) the library picks for nf frequencies; needs no GPU."""
    G, G1, G2 = i64(), i32(), i32()
    raise_for(load().cuvgls_plan_nf(float(sigma), int(m), int(nf), ctypes.byref(G),
                                    ctypes.byref(G1), ctypes.byref(G2)), None,
              f"plan nf={nf}")
    return int(G.value), int(G1.value), int(G2.value)


class Stream:
    """A non-blocking CUDA stream created by the library."""

    def __init__(self):
        L = load()
        s = vp()
        raise_for(L.cuvgls_stream_create(ctypes.byref(s)), None, "stream create")
        self.ptr = s
        self._lib = L

    def close(self):
        if getattr(self, "ptr", None):
            self._lib.cuvgls_stream_destroy(self.ptr)
            self.ptr = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class _View:
    """__array_interface__ holder: numpy arrays made from it keep `owner`."""

    def __init__(self, owner, addr, dt, count):
        self._owner = owner
        self.__array_interface__ = {"shape": (int(count),), "typestr": dt.str,
                                    "data": (int(addr), False), "version": 3}


class PinnedBuffer:
    """Page-locked host memory (cudaMallocHost) exposed as a numpy array."""

    def __init__(self, nbytes: int):
        import numpy as np  # local: keep module import light
        L = load()
        p = vp()
        nbytes = max(int(nbytes), 16)
        raise_for(L.cuvgls_host_alloc(ctypes.byref(p), nbytes), None, "pinned alloc")
        self.ptr = p
        self.nbytes = nbytes
        self._lib = L
        self._np = np

    def view(self, dtype, count, offset_bytes=0):
        """numpy view of the buffer; the view keeps the buffer alive."""
        np = self._np
        dt = np.dtype(dtype)
        if offset_bytes + dt.itemsize * count > self.nbytes:
            raise ValueError("view outside the pinned buffer")
        return np.asarray(_View(self, self.ptr.value + offset_bytes, dt, count))

    def close(self):
        if getattr(self, "ptr", None):
            self._lib.cuvgls_host_free(self.ptr)
            self.ptr = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
