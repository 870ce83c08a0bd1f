"""Host-side logic that needs no GPU: utilities against the reference's
outputs, the C ABI's exported symbols and the grid planner."""
import ctypes
import os
import re

import numpy as np
import pytest

from cuvarbase_gb300 import utils
from cuvarbase_gb300.lombscargle import check_k0, fap_baluev, get_k0

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_autofrequency_matches_reference(golden):
    t = golden["ls_t_norm"]
    np.testing.assert_array_equal(utils.autofrequency(t), golden["af_default"])
    np.testing.assert_array_equal(
        utils.autofrequency(t, minimum_frequency=2.0, maximum_frequency=40.0,
                            samples_per_peak=5), golden["af_minmax"])
    np.testing.assert_array_equal(utils.autofrequency(t, samples_per_peak=1, nyquist_factor=2),
                                  golden["af_spp1"])
    np.testing.assert_array_equal(utils.autofrequency(t, nyquist_factor=3, samples_per_peak=3),
                                  golden["ls_freqs"])


def test_weights_and_normalize_match_reference(golden):
    np.testing.assert_array_equal(utils.weights(golden["ls_dy_raw"]), golden["ls_weights"])
    (tn, yn, dyn), = utils.normalize_light_curves(
        [(golden["ls_t_raw"], golden["ls_y_raw"], golden["ls_dy_raw"])])
    np.testing.assert_array_equal(tn, golden["ls_t_norm"])
    np.testing.assert_array_equal(yn, golden["ls_y_norm"])
    np.testing.assert_array_equal(dyn, golden["ls_dy_raw"])


def test_fap_baluev_matches_reference(golden):
    z = golden["fap_z"]
    fap = fap_baluev(golden["ls_t_raw"], golden["ls_dy_raw"], z, float(golden["ls_freqs"].max()))
    np.testing.assert_allclose(fap, golden["fap"], rtol=1e-13, atol=0)


def test_k0_helpers():
    df = 0.01
    f = df * (3 + np.arange(10))
    assert get_k0(f) == 3
    check_k0(f)
    with pytest.raises(AssertionError):
        check_k0(f + 0.3 * df, k0=3)


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "cuvgls.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*\**\s*(cuvgls_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(lib):
    names = _declared_functions()
    assert len(names) >= 15
    from cuvarbase_gb300 import _lib
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, n
    assert lib.cuvgls_version() == 1000


def test_struct_layouts_match_header():
    """ctypes mirrors of the header structs have the C sizes."""
    from cuvarbase_gb300 import _lib
    assert ctypes.sizeof(_lib.Opts) == 32
    assert ctypes.sizeof(_lib.Curve) == 80
    assert ctypes.sizeof(_lib.GlsInput) == 72
    assert ctypes.sizeof(_lib.NfftCurve) == 48
    assert ctypes.sizeof(_lib.NfftInput) == 48
    assert ctypes.sizeof(_lib.GridCurve) == 56
    assert ctypes.sizeof(_lib.GridFinCurve) == 72
    assert ctypes.sizeof(_lib.RawCurve) == 48
    assert ctypes.sizeof(_lib.RawInput) == 72
    assert ctypes.sizeof(_lib.ServerOpts) == 80


@pytest.mark.parametrize("nf", [1, 7, 450, 1000, 20000, 50000, 100000, 215443, 1000000])
def test_planner_sizes(lib, nf):
    from cuvarbase_gb300 import _lib
    G, G1, G2 = _lib.plan_nf(nf, 2.0, 8)
    assert G == G1 * G2
    assert G >= 2 * nf and G >= 256
    for L in (G1, G2):
        x = L
        for p in (2, 3, 5):
            while x % p == 0:
                x //= p
        assert x == 1 and L % 8 == 0 and L <= 2048
    assert G <= max(1.3 * 2 * nf + 64, 1024)


def test_planner_rejects_oversized(lib):
    from cuvarbase_gb300 import _lib
    with pytest.raises(ValueError):
        _lib.plan_nf(5_000_000, 2.0, 8)
    with pytest.raises(ValueError):
        _lib.plan_nf(100, 0.5, 8)


def test_library_error_paths_without_gpu(lib):
    """Invalid arguments are rejected before any device work."""
    assert lib.cuvgls_create(None, None) == -1
    assert lib.cuvgls_destroy(None) == -1
    assert lib.cuvgls_sync(None, None, 0) == -1
    # plan queries and the grid-shape tuner's entry points
    assert lib.cuvgls_plan_window(None, 1000, None, None) == -1
    assert lib.cuvgls_plan_shapes(None, 1000, 0, None, None, None) == -1
    assert lib.cuvgls_plan_pin(None, 1000, 320, 400) == -1


def test_es_window_plan_shapes(lib):
    """The autotuner's ES candidate (sigma 1.28, m = 5) on the grid shapes
    of least measured cost, without a GPU (cuvgls_plan_nf)."""
    from cuvarbase_gb300 import _lib
    for nf, shape in [(10000, (160, 80)), (20000, (160, 160)), (50000, (160, 400)),
                      (100000, (320, 400)), (200000, (640, 400)), (1000000, (1024, 1280))]:
        G, G1, G2 = _lib.plan_nf(nf, 1.28, 5)
        assert (G1, G2) == shape and G == G1 * G2 and G >= 1.28 * nf


def test_autotune_rejects_bad_input_before_device_work():
    from cuvarbase_gb300.tune import autotune

    class NoDevice:      # any device call would fail the test
        def __getattr__(self, name):
            raise AssertionError(f"device touched: {name}")

    t = np.linspace(0, 10, 50)
    curve = (t, np.sin(t), np.full(50, 0.1))
    with pytest.raises(ValueError):
        autotune(NoDevice(), [], np.arange(1, 101) * 0.01)
    with pytest.raises(ValueError):          # one grid per curve, all the same length
        autotune(NoDevice(), [curve, curve], [np.arange(1, 101) * 0.01, np.arange(1, 51) * 0.01])
    with pytest.raises(ValueError):
        autotune(NoDevice(), [curve, curve], [np.arange(1, 101) * 0.01])
