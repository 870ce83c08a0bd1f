"""Run-time grid-shape tuner (cuvgls_plan_shapes / cuvgls_plan_pin,
cuvarbase_gb300.tune): the shapes the planner weighs, pinning and its
validation, and a tuned plan that still matches the FP64 oracle."""
import numpy as np
import pytest

from test_gpu_gls import cfg2_curve, oracle_P

pytestmark = pytest.mark.gpu

NF = 100_000


def _data(seed, n):
    rng = np.random.default_rng(seed)
    data, grids = [], []
    for _ in range(n):
        t, y, dy, _ = cfg2_curve(rng)
        data.append((t, y, dy))
        grids.append((1 + np.arange(NF)) / (5 * (t.max() - t.min())))
    return data, grids


def test_shapes_pin_and_validation():
    from cuvarbase_gb300 import _lib
    h = _lib.Handle(sigma=-1.0, m=8)
    try:
        shapes = h.plan_shapes(NF)
        assert shapes[0] == (320, 400) and len(shapes) >= 4
        assert all(G1 * G2 >= 1.28 * NF for G1, G2 in shapes)
        assert h.plan(NF)[1:3] == (320, 400)
        h.plan_pin(NF, 160, 800)
        assert h.plan(NF)[1:3] == (160, 800)
        assert h.plan(NF - 1)[1:3] == (320, 400)      # pins are per frequency count
        with pytest.raises(ValueError):
            h.plan_pin(NF, 16, 16)                    # far too small a grid
        assert h.plan(NF)[1:3] == (160, 800)           # a rejected pin changes nothing
        h.plan_pin(NF, 0, 0)
        assert h.plan(NF)[1:3] == (320, 400)
    finally:
        h.close()


def test_autotune_pins_the_fastest_and_stays_exact(oracle):
    from cuvarbase_gb300.lombscargle import LombScargleAsyncProcess
    data, grids = _data(3003, 200)
    p = LombScargleAsyncProcess(sigma="auto")
    res = p.autotune(data, grids, steps=2, max_shapes=4)
    assert len(res) == 4 and res[0]["ms"] <= res[-1]["ms"]
    h = p._gls_handle(NF)
    assert h.plan(NF)[1:3] == (res[0]["G1"], res[0]["G2"])
    out = p.run(data[:6], freqs=grids[:6])
    p.finish()
    for (t, y, dy), fr, (f, P) in zip(data[:6], grids[:6], out):
        Pref = oracle_P(oracle, t, y, dy, fr)
        assert np.abs(P - Pref).max() <= 3e-5
        assert int(np.argmax(P)) == int(np.argmax(Pref))
