"""The packing autotuner (whale.jl_gb300/autotune.py) without a device: its knobs
reach the packer and change the layout, out-of-range values are refused, and
the coordinate descent finds the optimum of a known cost."""
import ctypes

import numpy as np
import pytest


def _tasks(W, wm, ccds):
    from whale_gb300 import _native as N

    arr = (ctypes.c_void_p * len(ccds))(*[c._h for c in ccds])
    n = N.i64()
    N.check(N.lib().wg_pack_tasks(wm._struct.h, arr, len(ccds), 1, None, 0, ctypes.byref(n)))
    out = np.zeros(12 * n.value, np.int32)
    N.check(N.lib().wg_pack_tasks(wm._struct.h, arr, len(ccds), 1, out.ctypes.data_as(N.P_i32), out.size,
                                  ctypes.byref(n)))
    return out.reshape(-1, 12)


def test_knobs_reach_the_packer(W):
    from whale_gb300 import autotune as tune, synth

    wl = synth.config1(n_families=120)
    wm, ccds = wl.model, wl.ccds()
    base = _tasks(W, wm, ccds)
    with tune.packing(tune.DEFAULTS):
        assert np.array_equal(_tasks(W, wm, ccds), base)  # the defaults are the library's
    with tune.packing({"target_ops": 960}):
        wide = _tasks(W, wm, ccds)
    assert len(wide) < len(base)  # more families per task, fewer tasks
    with tune.packing({"target_j": 5}):
        deep = _tasks(W, wm, ccds)
    assert np.mean(deep[:, 4][deep[:, 4] > 0]) > np.mean(base[:, 4][base[:, 4] > 0])  # deeper row programs
    with tune.packing({"root_group": 4}):
        roots = _tasks(W, wm, ccds)
    assert np.sum(roots[:, 9] > 0) >= np.sum(base[:, 9] > 0)
    with pytest.raises(W.WhaleError):
        with tune.packing({"target_j": 99}):
            _tasks(W, wm, ccds)
    assert np.array_equal(_tasks(W, wm, ccds), base)  # the environment is restored


def test_malformed_knob_is_refused(W, monkeypatch):
    from whale_gb300 import synth

    wl = synth.config0(n_families=4)
    monkeypatch.setenv("WG_PACK_TARGET_OPS", "480x")
    with pytest.raises(W.WhaleError, match="not an integer"):
        _tasks(W, wl.model, wl.ccds())


def test_descent_finds_the_optimum_of_a_known_cost(W):
    from whale_gb300 import autotune as tune

    target = {"target_ops": 720, "target_j": 2, "root_group": 8, "heavy_ops": 2048}

    def cost(s):
        return 1.0 + sum(abs(np.log(s[k] / target[k])) for k in target)

    best, batch, log = tune.tune(None, [], measure=cost)
    assert best == target and batch is None
    assert log[0][0] == tune.DEFAULTS and min(ms for _, ms in log) == cost(target)
