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

    nb = {k: tune.NEIGHBOURS[k] for k in target}
    best, batch, log = tune.tune(None, [], measure=cost, neighbours=nb)
    assert {k: best[k] for k in target} == target and batch is None
    assert all(log[0][0][k] == tune.DEFAULTS[k] for k in target) and min(ms for _, ms in log) == cost(target)


def test_shape_knobs_reach_the_environment(W):
    # the size-class bounds, the per-class CTA shapes and the layout are
    # knobs too: class bounds and per-class 256-thread thresholds go to the
    # packer's environment, a class threshold of 0 follows heavy_ops
    import os

    from whale_gb300 import autotune as tune

    with tune.packing({"classes": 2, "heavy_c2": 2048, "heavy_c3": 0, "persist_ctas": 4}):
        assert os.environ["WG_CLASS_BOUNDS"] == ",".join(map(str, tune.CLASS_BOUNDS[2]))
        assert os.environ["WG_PACK_HEAVY_OPS_C2"] == "2048"
        assert "WG_PACK_HEAVY_OPS_C3" not in os.environ
        assert os.environ["WG_PERSIST_CTAS"] == "4"
    assert "WG_CLASS_BOUNDS" not in os.environ and "WG_PACK_HEAVY_OPS_C2" not in os.environ
    sh = tune.shapes({"classes": 2, "heavy_ops": 1024, "heavy_c0": 256})
    assert [x["clades"] for x in sh] == [(1, 128), (129, 512), (513, 1536), (1537, None)]
    assert sh[0]["heavy_ops"] == 256 and sh[1]["heavy_ops"] == 1024
    assert tune.shapes({"persistent": 1, "persist_ctas": 4})[0]["ctas_per_sm"] == 4
