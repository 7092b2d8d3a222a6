"""Warp-uniform program columns, host side: the packer checks every entry of
every program against its column's kind (a product column holds products or
idle lanes, a finalize column no product, a partial-sum column only
partial-sum stores) and fails the pack otherwise.  Packing gradient batches
under settings that change the bundles (program depth, level depth, the
warp-combine threshold, 128- or 256-thread tasks) exercises that check; the
task layout itself does not depend on the combine threshold."""
import ctypes
import os

import numpy as np
import pytest


def _tasks(wm, ccds, flags):
    from whale_gb300 import _native as N

    arr = (ctypes.c_void_p * len(ccds))(*[c._h for c in ccds])
    k = N.i64()
    N.check(N.lib().wg_pack_tasks(wm._struct.h, arr, len(ccds), flags, None, 0, ctypes.byref(k)))
    out = np.zeros(12 * k.value, np.int32)
    N.check(N.lib().wg_pack_tasks(wm._struct.h, arr, len(ccds), flags, out.ctypes.data_as(N.P_i32), out.size,
                                  ctypes.byref(k)))
    return out.reshape(-1, 12)


@pytest.mark.parametrize("env", [
    {},
    {"WG_PACK_COMB_WARP": "2"},
    {"WG_PACK_COMB_WARP": "0"},
    {"WG_PACK_TARGET_J": "2", "WG_PACK_LEVEL_J": "1"},
    {"WG_PACK_TARGET_J": "5", "WG_PACK_LEVEL_J": "6"},
    {"WG_PACK_HEAVY_OPS": "64"},
])
def test_columns_fit_their_kind(W, env):
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        for wl in (synth.config1(n_families=120), synth.config0(n_families=40)):
            wm, ccds = wl.model, wl.ccds()
            wm.load()
            t = _tasks(wm, ccds, N.BATCH_GRAD)  # raises if an entry does not fit its column
            assert len(t) > 0
            # lanes are whole warps; program depths are positive where there are lanes
            for J, lanes in ((t[:, 4], t[:, 5]), (t[:, 6], t[:, 7]), (t[:, 8], t[:, 9])):
                assert np.all(lanes % 32 == 0)
                assert np.all((lanes == 0) | (J > 0))
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def test_combine_threshold_keeps_the_layout(W):
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    wl = synth.config1(n_families=120)
    wm, ccds = wl.model, wl.ccds()
    wm.load()
    base = _tasks(wm, ccds, N.BATCH_GRAD)
    os.environ["WG_PACK_COMB_WARP"] = "2"
    try:
        warp = _tasks(wm, ccds, N.BATCH_GRAD)
    finally:
        os.environ.pop("WG_PACK_COMB_WARP", None)
    assert np.array_equal(base, warp)
