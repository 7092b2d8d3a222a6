"""Per-branch checkpoint/recompute of the adjoint's DP tables, host side: the
layout keeps one height level's tables at a time (every level's tasks share
a region from offset 0), so the doubles it holds are the largest level's
sum of rows x width, below the sum over all levels."""
import ctypes

import numpy as np


def _pack(W, wm, ccds, flags):
    from whale_gb300 import _native as N

    arr = (ctypes.c_void_p * len(ccds))(*[c._h for c in ccds])
    tab = N.i64()
    N.check(N.lib().wg_pack_info(wm._struct.h, arr, len(ccds), flags, None, None, ctypes.byref(tab), None, None))
    k = N.i64()
    N.check(N.lib().wg_pack_tasks(wm._struct.h, arr, len(ccds), flags, None, 0, ctypes.byref(k)))
    out = np.zeros(12 * k.value, np.int32)
    N.check(N.lib().wg_pack_tasks(wm._struct.h, arr, len(ccds), flags, out.ctypes.data_as(N.P_i32), out.size,
                                  ctypes.byref(k)))
    return tab.value, out.reshape(-1, 12)


def test_checkpoint_layout_holds_one_level(W):
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    wl = synth.config1(n_families=300)
    wm = wl.model
    ccds = wl.ccds()
    wm.load()
    nrow = np.asarray(wm._struct.nrow)
    full, tasks = _pack(W, wm, ccds, N.BATCH_GRAD)
    kept, tasks_c = _pack(W, wm, ccds, N.BATCH_GRAD | N.BATCH_CHECKPOINT)
    assert np.array_equal(tasks, tasks_c)  # the same tasks and programs
    stride = tasks[:, 2] + (tasks[:, 2] & 1)  # table rows of an even number of doubles
    per_task = nrow[tasks[:, 0]].astype(np.int64) * stride
    assert full == per_task.sum()
    levels = tasks[:, 1]
    by_level = [per_task[levels == h].sum() for h in np.unique(levels)]
    assert kept == max(by_level)
    assert kept < full / 2  # the other levels' tables are not held
    # logpdf! keeps every table: the flag does not apply with WG_BATCH_TABLES
    both, _ = _pack(W, wm, ccds, N.BATCH_GRAD | N.BATCH_TABLES | N.BATCH_CHECKPOINT)
    assert both == full


def test_persistent_layout_schedule(W):
    # the persistent layout packs every task for 128 threads and builds its
    # ticket orders and dependency lists (checked topological on the host)
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    for wl in (synth.config1(n_families=300), synth.config0(n_families=50)):
        wm, ccds = wl.model, wl.ccds()
        tab, tasks = _pack(W, wm, ccds, N.BATCH_GRAD | N.BATCH_PERSISTENT)
        assert np.all(tasks[:, 5] <= 128) and np.all(tasks[:, 9] <= 128)
        full, _ = _pack(W, wm, ccds, N.BATCH_GRAD)
        assert tab > 0 and full > 0
