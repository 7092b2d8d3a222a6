"""The allocation-free forward entry point (wg_logpdf_noalloc).

It serves callers that cannot allocate device memory when they evaluate the
likelihood -- hosts whose device memory belongs to another allocator or pool,
and sampler loops that must not enter the allocator between steps.  Its
scratch is one fixed device array inside the library, so it must give the
same per-family log-likelihoods as the ordinary batched entry point, call
after call, and refuse batches that need more scratch than that array holds.
This file is collected last so that a failure here leaves every other test
already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
REL = 1e-10


def _noalloc(N, b, wm, n):
    wm.load()  # slice tables of this model's rates (host side)
    per = np.zeros(n)
    tot = N.dbl()
    N.check(N.lib().wg_logpdf_noalloc(b.ctx.h, wm._struct.h, b.h, N.dptr(per), ctypes.byref(tot)))
    return tot.value, per


def test_noalloc_matches_batched_entry_point(W):
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    wl = synth.config0(seed=2, n_families=60)
    wm = wl.model
    ccds = wl.ccds()
    b = W.Batch(wm, ccds)  # device memory is set up here, before the calls under test
    ref_tot, ref_per = b.logpdf(wm, per_family=True)
    for _ in range(2):  # two calls in a row share the scratch array
        tot, per = _noalloc(N, b, wm, len(ccds))
        assert np.max(np.abs(per - ref_per) / np.abs(ref_per)) <= REL
        assert tot == pytest.approx(ref_tot, rel=REL)
    # a re-parameterised model through the same batch
    w2 = wm(W.ConstantDLWGD(λ=0.3, μ=0.25, q=[0.4], η=0.6))
    ref_tot2, ref_per2 = b.logpdf(w2, per_family=True)
    tot2, per2 = _noalloc(N, b, w2, len(ccds))
    assert np.max(np.abs(per2 - ref_per2) / np.abs(ref_per2)) <= REL
    assert tot2 == pytest.approx(ref_tot2, rel=REL)


def test_noalloc_rejects_batches_beyond_its_scratch(W):
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    wl = synth.config1(n_families=2000)
    wm = wl.model
    b = W.Batch(wm, wl.ccds())
    with pytest.raises(W.WhaleError) as ei:
        _noalloc(N, b, wm, b.n)
    assert ei.value.code == N.WG_ERANGE and "scratch" in str(ei.value)


def test_noalloc_refuses_while_an_enqueued_evaluation_is_unfetched(W):
    # an evaluation enqueued with wg_enqueue owns the batch's result buffers
    # until wg_fetch: the allocation-free call is refused meanwhile, and the
    # fetch then returns the enqueued evaluation's own results
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    wl = synth.config0(seed=5, n_families=40)
    wm = wl.model
    b = W.Batch(wm, wl.ccds())
    ref_tot, ref_per = b.logpdf(wm, per_family=True)
    L = N.lib()
    wm.load()
    N.check(L.wg_enqueue(b.ctx.h, wm._struct.h, b.h, 0))
    with pytest.raises(W.WhaleError) as ei:
        _noalloc(N, b, wm, b.n)
    assert ei.value.code == N.WG_ESTATE
    per = np.zeros(b.n)
    tot = N.dbl()
    N.check(L.wg_fetch(b.ctx.h, wm._struct.h, b.h, N.dptr(per), ctypes.byref(tot), None, None, None, None))
    assert np.array_equal(per, ref_per)
    assert tot.value == ref_tot
    # and once fetched, the call goes through
    tot2, per2 = _noalloc(N, b, wm, b.n)
    assert np.max(np.abs(per2 - ref_per) / np.abs(ref_per)) <= REL


def test_noalloc_nowhere_extinct_condition(W):
    # the total under NowhereExtinctCondition (condition on the host here, on
    # the device in wg_logpdf) agrees with the batched entry point
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    wl = synth.config0(seed=6, n_families=30)
    base = wl.model
    wm = W.WhaleModel(base.rates, base.tree, base.Δt, condition=W.NowhereExtinctCondition(base.tree))
    ccds = [W.parse_ale_text(a, wm) for a in wl.ale]
    b = W.Batch(wm, ccds)
    ref_tot, ref_per = b.logpdf(wm, per_family=True)
    for _ in range(2):
        tot, per = _noalloc(N, b, wm, b.n)
        assert np.max(np.abs(per - ref_per) / np.abs(ref_per)) <= REL
        assert tot == pytest.approx(ref_tot, rel=REL)


def test_noalloc_rows_in_device_memory(W):
    # every task forced onto the device-memory rows path: the allocation-free
    # call launches those kernel variants too
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    wl = synth.config1(seed=3, n_families=60)
    wm = wl.model
    ccds = [c for c in wl.ccds() if c.n_clades <= 600]
    b = W.Batch(wm, ccds, scratch_rows=True)
    ref_tot, ref_per = b.logpdf(wm, per_family=True)
    for _ in range(2):
        tot, per = _noalloc(N, b, wm, b.n)
        assert np.max(np.abs(per - ref_per) / np.abs(ref_per)) <= REL
        assert tot == pytest.approx(ref_tot, rel=REL)
