"""NowhereExtinctCondition on the device (src/condition.jl:31-36,
src/bdputil.jl:84-135): the 2^L-term pgf and its adjoint against the oracle,
on trees that take every layout of the kernels (one root tile, 128 tiles,
512 tiles with the reverse sweep's sums in device memory, WGD nodes), and
inside batched evaluations (value, gradient, rates changed between calls,
conditions switched on one batch)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GREL = 1e-8


def _close(g, ref):
    g, ref = np.asarray(g), np.asarray(ref)
    return np.max(np.abs(g - ref) / np.maximum(np.abs(ref), 1.0))


def _extree_wgd(W):
    t = W.extree()
    W.insertnode(W.getlca(t, "ATHA", "ATHA"), name="wgd_1")
    W.insertnode(W.getlca(t, "ATHA", "ATRI"), name="wgd_2")
    return t


def _caterpillar(W, n, wgd=True):
    nwk = "A:1"
    for c in "BCDEFGHIJKLMNOPQRSTUV"[: n - 1]:
        nwk = f"({nwk},{c}:1):0.5"
    t = W.readnw(nwk[:-4] + ";")
    if wgd:
        W.insertnode(W.getlca(t, "A", "A"), name="wgd_1")
        W.insertnode(W.getlca(t, "A", "C"), name="wgd_2")
    return t


def _model(W, t, dt, seed, m0=-1.5, m1=-1.7):
    rng = np.random.default_rng(seed)
    nw = sum(1 for x in W.postwalk(t) if x.name.startswith("wgd"))
    n = len(W.postwalk(t)) - nw
    lam, mu, q = rng.normal(m0, 0.4, n), rng.normal(m1, 0.4, n), rng.uniform(0.1, 0.6, nw)
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=q, η=0.7), t, dt, condition=W.NowhereExtinctCondition(t))
    return wm, lam, mu, q


def _cases(W):
    from whale_gb300 import synth

    t1 = synth.config1(n_families=2).model.tree
    return [
        ("extree+2wgd", _extree_wgd(W), 0.05, -1.5, -1.7),  # 13 leaves: one root tile
        ("config1-17", t1, 0.02, -1.5, -1.7),  # 17 leaves: 128 root tiles
        ("caterpillar-15", _caterpillar(W, 15), 0.1, -3.0, -3.2),  # 512 tiles, sums in device memory
    ]


def test_value_against_oracle(W, O):
    for name, t, dt, m0, m1 in _cases(W):
        wm, lam, mu, q = _model(W, t, dt, 3, m0, m1)
        om = O.OracleModel(W.nwstr(t), dt, condition="nowhere")
        ref = om.condition(lam, mu, q=q, eta=0.7)
        v = W.nowhere_condition(wm)
        assert np.isfinite(ref), name
        assert v == pytest.approx(ref, rel=1e-11), name
        assert v == pytest.approx(W.condition(wm), rel=1e-10), name  # the library's host version
        # the value does not depend on whether the adjoint runs
        v2, g = W.nowhere_condition(wm, grad=True)
        assert v2 == v, name


def test_even_leaf_count_is_minus_inf_like_the_reference(W, O):
    # treepgf_allbinary_sign gives x = 1 the sign -1: with an even number of
    # leaves the reference's sum is 2 - P, outside (0, 1), and the condition
    # is -Inf (src/condition.jl:31-36); the device reproduces it
    t = _caterpillar(W, 6, wgd=False)
    wm, lam, mu, q = _model(W, t, 0.1, 2, -3.0, -3.2)
    om = O.OracleModel(W.nwstr(t), 0.1, condition="nowhere")
    assert om.condition(lam, mu, q=q, eta=0.7) == -np.inf
    v, g = W.nowhere_condition(wm, grad=True)
    assert v == -np.inf
    assert not np.any(g["λ"]) and g["η"] == 0.0


def test_batch_gradient_against_oracle_duals(W, O):
    # the batched evaluation forks the condition beside the DP; its gradient
    # joins the DP's on the host.  17-leaf tree: the multi-tile root.
    from whale_gb300 import synth

    wl = synth.config1(n_families=40)
    ccds = wl.ccds()
    keep = [i for i, c in enumerate(ccds) if c.n_clades <= 300][:12]
    t = wl.model.tree
    rng = np.random.default_rng(8)
    n = len(wl.model.rates.λ)
    lam, mu = rng.normal(-1.6, 0.3, n), rng.normal(-1.8, 0.3, n)
    q = np.asarray(wl.model.rates.q)
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=q, η=0.69), t, wl.model.Δt,
                      condition=W.NowhereExtinctCondition(t))
    ccds = [ccds[i] for i in keep]
    tot, gd = W.logpdf_gradient(wm, ccds)
    g = np.concatenate([gd["λ"], gd["μ"], gd["q"], [gd["η"]]])
    om = O.OracleModel(W.nwstr(t), wl.model.Δt, condition="nowhere")
    occ = [O.OracleCCD(om, wl.ale[i]) for i in keep]
    otot, og = om.gradient(occ, lam, mu, q=q, eta=0.69)
    assert tot == pytest.approx(otot, rel=1e-10)
    assert _close(g, og) <= GREL


def test_batch_rates_change_and_condition_switch(W, O, ex1_tree, ex1_files):
    # one batch: new rates every call (the captured sequence re-stages the
    # condition's coefficients) and the condition switched between calls
    t = W.readnw(ex1_tree)
    r0 = W.DLWGD(λ=np.full(17, -1.0), μ=np.full(17, -1.2), q=[0.3, 0.4], η=0.7)
    wm_n = W.WhaleModel(r0, t, 0.05, condition=W.NowhereExtinctCondition(t))
    wm_r = W.WhaleModel(r0, t, 0.05)
    ccds = W.read_ale(os.path.dirname(ex1_files[0]), wm_n)
    b = W.Batch(wm_n, ccds)
    om_n = O.OracleModel(ex1_tree, 0.05, condition="nowhere")
    om_r = O.OracleModel(ex1_tree, 0.05)
    occ_n = O.read_ale_files(om_n, ex1_files)
    occ_r = O.read_ale_files(om_r, ex1_files)
    rng = np.random.default_rng(11)
    for step in range(5):
        lam, mu = rng.normal(-0.8, 0.3, 17), rng.normal(-1.0, 0.3, 17)
        nowhere = step % 2 == 0
        wm = (wm_n if nowhere else wm_r)(W.DLWGD(λ=lam, μ=mu, q=[0.3, 0.4], η=0.7))
        tot = b.logpdf(wm)
        om, occ = (om_n, occ_n) if nowhere else (om_r, occ_r)
        otot, _ = om.logpdf(occ, lam, mu, q=[0.3, 0.4], eta=0.7)
        assert tot == pytest.approx(otot, rel=1e-10), step
