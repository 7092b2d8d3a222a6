"""Per-branch checkpoint/recompute on the device: a gradient batch whose
adjoint recomputes each height level's DP tables from the children's top rows
gives the same log-likelihoods and gradients as the batch that keeps every
table (the recomputation runs the same forward kernel on the same inputs),
on config-1 families, on 40-taxon config-4 families whose widest rows live in
device memory (and against the oracle there), and when a small table budget
makes the batch choose the layout by itself."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _close(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0), initial=0.0)


def _same(W, wm, full, ck):
    t0, p0, *g0 = full.grad_nodes(wm)
    t1, p1, *g1 = ck.grad_nodes(wm)
    fin = np.isfinite(p0)
    assert np.array_equal(np.isneginf(p0), np.isneginf(p1))
    assert _close(p1[fin], p0[fin]) <= TOL
    assert t1 == pytest.approx(t0, rel=TOL)
    for a, b in zip(g1, g0):
        assert _close(a, b) <= TOL
    # a forward-only evaluation of the checkpointed batch keeps no tables
    assert ck.logpdf(wm) == pytest.approx(t0, rel=TOL)


def test_checkpoint_config1_matches_full_tables(W):
    from whale_gb300 import synth

    wl = synth.config1(n_families=400)
    wm, ccds = wl.model, wl.ccds()
    full = W.Batch(wm, ccds, grad=True)
    ck = W.Batch(wm, ccds, grad=True, checkpoint=True)
    c, k, tf, tk = ck.tables_layout()
    assert k == c and tk < tf / 2
    assert full.tables_layout()[1] == 0
    assert ck.device_bytes < full.device_bytes
    _same(W, wm, full, ck)


def test_checkpoint_config4_against_oracle(W, O):
    from whale_gb300 import synth

    wl = synth.config4(indices=list(range(120)))
    wm, ccds = wl.model, wl.ccds()
    full = W.Batch(wm, ccds, grad=True)
    ck = W.Batch(wm, ccds, grad=True, checkpoint=True)
    _same(W, wm, full, ck)
    # small families against the oracle: log L and the duals' gradient
    n = np.array([c.n_clades for c in ccds])
    pick = np.where(n <= 300)[0][:25]
    sub = W.Batch(wm, [ccds[i] for i in pick], grad=True, checkpoint=True)
    tot, per, *_ = sub.grad_nodes(wm)
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt)
    occ = [O.OracleCCD(om, wl.ale[i]) for i in pick]
    r = wm.rates
    otot, oper = om.logpdf(occ, r.λ, r.μ, q=r.q, eta=r.η)
    assert np.max(np.abs(per - oper) / np.abs(oper)) <= 1e-10
    from whale_gb300.core import map_gradient

    _, _, dl, dm, dq, de = sub.grad_nodes(wm)
    g = map_gradient(wm, dl, dm, dq, de)
    flat = np.concatenate([g["λ"], g["μ"], g["q"], [g["η"]]])
    _, og = om.gradient(occ, r.λ, r.μ, q=r.q, eta=r.η)
    assert _close(flat, og) <= 1e-8


def test_checkpoint_chosen_by_table_budget(W, monkeypatch):
    from whale_gb300 import synth

    wl = synth.config1(seed=3, n_families=300)
    wm, ccds = wl.model, wl.ccds()
    full = W.Batch(wm, ccds, grad=True)
    c, k, tf, tk = full.tables_layout()
    assert k == 0 and tk == tf
    # a budget below the stored tables: the largest classes switch over
    monkeypatch.setenv("WG_TABLE_BUDGET_BYTES", str(8 * tf // 2))
    auto = W.Batch(wm, ccds, grad=True)
    c2, k2, tf2, tk2 = auto.tables_layout()
    assert c2 == c and 1 <= k2 and tf2 == tf and 8 * tk2 <= 8 * tf // 2
    _same(W, wm, full, auto)
