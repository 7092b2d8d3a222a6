"""One persistent launch per pass (WG_BATCH_PERSISTENT): CTAs take tasks in a
topological order and wait, with a poll limit, for the tasks whose rows they
read.  Per-family log L within 1e-10 of the oracle and of the level-launch
path, gradients within 1e-8 of the oracle's duals, results bit-identical run
to run, tasks wider than shared memory taking the device-memory rows inside
the same launch (40-taxon families), and a wait that runs out (on a flag
nothing sets, with a small poll limit) coming back as WG_ECUDA with the
context still usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
REL = 1e-10


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    both = np.isneginf(a) & np.isneginf(b)
    return np.where(both, 0.0, np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def _gclose(g, ref):
    g, ref = np.asarray(g), np.asarray(ref)
    return np.max(np.abs(g - ref) / np.maximum(np.abs(ref), 1.0))


def _flat(W, wm, dl, dm, dq, de):
    from whale_gb300.core import map_gradient

    g = map_gradient(wm, dl, dm, dq, de)
    return np.concatenate([np.atleast_1d(g["λ"]), np.atleast_1d(g["μ"]), g["q"], [g["η"]]])


def test_persistent_config1_against_oracle_and_levels(W, O):
    from whale_gb300 import synth

    wl = synth.config1(n_families=400)
    wm, ccds = wl.model, wl.ccds()
    pb = W.Batch(wm, ccds, grad=True, persistent=True)
    lb = W.Batch(wm, ccds, grad=True)
    t0, p0, *g0 = pb.grad_nodes(wm)
    t1, p1, *g1 = lb.grad_nodes(wm)
    assert np.max(_rel(p0, p1)) <= 1e-12
    for a, b in zip(g0, g1):
        assert _gclose(a, b) <= 1e-10
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt)
    occ = O.parse_texts(om, wl.ale)
    r = wm.rates
    otot, oper = om.logpdf(occ, r.λ, r.μ, q=r.q, eta=r.η)
    assert np.max(_rel(p0, oper)) <= REL
    assert t0 == pytest.approx(otot, rel=REL)
    sub = list(range(0, 400, 5))
    sb = W.Batch(wm, [ccds[i] for i in sub], grad=True, persistent=True)
    _, _, dl, dm, dq, de = sb.grad_nodes(wm)
    _, og = om.gradient([occ[i] for i in sub], r.λ, r.μ, q=r.q, eta=r.η)
    assert _gclose(_flat(W, wm, dl, dm, dq, de), og) <= 1e-8
    # forward-only evaluations and repeated gradients are bit-identical
    assert pb.logpdf(wm) == t0
    t2, p2, *g2 = pb.grad_nodes(wm)
    assert t2 == t0 and np.array_equal(p2, p0)
    for a, b in zip(g2, g0):
        assert np.array_equal(np.asarray(a), np.asarray(b))


def test_persistent_wide_families(W, O):
    # 40-taxon families: tasks wider than the persistent launch's shared
    # memory keep their rows in device memory within the same launch
    from whale_gb300 import synth

    wl = synth.config4(indices=list(range(120)))
    wm, ccds = wl.model, wl.ccds()
    pb = W.Batch(wm, ccds, grad=True, persistent=True)
    lb = W.Batch(wm, ccds, grad=True)
    t0, p0, *g0 = pb.grad_nodes(wm)
    t1, p1, *g1 = lb.grad_nodes(wm)
    assert np.array_equal(np.isneginf(p0), np.isneginf(p1))
    assert np.max(_rel(p0, p1)) <= 1e-12
    for a, b in zip(g0, g1):
        assert _gclose(a, b) <= 1e-10
    n = np.array([c.n_clades for c in ccds])
    pick = np.where(n <= 300)[0][:25]
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt)
    occ = [O.OracleCCD(om, wl.ale[i]) for i in pick]
    r = wm.rates
    _, oper = om.logpdf(occ, r.λ, r.μ, q=r.q, eta=r.η)
    assert np.max(_rel(p0[pick], oper)) <= REL


def test_persistent_wait_that_runs_out_is_reported(W, monkeypatch):
    # every task also waits on a flag that nothing sets, with a small poll
    # limit: the waits give up, the call reports WG_ECUDA, and the context
    # evaluates normally afterwards
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    wl = synth.config0(n_families=20)
    wm, ccds = wl.model, wl.ccds()
    ref = W.Batch(wm, ccds, grad=True).logpdf(wm)
    monkeypatch.setenv("WG_PERSIST_TEST_UNSET_WAIT", "1")
    monkeypatch.setenv("WG_PERSIST_SPIN_CAP", "32")
    bad = W.Batch(wm, ccds, grad=True, persistent=True)
    with pytest.raises(W.WhaleError) as ei:
        bad.logpdf(wm)
    assert ei.value.code == N.WG_ECUDA and "ran out" in str(ei.value)
    with pytest.raises(W.WhaleError):
        bad.grad_nodes(wm)
    monkeypatch.delenv("WG_PERSIST_TEST_UNSET_WAIT")
    monkeypatch.delenv("WG_PERSIST_SPIN_CAP")
    good = W.Batch(wm, ccds, grad=True, persistent=True)
    assert good.logpdf(wm) == pytest.approx(ref, rel=1e-12)
