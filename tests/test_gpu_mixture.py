"""MixtureModel and ModelArray (src/core.jl:66-79) on the GPU path against the
oracle: the mixture is composed from the oracle's per-family log L and
per-family gradients (each family's ∇(log L_ij - condition_j) weighted by
its posterior component weight).  Tolerances: 1e-10 relative on the
log-likelihood, 1e-8 on gradients."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(g, ref):
    g, ref = np.asarray(g, dtype=float), np.asarray(ref, dtype=float)
    return np.max(np.abs(g - ref) / np.maximum(np.abs(ref), 1.0))


@pytest.fixture(scope="module")
def setting(W, O):
    from whale_gb300 import synth

    wl = synth.config0(seed=6, n_families=14)
    wm1 = wl.model
    wm2 = wm1({"λ": 0.35, "μ": 0.25, "q": [0.4], "η": 0.8})
    ccds = wl.ccds()
    om = O.OracleModel(W.nwstr(wm1.tree), wm1.Δt)
    occ = [O.OracleCCD(om, a) for a in wl.ale]
    return wm1, wm2, ccds, om, occ, wl.ale


def setting_ale(setting):
    return setting[5]


def _oracle_family(om, occ, wm):
    """Per family: log L - condition and ∇(log L - condition) as [λ, μ, q, η]."""
    r = wm.rates
    vals, grads = [], []
    for oc in occ:
        t, g = om.gradient([oc], [r.λ], [r.μ], q=r.q, eta=r.η, kind="ConstantDLWGD")
        vals.append(t)
        grads.append(np.asarray(g))
    return np.array(vals), np.array(grads)


def test_mixture_logpdf_and_gradient(W, O, setting):
    wm1, wm2, ccds, om, occ, _ = setting
    prior = [0.3, 0.7]
    mm = W.MixtureModel([wm1, wm2], prior)
    a1, g1 = _oracle_family(om, occ, wm1)
    a2, g2 = _oracle_family(om, occ, wm2)
    a = np.stack([a1 + np.log(prior[0]), a2 + np.log(prior[1])], axis=1)
    lse = np.logaddexp(a[:, 0], a[:, 1])
    assert W.logpdf(mm, ccds) == pytest.approx(lse.sum(), rel=1e-10)
    tot, grads, dprior = W.logpdf_gradient(mm, ccds)
    assert tot == pytest.approx(lse.sum(), rel=1e-10)
    w = np.exp(a - lse[:, None])
    for j, (gd, go) in enumerate(zip(grads, (g1, g2))):
        ref = (w[:, j:j + 1] * go).sum(axis=0)
        got = np.concatenate([[gd["λ"], gd["μ"]], gd["q"], [gd["η"]]])
        assert _close(got, ref) <= 1e-8
    assert _close(dprior, w.sum(axis=0) / np.array(prior)) <= 1e-10


def test_model_array(W, O, setting):
    wm1, wm2, ccds, om, occ, _ = setting
    models = [wm1 if i % 3 else wm2 for i in range(len(ccds))]
    ma = W.ModelArray(models)
    ref = 0.0
    for i, oc in enumerate(occ):
        r = models[i].rates
        _, per = om.logpdf([oc], [r.λ], [r.μ], q=r.q, eta=r.η, kind="ConstantDLWGD")
        ref += per[0]  # single-CCD form: no condition (src/core.jl:39)
    assert W.logpdf(ma, ccds) == pytest.approx(ref, rel=1e-10)
    tot, per_model = W.logpdf_gradient(ma, ccds)
    assert tot == pytest.approx(ref, rel=1e-10)
    # the unconditioned sums' gradients, from an oracle model without condition
    om_nc = O.OracleModel(W.nwstr(wm1.tree), wm1.Δt, condition="none")
    occ_nc = [O.OracleCCD(om_nc, a) for a in setting_ale(setting)]
    for wm, gd in per_model:
        idx = [i for i, m in enumerate(models) if m is wm]
        r = wm.rates
        _, og = om_nc.gradient([occ_nc[i] for i in idx], [r.λ], [r.μ], q=r.q, eta=r.η, kind="ConstantDLWGD")
        got = np.concatenate([[gd["λ"], gd["μ"]], gd["q"], [gd["η"]]])
        assert _close(got, og) <= 1e-8
