"""Hand-written adjoint against the oracle's forward-mode duals (the stand-in
for ForwardDiff over the reference's logpdf) and against central differences
of the GPU forward.  Tolerance: 1e-8 relative (absolute for entries near 0)."""
import os

import numpy as np
import pytest

from conftest import read

pytestmark = pytest.mark.gpu
GREL = 1e-8


def _close(g, ref, rel=GREL):
    g, ref = np.asarray(g), np.asarray(ref)
    scale = np.maximum(np.abs(ref), 1.0)
    return np.max(np.abs(g - ref) / scale)


def test_gradient_golden_setting_critical_rates(W, O, ex1_tree, ex1_files):
    # test/runtests.jl:36-38: x = [ones(n); ones(n); [0.1, 0.2]; 0.8] -- λ = μ
    # everywhere, so every branch takes the critical formula of getα
    t = W.readnw(ex1_tree)
    x = np.r_[np.ones(17), np.ones(17), [0.1, 0.2], 0.8]
    wm = W.WhaleModel(W.DLWGD(λ=x[:17], μ=x[17:34], q=x[34:36], η=x[36]), t, 0.05)
    ccds = W.read_ale(os.path.dirname(ex1_files[0]), wm)
    g = W.gradient(wm, ccds)
    om = O.OracleModel(ex1_tree, 0.05)
    otot, og = om.gradient(O.read_ale_files(om, ex1_files), x[:17], x[17:34], q=x[34:36], eta=x[36])
    assert np.all(np.isfinite(g))
    assert _close(g, og) <= GREL


def test_gradient_general_rates(W, O, ex1_tree, ex1_files):
    t = W.readnw(ex1_tree)
    rng = np.random.default_rng(1)
    lam, mu = rng.normal(-0.5, 0.5, 17), rng.normal(-0.7, 0.5, 17)
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=[0.3, 0.45], η=0.7), t, 0.05)
    ccds = W.read_ale(os.path.dirname(ex1_files[0]), wm)
    tot, gd = W.logpdf_gradient(wm, ccds)
    g = np.concatenate([gd["λ"], gd["μ"], gd["q"], [gd["η"]]])
    om = O.OracleModel(ex1_tree, 0.05)
    otot, og = om.gradient(O.read_ale_files(om, ex1_files), lam, mu, q=[0.3, 0.45], eta=0.7)
    assert tot == pytest.approx(otot, rel=1e-10)
    assert _close(g, og) <= GREL


def test_gradient_constant_rates(W, O, ex1_tree, ex1_files):
    t = W.readnw(ex1_tree)
    wm = W.WhaleModel(W.ConstantDLWGD(λ=0.25, μ=0.35, q=[0.3, 0.45], η=0.7), t, 0.05)
    ccds = W.read_ale(os.path.dirname(ex1_files[0]), wm)
    g = W.gradient(wm, ccds)
    om = O.OracleModel(ex1_tree, 0.05)
    otot, og = om.gradient(O.read_ale_files(om, ex1_files), [0.25], [0.35], q=[0.3, 0.45], eta=0.7,
                           kind="ConstantDLWGD")
    assert _close(g, og) <= GREL


def test_gradient_config1_subset(W, O):
    from whale_gb300 import synth

    wl = synth.config1(n_families=120)
    wm = wl.model
    ccds = wl.ccds()
    keep = [i for i, c in enumerate(ccds) if c.n_clades <= 400][:60]
    ccds = [ccds[i] for i in keep]
    g = W.gradient(wm, ccds)
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt)
    occ = [O.OracleCCD(om, wl.ale[i]) for i in keep]
    r = wm.rates
    otot, og = om.gradient(occ, r.λ, r.μ, q=r.q, eta=r.η)
    assert _close(g, og) <= GREL


def test_gradient_vs_central_differences_of_gpu_forward(W, O):
    from whale_gb300 import synth

    wl = synth.config0(seed=5, n_families=30)
    wm = wl.model
    ccds = wl.ccds()
    g = W.gradient(wm, ccds)
    r = wm.rates
    base = np.r_[r.λ, r.μ, r.q, r.η]
    h = 1e-6
    fd = np.zeros_like(base)
    for i in range(base.size):
        xp, xm = base.copy(), base.copy()
        xp[i] += h
        xm[i] -= h
        fp = W.logpdf(wm(W.ConstantDLWGD(λ=xp[0], μ=xp[1], q=xp[2:-1], η=xp[-1])), ccds)
        fm = W.logpdf(wm(W.ConstantDLWGD(λ=xm[0], μ=xm[1], q=xm[2:-1], η=xm[-1])), ccds)
        fd[i] = (fp - fm) / (2 * h)
    assert np.allclose(g, fd, rtol=1e-5, atol=1e-5)


def test_gradient_deterministic(W, ex1_tree, ex1_files):
    t = W.readnw(ex1_tree)
    wm = W.WhaleModel(W.DLWGD(λ=np.ones(17) * 0.3, μ=np.ones(17) * 0.1, q=[0.2, 0.1], η=0.9), t, 0.05)
    ccds = W.read_ale(os.path.dirname(ex1_files[0]), wm)
    a = W.gradient(wm, ccds)
    b = W.gradient(wm, ccds)
    assert np.array_equal(a, b)


def test_gradient_nowhere_extinct_condition(W, O, ex1_tree, ex1_files):
    # NowhereExtinctCondition (src/condition.jl:31-36) depends on the rates
    # directly; its gradient joins the DP's through the host chain rule
    t = W.readnw(ex1_tree)
    rng = np.random.default_rng(9)
    lam, mu = rng.normal(-0.6, 0.4, 17), rng.normal(-0.8, 0.4, 17)
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=[0.25, 0.5], η=0.72), t, 0.05,
                      condition=W.NowhereExtinctCondition(t))
    ccds = W.read_ale(os.path.dirname(ex1_files[0]), wm)
    tot, gd = W.logpdf_gradient(wm, ccds)
    g = np.concatenate([gd["λ"], gd["μ"], gd["q"], [gd["η"]]])
    om = O.OracleModel(ex1_tree, 0.05, condition="nowhere")
    otot, og = om.gradient(O.read_ale_files(om, ex1_files), lam, mu, q=[0.25, 0.5], eta=0.72)
    assert tot == pytest.approx(otot, rel=1e-10)
    assert _close(g, og) <= GREL


def _slow_rates_case(W, O, lam_mean, mu_mean):
    from whale_gb300 import synth

    wl = synth.config1(n_families=60)
    ccds = wl.ccds()
    keep = [i for i, c in enumerate(ccds) if c.n_clades <= 300][:20]
    n = len(wl.model.rates.λ)
    rng = np.random.default_rng(3)
    lam, mu = rng.normal(np.log(lam_mean), 0.3, n), rng.normal(np.log(mu_mean), 0.3, n)
    q = np.asarray(wl.model.rates.q)
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=q, η=0.7), wl.model.tree, wl.model.Δt)
    g = W.gradient(wm, [ccds[i] for i in keep])
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt)
    otot, og = om.gradient([O.OracleCCD(om, wl.ale[i]) for i in keep], lam, mu, q=q, eta=0.7)
    return g, og


def test_gradient_slow_rates_one_dot_rows(W, O):
    # λ ~ 0.005, Δt = 0.02: ψ per slice ~ 1e-4, where the one-dot form of the
    # row adjoints divides a difference of two sums by ψ
    g, og = _slow_rates_case(W, O, 0.005, 0.004)
    assert _close(g, og) <= GREL


def test_gradient_tiny_duplication_rate_two_dot_rows(W, O):
    # λ ~ 1e-5: ψ below the one-dot threshold on every branch, the two-dot form
    g, og = _slow_rates_case(W, O, 1e-5, 0.01)
    assert _close(g, og) <= GREL


@pytest.mark.parametrize("log_lam", [-5.0, -7.0, -9.0])
def test_one_dot_row_adjoints_with_small_duplication_term(W, O, ex1_tree, ex1_files, log_lam):
    # low duplication and high loss on every branch: ψ per slice is 2.5e-4 down
    # to 4.6e-6 (above the 1e-6 switch to the two-dot form), so the ψ term is a
    # tiny share of each row's dot and ∂ψ_r = (E_{r-1} - E_r)/ψ_r is a
    # difference of nearly equal sums; the gradient must still match the duals.
    # No survival condition: at these rates the root condition's
    # 1 - g(εf) - g(εg) + g(εr) cancels to ~3e-12 (extinction ≈ 1), which
    # leaves ~1e-5 relative rounding in the condition and its derivative, in
    # the reference's own arithmetic as much as here.
    t = W.readnw(ex1_tree)
    lam = np.full(17, log_lam)
    mu = np.full(17, np.log(3.0))
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=[0.3, 0.45], η=0.7), t, 0.05, condition=W.NoCondition())
    ccds = W.read_ale(os.path.dirname(ex1_files[0]), wm)
    tot, gd = W.logpdf_gradient(wm, ccds)
    g = np.concatenate([gd["λ"], gd["μ"], gd["q"], [gd["η"]]])
    om = O.OracleModel(ex1_tree, 0.05, condition="none")
    otot, og = om.gradient(O.read_ale_files(om, ex1_files), lam, mu, q=[0.3, 0.45], eta=0.7)
    assert np.isfinite(otot)
    assert tot == pytest.approx(otot, rel=1e-10)
    assert _close(g, og) <= GREL
