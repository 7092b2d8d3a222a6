"""CUDA forward path against the oracle and the reference's pinned values.
Tolerance: per-family log-likelihood within 1e-10 relative (FP64 throughout)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, read

pytestmark = pytest.mark.gpu
REL = 1e-10


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    both_inf = np.isneginf(a) & np.isneginf(b)
    d = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    return np.where(both_inf, 0.0, d)


@pytest.fixture(scope="module")
def ex1(W, ex1_tree, ex1_files):
    t = W.readnw(ex1_tree)
    wm = W.WhaleModel(W.DLWGD(λ=np.ones(17), μ=np.ones(17), q=[0.2, 0.1], η=0.9), t, 0.05)
    return wm, W.read_ale(os.path.dirname(ex1_files[0]), wm)


def test_golden_single_family(W, ex1_tree, ex1_files, golden):
    # test/runtests.jl:15-19
    g = golden["single_family"]
    t = W.readnw(ex1_tree)
    wm = W.WhaleModel(W.DLWGD(λ=np.ones(17), μ=np.ones(17), q=g["q"], η=g["eta"]), t, g["dt"], maxn=g["maxn"])
    ccd = W.read_ale(os.path.dirname(ex1_files[0]), wm)
    assert W.logpdf(wm, ccd[0]) == pytest.approx(g["logpdf"], rel=REL)


def test_golden_twelve_families(W, ex1, golden):
    # test/runtests.jl:21-34 (logpdf! and logpdf)
    wm, ccds = ex1
    want = golden["twelve_families"]["logpdf"]
    assert W.logpdf(wm, ccds) == pytest.approx(want, rel=REL)
    assert W.logpdf_inplace(wm, ccds) == pytest.approx(want, rel=REL)


def test_root_rates_have_no_effect(W, ex1_tree, ex1_files, golden):
    # test/runtests.jl:44-49
    t = W.readnw(ex1_tree)
    lam, mu = np.ones(17), np.ones(17)
    r0 = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=[0.2, 0.1], η=0.9), t, 0.05)
    root_id = r0.root().id
    lam[root_id - 1] = np.nan
    mu[root_id - 1] = np.nan
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=[0.2, 0.1], η=0.9), t, 0.05)
    ccds = W.read_ale(os.path.dirname(ex1_files[0]), wm)
    assert W.logpdf_inplace(wm, ccds) == pytest.approx(golden["twelve_families"]["logpdf"], rel=REL)


def test_logpdf_tables_match_oracle(W, O, ex1, ex1_tree, ex1_files):
    # logpdf! keeps every DP table (src/core.jl:29); compare them entry-wise
    wm, ccds = ex1
    W.logpdf_inplace(wm, ccds[:3])
    om = O.OracleModel(ex1_tree, 0.05)
    for c, f in zip(ccds[:3], ex1_files[:3]):
        oc = O.OracleCCD(om, read(f))
        ref = om.family_tables(oc, np.ones(17), np.ones(17), q=[0.2, 0.1], eta=0.9)
        got = np.concatenate([x.reshape(-1) for x in c.ℓ])
        assert got.shape == ref.shape
        assert np.allclose(got, ref, rtol=1e-11, atol=1e-300)


def _check_workload(W, O, wl, n=None):
    wm = wl.model
    ccds = wl.ccds()[:n] if n else wl.ccds()
    texts = wl.ale[: len(ccds)]
    tot, per = W.get_batch(wm, ccds).logpdf(wm, per_family=True)
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt, minn=wm.minn, maxn=wm.maxn)
    occ = [O.OracleCCD(om, s) for s in texts]
    r = wm.rates
    kind = "ConstantDLWGD" if isinstance(r, W.ConstantDLWGD) else "DLWGD"
    otot, oper = om.logpdf(occ, r.λ, r.μ, q=r.q, eta=r.η, kind=kind)
    assert np.max(_rel(per, oper)) <= REL
    assert tot == pytest.approx(otot, rel=REL)
    return wm, ccds, per


def test_config0_per_family(W, O):
    from whale_gb300 import synth

    _check_workload(W, O, synth.config0())


def test_config1_subset_per_family(W, O):
    from whale_gb300 import synth

    wm, ccds, per = _check_workload(W, O, synth.config1(n_families=400))
    # the plain one-family-per-launch path gives the same numbers
    tot_p, per_p = W.get_batch(wm, ccds).logpdf_plain(wm)
    assert np.max(_rel(per_p, per)) <= 1e-12


def test_mul_tree(W, O):
    # test/runtests.jl:111-126 style MUL tree (example-5 has duplicated leaves)
    nw = read(os.path.join(GOLDEN, "example5_tree.nw")).strip()
    t = W.readnw(nw)
    n = len(W.postwalk(t))
    rng = np.random.default_rng(2)
    lam, mu = rng.normal(-1, 0.3, n), rng.normal(-1, 0.3, n)
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, η=0.9), t, 0.05)
    files = [os.path.join(GOLDEN, "example5", f) for f in sorted(os.listdir(os.path.join(GOLDEN, "example5")))]
    ccds = [W.read_ale(f, wm)[0] for f in files]
    tot, per = W.get_batch(wm, ccds).logpdf(wm, per_family=True)
    om = O.OracleModel(nw, 0.05)
    otot, oper = om.logpdf([O.OracleCCD(om, read(f)) for f in files], lam, mu, q=[], eta=0.9)
    assert np.isfinite(tot)
    assert np.max(_rel(per, oper)) <= REL


def test_single_ccd_batch_and_reparameterisation(W, O, ex1, ex1_tree, ex1_files):
    wm, ccds = ex1
    om = O.OracleModel(ex1_tree, 0.05)
    oc = O.OracleCCD(om, read(ex1_files[5]))
    rng = np.random.default_rng(9)
    for _ in range(3):
        lam, mu = rng.normal(0, 0.5, 17), rng.normal(0, 0.5, 17)
        w2 = wm({"λ": lam, "μ": mu, "q": [0.4, 0.05], "η": 0.6})
        got = W.logpdf(w2, ccds[5])
        _, ref = om.logpdf([oc], lam, mu, q=[0.4, 0.05], eta=0.6)
        assert got == pytest.approx(ref[0], rel=REL)


def test_underflow_gives_minus_inf_like_reference(W, O, ex1_tree, ex1_files):
    # extreme loss rates drive L below the FP64 range: -Inf, as src/core.jl:36
    t = W.readnw(ex1_tree)
    lam = np.full(17, -8.0)
    mu = np.full(17, 6.5)
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, q=[0.2, 0.1], η=0.9), t, 0.05)
    ccds = W.read_ale(os.path.dirname(ex1_files[0]), wm)
    om = O.OracleModel(ex1_tree, 0.05)
    occ = O.read_ale_files(om, ex1_files)
    tot, per = W.get_batch(wm, ccds).logpdf(wm, per_family=True)
    otot, oper = om.logpdf(occ, lam, mu, q=[0.2, 0.1], eta=0.9)
    assert np.array_equal(np.isneginf(per), np.isneginf(oper))
    fin = np.isfinite(oper)
    assert np.max(_rel(per[fin], oper[fin]), initial=0.0) <= REL
    assert (tot == otot) or tot == pytest.approx(otot, rel=REL)


def test_results_do_not_depend_on_pack_threads(W, monkeypatch):
    # the packer builds tasks on host threads and merges them in a fixed
    # order: one thread or many give the same layout, hence bit-identical
    # log L and gradients
    from whale_gb300 import synth

    wl = synth.config1(n_families=200)
    wm, ccds = wl.model, wl.ccds()
    out = []
    for th in ("1", "0"):
        monkeypatch.setenv("WG_PACK_THREADS", th)
        b = W.Batch(wm, ccds, grad=True)
        out.append(b.grad_nodes(wm))
        del b
    for x, y in zip(*out):
        assert np.array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("sub,tree", [("example4", "example4_tree.nw"), ("landplant", "landplant_tree.nw")])
def test_real_data_against_oracle(W, O, sub, tree):
    # the reference's own data (example/example-4: one family of 4,917 clades
    # on a 44-taxon tree; docs/data/landplant/100fams: 100 families on 13
    # taxa) under branch-wise rates: per-family log L within 1e-10 of the
    # oracle and the gradient within 1e-8 of its duals
    from conftest import GOLDEN, read

    nw = read(os.path.join(GOLDEN, tree)).strip()
    d = os.path.join(GOLDEN, sub)
    files = [os.path.join(d, f) for f in sorted(os.listdir(d))]
    t = W.readnw(nw)
    n = len(W.postwalk(t))
    rng = np.random.default_rng(11)
    lam, mu = rng.normal(np.log(0.2), 0.3, n), rng.normal(np.log(0.25), 0.3, n)
    wm = W.WhaleModel(W.DLWGD(λ=lam, μ=mu, η=0.7), t, 0.1)
    ccds = W.read_ale(d, wm)
    om = O.OracleModel(nw, 0.1)
    occ = O.read_ale_files(om, files)
    tot, per = W.Batch(wm, ccds).logpdf(wm, per_family=True)
    otot, oper = om.logpdf(occ, lam, mu, q=[], eta=0.7)
    assert np.all(np.isfinite(oper))
    for a, b in zip(per, oper):
        assert a == pytest.approx(b, rel=1e-10)
    assert tot == pytest.approx(otot, rel=1e-10)
    g = W.gradient(wm, ccds)
    _, og = om.gradient(occ, lam, mu, q=[], eta=0.7)
    assert np.max(np.abs(g - og) / np.maximum(np.abs(og), 1.0)) <= 1e-8


def test_config1_full_batch(W, O):
    # the bench's timed workload as the bench packs it (all 5,000 config-1
    # families in one gradient batch): every family's log L from the
    # gradient evaluation within 1e-10 of the oracle, and the gradient of a
    # 200-family sample (weights 1 on the sample, 0 elsewhere, the condition
    # scaled by the sample size) within 1e-8 of the oracle's duals
    from whale_gb300 import synth
    from whale_gb300.core import map_gradient

    wl = synth.config1(seed=1, n_families=5000)
    wm = wl.model
    b = W.Batch(wm, wl.ccds(), grad=True)
    tot, per, *_ = b.grad_nodes(wm)
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt, minn=wm.minn, maxn=wm.maxn)
    occ = O.parse_texts(om, wl.ale)
    r = wm.rates
    otot, oper = om.logpdf(occ, r.λ, r.μ, q=r.q, eta=r.η)
    assert len(per) == 5000
    assert np.max(_rel(per, oper)) <= REL
    assert tot == pytest.approx(otot, rel=REL)
    sample = np.sort(np.random.default_rng(11).choice(5000, size=200, replace=False))
    w = np.zeros(5000)
    w[sample] = 1.0
    _, _, dl, dm, dq, de = b.grad_nodes_weighted(wm, w, 200.0)
    g = map_gradient(wm, dl, dm, dq, de)
    flat = np.concatenate([g["λ"], g["μ"], g["q"], [g["η"]]])
    _, og = om.gradient([occ[i] for i in sample], r.λ, r.μ, q=r.q, eta=r.η)
    assert np.max(np.abs(flat - og) / np.maximum(np.abs(og), 1.0)) <= 1e-8
