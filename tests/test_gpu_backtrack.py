"""Backtracking (src/track.jl:180-488): sampled reconciled trees are valid
reconciliations of the family, and the first event drawn at the root follows
the DP.  The event terms are recomputed here from the oracle's own DP tables
(the root recursion of src/core.jl:130-158 must add up to the root value),
and 4,000 sampled trees must reproduce their probabilities within 4 standard
errors."""
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _genes(ale_text):
    out, on = [], False
    for ln in ale_text.splitlines():
        if ln.startswith("#"):
            on = ln.strip() == "#leaf-id"
            continue
        if on and ln.strip():
            out.append(ln.split()[0])
    return sorted(out)


@pytest.fixture(scope="module")
def fam(W, O):
    from whale_gb300 import synth

    wl = synth.config0(seed=8, n_families=6)
    wm = wl.model
    ccds = wl.ccds()
    return wl, wm, ccds


def test_sampled_trees_are_reconciliations(W, fam):
    wl, wm, ccds = fam
    labels = {"speciation", "duplication", "wgd", "wgdloss", "sploss", "loss"}
    for i in range(3):
        trees = W.backtrack(wm, ccds[i], n=200, seed=11 + i)
        assert len(trees) == 200
        genes = _genes(wl.ale[i])
        for tr in trees:
            root = tr.root
            assert root.node == len(wm.order) - 1 and root.clade == ccds[i].n_clades - 1
            leaves = [n for n in root.postwalk() if n.isleaf()]
            assert sorted(n.name for n in leaves if n.label != "loss") == genes
            for n in root.postwalk():
                assert n.label in labels
                if n.label == "loss":
                    assert n.clade == -1 and n.isleaf()
                if n.label == "duplication":
                    assert len(n.children) == 2 and all(c.node == n.node for c in n.children)
                if not n.isleaf():
                    assert all(c.distance >= -1e-12 for c in n.children)
    # the same seed gives the same trees
    a = [t.newick for t in W.backtrack(wm, ccds[0], n=5, seed=3)]
    b = [t.newick for t in W.backtrack(wm, ccds[0], n=5, seed=3)]
    assert a == b


def test_root_event_frequencies_follow_the_dp(W, O, fam):
    wl, wm, ccds = fam
    i = max(range(len(ccds)), key=lambda j: ccds[j].n_clades)
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt)
    oc = O.OracleCCD(om, wl.ale[i])
    r = wm.rates
    tab = om.family_tables(oc, [r.λ], [r.μ], q=r.q, eta=r.η, kind="ConstantDLWGD")
    order = wm.order
    arr = ccds[i].arrays()
    so, sp = arr["species_offsets"], arr["species"]
    nc = ccds[i].n_clades
    spec = [set(sp[so[g]:so[g + 1]]) for g in range(nc)]
    base, cols = {}, {}
    o = 0
    for m in order:
        comp = [g for g in range(nc) if spec[g] <= set(m.clade)]
        cols[m.pos] = {g: j for j, g in enumerate(comp)}
        base[m.pos] = (o, len(comp))
        o += (m.nslices + 1) * len(comp)

    def L(k, g, t):  # t is 1-based
        c = cols[k].get(g)
        if c is None:
            return 0.0
        b0, w = base[k]
        return tab[b0 + (t - 1) * w + c]

    root = order[-1]
    f, h = root.children
    top = lambda k, g: L(k, g, order[k].nslices + 1)
    eps = om.tables([r.λ], [r.μ], q=r.q, eta=r.η, kind="ConstantDLWGD")[0]
    offs = np.cumsum([0] + [m.nslices + 1 for m in order])
    etop = lambda k: eps[offs[k + 1] - 1]
    eta, er = r.η, etop(root.pos)
    xi = 1 - (1 - eta) * er
    cd, cs = xi * (1 - eta) / eta, eta * (1 - er) / xi ** 2
    ub = nc - 1
    sof, g1, g2, p = arr["split_offsets"], arr["g1"], arr["g2"], arr["p"]
    dup = spe = 0.0
    for k in range(sof[ub], sof[ub + 1]):
        a, b = g1[k], g2[k]
        dup += p[k] * L(root.pos, a, 1) * L(root.pos, b, 1) * cd
        spe += p[k] * (top(f, a) * top(h, b) + top(h, a) * top(f, b)) * cs
    los = (top(f, ub) * etop(h) + top(h, ub) * etop(f)) * cs
    total = L(root.pos, ub, 1)
    assert dup + spe + los == pytest.approx(total, rel=1e-10)
    n = 4000
    trees = W.backtrack(wm, ccds[i], n=n, seed=2024)
    cnt = {"duplication": 0, "speciation": 0, "sploss": 0}
    for tr in trees:
        cnt[tr.root.label] += 1
    for key, pr in (("duplication", dup / total), ("speciation", spe / total), ("sploss", los / total)):
        se = np.sqrt(max(pr * (1 - pr), 1e-4) / n)
        assert abs(cnt[key] / n - pr) <= 4 * se


def test_track_matches_per_family_backtracking(W, fam):
    # TreeTracker on the device (src/track.jl:11-82): one batched logpdf! per
    # pick, each family's tables downloaded without re-evaluating
    # (wg_batch_tables) and sampled; every tree equals wg_backtrack's on the
    # same layout, draw and seed
    import ctypes as C

    from whale_gb300 import _native as N
    from whale_gb300.track import _draw_seed

    wl, wm, ccds = fam
    r = wm.rates
    draws = [r, r(dict(λ=r.λ * 3, μ=r.μ * 0.5))]
    trees = W.track(wm, ccds, draws, 5, seed=21, summary=False)
    picks = np.random.default_rng(21).integers(len(draws), size=5)
    b = W.Batch(wm, ccds, tables=True)
    with pytest.raises(W.WhaleError, match="evaluate it first"):
        b.last_tables(0)
    L = N.lib()
    for j, i in enumerate(picks):
        m = wm(draws[i])
        m.load()
        for f in range(len(ccds)):
            seed = C.c_uint64(_draw_seed(21, j, f))
            need = N.i64()
            N.check(L.wg_backtrack(b.ctx.h, m._struct.h, b.h, f, 1, seed, None, 0, C.byref(need)))
            buf = C.create_string_buffer(need.value)
            N.check(L.wg_backtrack(b.ctx.h, m._struct.h, b.h, f, 1, seed, buf, need.value, C.byref(need)))
            ref = [ln for ln in buf.value.decode().split("\n") if ln]
            assert [trees[f][j].newick] == ref
    # after an evaluation the download equals logpdf!'s own tables
    ll, tab = b.family_tables(wm, 2)
    ll2, tab2 = b.last_tables(2)
    assert ll2 == ll and np.array_equal(tab2, tab)
    s = W.track(wm, ccds[:2], draws, 30, seed=2)
    assert all(abs(sum(fr for fr, _ in x.trees) - 1) < 1e-12 for x in s)


def test_pairwise_event_pps_sum_to_one(W, ex1_tree, ex1_files):
    # test/runtests.jl:95-109: 100 trees of the first example-1 family,
    # summarised, and every gene pair's event probabilities sum to 1
    t = W.readnw(ex1_tree)
    wm = W.WhaleModel(W.DLWGD(λ=np.ones(17), μ=np.ones(17), q=[0.2, 0.1], η=0.9), t, 0.05)
    ccd = W.read_ale(ex1_files[0], wm)[0]
    trees = W.backtrack(wm, ccd, n=100, seed=1)
    fam, pairs, labels, pp = W.getpairs([W.sumtrees(trees, ccd, wm)], wm)[0]
    assert len(pairs) == 78 and len(labels) == 40
    assert np.allclose(pp.sum(axis=1), 1.0)
