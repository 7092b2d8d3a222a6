"""Backtracking on the host from the oracle's own DP tables (no GPU): valid
reconciliations, and the root's first event drawn with the probabilities of
the root recursion's terms (src/core.jl:130-158, src/track.jl:233-250,
359-401) within 4 standard errors over 4,000 trees."""
import numpy as np
import pytest

from test_gpu_backtrack import _genes


def _setting(W, O):
    from whale_gb300 import synth

    wl = synth.config0(seed=8, n_families=6)
    wm = wl.model
    ccds = wl.ccds()
    i = max(range(len(ccds)), key=lambda j: ccds[j].n_clades)
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt)
    oc = O.OracleCCD(om, wl.ale[i])
    r = wm.rates
    tab = om.family_tables(oc, [r.λ], [r.μ], q=r.q, eta=r.η, kind="ConstantDLWGD")
    return wl, wm, ccds[i], i, om, tab


def test_host_backtracking_from_oracle_tables(W, O):
    from whale_gb300.track import backtrack_tables

    wl, wm, ccd, i, om, tab = _setting(W, O)
    r = wm.rates
    trees = backtrack_tables(wm, ccd, tab, n=4000, seed=99)
    genes = _genes(wl.ale[i])
    for tr in trees[:300]:
        leaves = [n for n in tr.root.postwalk() if n.isleaf()]
        assert sorted(n.name for n in leaves if n.label != "loss") == genes
    # root event probabilities from the oracle's tables
    order = wm.order
    arr = ccd.arrays()
    so, sp = arr["species_offsets"], arr["species"]
    nc = ccd.n_clades
    spec = [set(sp[so[g]:so[g + 1]]) for g in range(nc)]
    base, cols, o = {}, {}, 0
    for m in order:
        comp = [g for g in range(nc) if spec[g] <= set(m.clade)]
        cols[m.pos] = {g: j for j, g in enumerate(comp)}
        base[m.pos] = (o, len(comp))
        o += (m.nslices + 1) * len(comp)
    assert o == tab.size

    def L(k, g, t):
        c = cols[k].get(g)
        return 0.0 if c is None else tab[base[k][0] + (t - 1) * base[k][1] + c]

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
    dup = sum(p[k] * L(root.pos, g1[k], 1) * L(root.pos, g2[k], 1) * cd for k in range(sof[ub], sof[ub + 1]))
    spe = sum(p[k] * (top(f, g1[k]) * top(h, g2[k]) + top(h, g1[k]) * top(f, g2[k])) * cs
              for k in range(sof[ub], sof[ub + 1]))
    los = (top(f, ub) * etop(h) + top(h, ub) * etop(f)) * cs
    total = L(root.pos, ub, 1)
    assert dup + spe + los == pytest.approx(total, rel=1e-10)
    cnt = {"duplication": 0, "speciation": 0, "sploss": 0}
    for tr in trees:
        cnt[tr.root.label] += 1
    for key, pr in (("duplication", dup / total), ("speciation", spe / total), ("sploss", los / total)):
        se = np.sqrt(max(pr * (1 - pr), 1e-4) / len(trees))
        assert abs(cnt[key] / len(trees) - pr) <= 4 * se


def test_track_from_oracle_tables(W, O):
    # TreeTracker (src/track.jl:11-82) with the oracle's tables standing in for
    # the device: picks, seeds and summaries (src/rectree.jl:123-143)
    from whale_gb300 import synth
    from whale_gb300.track import _draw_seed, backtrack_tables, sumtrees, track_tables

    wl = synth.config0(seed=8, n_families=6)
    wm = wl.model
    ccds = wl.ccds()[:3]
    om = O.OracleModel(W.nwstr(wm.tree), wm.Δt)
    ocs = [O.OracleCCD(om, t) for t in wl.ale[:3]]
    r = wm.rates

    def tables_of(m, f):
        x = m.rates
        return om.family_tables(ocs[f], [x.λ], [x.μ], q=x.q, eta=x.η, kind="ConstantDLWGD")

    # one draw: every pick is it, and tree j of family f is the tree sampled
    # directly from its tables with that pick's seed
    trees = track_tables(tables_of, wm, ccds, [r], 6, seed=3, summary=False)
    for f, c in enumerate(ccds):
        assert len(trees[f]) == 6
        for j in range(6):
            ref = backtrack_tables(wm, c, tables_of(wm, f), n=1, seed=_draw_seed(3, j, f))[0]
            assert trees[f][j].newick == ref.newick
        genes = _genes(wl.ale[f])
        for t in trees[f]:
            assert sorted(n.name for n in t.root.postwalk() if n.isleaf() and n.label != "loss") == genes
    again = track_tables(tables_of, wm, ccds, [r], 6, seed=3, summary=False, threads=1)
    assert [[t.newick for t in x] for x in again] == [[t.newick for t in x] for x in trees]
    # two draws (the second with ten times the duplication rate): both are used
    hi = r(dict(λ=r.λ * 10))
    sums = track_tables(tables_of, wm, ccds, [r, hi], 40, seed=4)
    raw = track_tables(tables_of, wm, ccds, [r, hi], 40, seed=4, summary=False)
    for s, t, c in zip(sums, raw, ccds):
        freqs = [fr for fr, _ in s.trees]
        assert abs(sum(freqs) - 1) < 1e-12 and freqs == sorted(freqs, reverse=True)
        assert all(0 < x <= 1 for cr in s.credibility for x in cr)
        # expected event counts = mean over the samples of each tree's counts
        K = len(wm.order)
        mean = {lab: np.zeros(K) for lab in s.events}
        for tr in t:
            for n in tr.root.postwalk():
                mean[n.label][n.node] += 1 / len(t)
        for lab in s.events:
            assert np.allclose(s.events[lab], mean[lab], atol=1e-12)
        s2 = sumtrees(t, c, wm)  # the summary of the same draws
        assert [(fr, tr.newick) for fr, tr in s2.trees] == [(fr, tr.newick) for fr, tr in s.trees]
    dup = sum(s.events["duplication"].sum() for s in sums)
    dup_lo = sum(s.events["duplication"].sum() for s in track_tables(tables_of, wm, ccds, [r], 40, seed=4))
    assert dup > dup_lo


def test_pairwise_event_pps_sum_to_one(W, O, ex1_tree, ex1_files):
    # test/runtests.jl:95-109 on the oracle's tables: 100 trees of the first
    # example-1 family under DLWGD(λ = μ = ones, q = [0.2, 0.1], η = 0.9),
    # Δt = 0.05; every gene pair's event probabilities sum to 1
    from conftest import read
    from whale_gb300.track import backtrack_tables, getpairs, sumtrees

    t = W.readnw(ex1_tree)
    wm = W.WhaleModel(W.DLWGD(λ=np.ones(17), μ=np.ones(17), q=[0.2, 0.1], η=0.9), t, 0.05)
    ccd = W.read_ale(ex1_files[0], wm)[0]
    om = O.OracleModel(ex1_tree, 0.05)
    tab = om.family_tables(O.OracleCCD(om, read(ex1_files[0])), np.ones(17), np.ones(17), q=[0.2, 0.1], eta=0.9)
    trees = backtrack_tables(wm, ccd, tab, n=100, seed=1)
    fam, pairs, labels, pp = getpairs([sumtrees(trees, ccd, wm)], wm)[0]
    assert len(pairs) == 13 * 12 // 2  # 13 genes
    assert len(labels) == 2 * 17 + 3 * 2  # two labels per node, three per WGD node (19 nodes)
    assert np.allclose(pp.sum(axis=1), 1.0)
