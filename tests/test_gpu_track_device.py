"""Backtracking on the device (wg_track_device, src/track.jl:180-414): one GPU
thread per tree samples from the tables a batched logpdf! left in device
memory.  It follows the host sampler's event order, arithmetic and random
stream, so every tree must equal the host sampler's (wg_backtrack_tables on
the downloaded tables) for the same seed, text for text; the root's first
event must follow the oracle's DP terms within 4 standard errors over 4,000
device-sampled trees; and the call refuses batches without tables or without
a fetched evaluation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_trees(W, b, wm, ccds, seeds):
    from whale_gb300.track import backtrack_tables

    out = []
    for f, s in enumerate(seeds):
        _, tab = b.last_tables(f)
        out.append(backtrack_tables(wm, ccds[f], tab, n=1, seed=int(s))[0].newick)
    return out


@pytest.mark.parametrize("which", ["config0", "config1"])
def test_device_trees_equal_host_trees(W, which):
    from whale_gb300 import synth
    from whale_gb300.track import sample_device, tree_of_nodes

    wl = synth.config0(seed=4, n_families=60) if which == "config0" else synth.config1(seed=2, n_families=80)
    wm, ccds = wl.model, wl.ccds()
    b = W.Batch(wm, ccds, tables=True)
    b.logpdf(wm)
    rng = np.random.default_rng(3)
    seeds = rng.integers(0, 2**63, size=len(ccds), dtype=np.uint64)
    arrs = sample_device(b, wm, list(range(len(ccds))), seeds)
    dev = [tree_of_nodes(wm, ccds[f], a).newick for f, a in enumerate(arrs)]
    host = _host_trees(W, b, wm, ccds, seeds)
    assert dev == host
    # a second draw with other seeds on the same tables, families repeated
    fams = [3, 3, 7, 0, 3]
    seeds2 = [11, 12, 11, 5, 11]
    arrs2 = sample_device(b, wm, fams, seeds2)
    assert tree_of_nodes(wm, ccds[3], arrs2[0]).newick == tree_of_nodes(wm, ccds[3], arrs2[4]).newick
    from whale_gb300.track import backtrack_tables

    for f, s, a in zip(fams, seeds2, arrs2):
        _, tab = b.last_tables(f)
        assert tree_of_nodes(wm, ccds[f], a).newick == backtrack_tables(wm, ccds[f], tab, n=1, seed=s)[0].newick


def test_device_root_event_frequencies_follow_the_dp(W, O):
    from whale_gb300 import synth
    from whale_gb300.track import sample_device, tree_of_nodes

    wl = synth.config0(seed=8, n_families=6)
    wm, ccds = wl.model, wl.ccds()
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

    def L(k, g, t):
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
        a, b_ = g1[k], g2[k]
        dup += p[k] * L(root.pos, a, 1) * L(root.pos, b_, 1) * cd
        spe += p[k] * (top(f, a) * top(h, b_) + top(h, a) * top(f, b_)) * cs
    los = (top(f, ub) * etop(h) + top(h, ub) * etop(f)) * cs
    total = L(root.pos, ub, 1)
    assert dup + spe + los == pytest.approx(total, rel=1e-10)
    b = W.Batch(wm, ccds, tables=True)
    b.logpdf(wm)
    n = 4000
    arrs = sample_device(b, wm, [i] * n, list(range(1, n + 1)))
    cnt = {"duplication": 0, "speciation": 0, "sploss": 0}
    for a in arrs:
        cnt[tree_of_nodes(wm, ccds[i], a).root.label] += 1
    for key, pr in (("duplication", dup / total), ("speciation", spe / total), ("sploss", los / total)):
        se = np.sqrt(max(pr * (1 - pr), 1e-4) / n)
        assert abs(cnt[key] / n - pr) <= 4 * se


def test_device_tracking_refuses_without_tables(W):
    from whale_gb300 import _native as N
    from whale_gb300 import synth
    from whale_gb300.track import sample_device

    wl = synth.config0(seed=1, n_families=10)
    wm, ccds = wl.model, wl.ccds()
    b = W.Batch(wm, ccds)
    b.logpdf(wm)
    with pytest.raises(W.WhaleError) as ei:
        sample_device(b, wm, [0], [1])
    assert ei.value.code == N.WG_ESTATE
    bt = W.Batch(wm, ccds, tables=True)
    with pytest.raises(W.WhaleError, match="evaluate it first"):
        sample_device(bt, wm, [0], [1])
    bt.logpdf(wm)
    with pytest.raises(W.WhaleError) as ei:
        sample_device(bt, wm, [len(ccds)], [1])
    assert ei.value.code == N.WG_EINVAL
