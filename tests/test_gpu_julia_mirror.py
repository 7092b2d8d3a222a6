"""The Julia drop-in (whale.jl_gb300/julia/WhaleGPU.jl) cannot run here: no
Julia on either machine.  This test replays its exact ccall sequence through
ctypes, with the same argument construction and the same host-side chain to
the rates struct:

  wg_ctx_create -> wg_model_create (GPUModel: wm.order, kinds, children as
  order positions, slice counts and widths, leaf probabilities, species sets,
  condition) -> wg_ccd_create per family (ccd_handle: the reference's CCD
  layout, here the oracle's restatement of it: clades by size, species,
  0-based split triples) -> wg_batch_create(WG_BATCH_GRAD) ->
  wg_model_set_rates (node_rates: getθ per node) -> wg_logpdf_grad with null
  per-family and table pointers -> rates_gradient (λ, μ on DLWGD's log scale
  by node id, q by WGD ordinal, η; ConstantDLWGD sums) -> the ForwardDiff
  method's contraction with the Duals' partials and the rrule's pullback.

Value within 1e-10 and gradient within 1e-8 of the oracle (its forward-mode
duals stand in for ForwardDiff over the reference's logpdf)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
NODE_LEAF, NODE_INTERNAL, NODE_WGD, NODE_ROOT = 0, 1, 2, 3


def _check(N, rc):
    N.check(rc)


def _gpu_model(N, wm):
    # GPUModel(wm)
    order = wm.order
    K = len(order)
    kind = np.array([m.kind for m in order], np.int32)
    c0 = np.array([m.children[0] if len(m.children) >= 1 else -1 for m in order], np.int32)
    c1 = np.array([m.children[1] if len(m.children) >= 2 else -1 for m in order], np.int32)
    nrow = np.array([m.nslices + 1 for m in order], np.int32)
    slen = np.array([m.slice_len if m.nslices > 0 else 0.0 for m in order])
    leafp = np.array([m.leafP for m in order])
    off, sp = [0], []
    for m in order:
        sp += sorted(m.clade)
        off.append(len(sp))
    off, sp = np.array(off, np.int32), np.array(sp, np.int32)
    cond = {"RootCondition": 1, "NonExtinctCondition": 2, "NowhereExtinctCondition": 3, "NoCondition": 0}[
        type(wm.condition).__name__]
    h = C.c_void_p()
    _check(N, N.lib().wg_model_create(K, N.iptr(kind), N.iptr(c0), N.iptr(c1), N.iptr(nrow), N.dptr(slen),
                                      N.dptr(leafp), N.iptr(off), N.iptr(sp), cond, C.byref(h)))
    return h


def _ccd_handle(N, oc):
    # ccd_handle(x::CCD) from the reference's CCD layout
    cl = [oc.clade(i) for i in range(oc.n_clades)]
    nleaves = np.array([c["nleaves"] for c in cl], np.int32)
    spo, sp, so, g1, g2, pp = [0], [], [0], [], [], []
    for c in cl:
        sp += sorted(c["species"])
        spo.append(len(sp))
        for a, b, p in c["splits"]:
            g1.append(a)
            g2.append(b)
            pp.append(p)
        so.append(len(g1))
    arr = [np.array(x, np.int32) for x in (spo, sp, so, g1, g2)]
    pp = np.array(pp)
    h = C.c_void_p()
    _check(N, N.lib().wg_ccd_create(len(cl), N.iptr(nleaves), N.iptr(arr[0]), N.iptr(arr[1]), N.iptr(arr[2]),
                                    N.iptr(arr[3]), N.iptr(arr[4]), N.dptr(pp), int(cl[0]["count"]), C.byref(h)))
    return h


def _rates_gradient(wm, lam, mu, dl, dm, dq, deta):
    # rates_gradient(wm, lam, mu, dl, dm, dq, dη)
    r = wm.rates
    gq = np.zeros(r.q.size)
    for k, m in enumerate(wm.order):
        if m.kind == NODE_WGD:
            gq[m.wgdid - 1] += dq[k]
    if type(r).__name__ == "ConstantDLWGD":
        ok = ~np.isnan(lam)
        return {"λ": float(np.sum(dl[ok])), "μ": float(np.sum(dm[ok])), "q": gq, "η": deta}
    gl, gm = np.zeros(r.λ.size), np.zeros(r.μ.size)
    for k, m in enumerate(wm.order):
        if np.isnan(lam[k]):
            continue
        tgt = wm.order[wm.nonwgdchild(k)].id if m.kind == NODE_WGD else m.id
        gl[tgt - 1] += dl[k] * lam[k]
        gm[tgt - 1] += dm[k] * mu[k]
    return {"λ": gl, "μ": gm, "q": gq, "η": deta}


def _flat(g):
    return np.concatenate([np.atleast_1d(g["λ"]), np.atleast_1d(g["μ"]), g["q"], [g["η"]]])


@pytest.mark.parametrize("which", ["config1", "config0"])
def test_julia_ccall_sequence(W, O, which):
    from whale_gb300 import _native as N
    from whale_gb300 import synth

    wl = synth.config1(n_families=150) if which == "config1" else synth.config0(n_families=60)
    wm = wl.model
    L = N.lib()
    ctx = C.c_void_p()
    _check(N, L.wg_ctx_create(0, C.byref(ctx)))
    mh = bh = None
    hs = []
    try:
        mh = _gpu_model(N, wm)
        om = O.OracleModel(W.nwstr(wm.tree), wm.Δt, minn=wm.minn, maxn=wm.maxn)
        occ = O.parse_texts(om, wl.ale)
        hs = [_ccd_handle(N, oc) for oc in occ]
        arr = (C.c_void_p * len(hs))(*[h.value for h in hs])
        bh = C.c_void_p()
        _check(N, L.wg_batch_create(ctx, mh, arr, len(hs), N.BATCH_GRAD, C.byref(bh)))
        lam, mu, q, eta, p = wm.node_rates()  # node_rates(wm): getθ per node
        _check(N, L.wg_model_set_rates(mh, N.dptr(lam), N.dptr(mu), N.dptr(q), eta, N.dptr(p)))
        K = len(wm.order)
        tot, de = N.dbl(), N.dbl()
        dl, dm, dq = np.zeros(K), np.zeros(K), np.zeros(K)
        _check(N, L.wg_logpdf_grad(ctx, mh, bh, None, C.byref(tot), N.dptr(dl), N.dptr(dm), N.dptr(dq),
                                   C.byref(de), None, None, None))
        g = _rates_gradient(wm, lam, mu, dl, dm, dq, de.value)
        r = wm.rates
        kind = type(r).__name__
        otot, og = om.gradient(occ, r.λ, r.μ, q=r.q, eta=r.η, kind=kind)
        assert tot.value == pytest.approx(otot, rel=1e-10)
        flat = _flat(g)
        assert np.max(np.abs(flat - og) / np.maximum(np.abs(og), 1.0)) <= 1e-8
        # the ForwardDiff method: partials = Σ_i g_i · partials(x_i), here for
        # three seeded directions (a chunk of 3)
        V = np.random.default_rng(5).normal(size=(flat.size, 3))
        got = flat @ V
        want = og @ V
        assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1.0)) <= 1e-8
        # the rrule's pullback: Δ times the rates gradient, field by field
        delta = 2.5
        pb = {k: delta * np.asarray(v) for k, v in g.items()}
        assert np.allclose(_flat(pb), delta * og, rtol=1e-8, atol=1e-8)
    finally:
        if bh is not None:
            L.wg_batch_destroy(bh)
        for h in hs:
            L.wg_ccd_destroy(h)
        if mh is not None:
            L.wg_model_destroy(mh)
        L.wg_ctx_destroy(ctx)
