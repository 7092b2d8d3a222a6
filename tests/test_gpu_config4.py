"""Config 4 as parity cases: the 40-taxon Yule tree with 10 WGDs and
Δt = 0.01, families from 500 NNI-perturbed trees with heavy-tailed clade
counts.  The first 400 of its 50,000 families (identical to theirs in the
full workload) run in one batch: per-family log L against the oracle
(1e-10, including the largest families, whose likelihood underflows FP64 to
-Inf as in the reference), gradients against the oracle's duals on small
families and against central differences of the GPU forward on the large
ones, whose adjoint rows live in device memory.  A family of ~18,000 clades
takes the device-memory path in the forward as well."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SMEM_DOUBLES = 227 * 1024 // 8  # shared memory of one CTA, in doubles


@pytest.fixture(scope="module")
def cfg4(W, O):
    from whale_gb300 import synth

    wl = synth.config4(n_families=400)
    ccds = wl.ccds()
    om = O.OracleModel(W.nwstr(wl.model.tree), wl.model.Δt)
    n = np.array([c.n_clades for c in ccds])
    return wl, ccds, om, n


def _task_widths(W, wm, ccds, grad):
    import ctypes

    from whale_gb300 import _native as N

    arr = (ctypes.c_void_p * len(ccds))(*[c._h for c in ccds])
    k = N.i64()
    N.check(N.lib().wg_pack_tasks(wm._struct.h, arr, len(ccds), 1 if grad else 0, None, 0, ctypes.byref(k)))
    out = np.zeros(12 * k.value, np.int32)
    N.check(N.lib().wg_pack_tasks(wm._struct.h, arr, len(ccds), 1 if grad else 0, out.ctypes.data_as(N.P_i32),
                                  out.size, ctypes.byref(k)))
    return out.reshape(-1, 12)[:, 2]


def test_config4_per_family_against_oracle(W, O, cfg4):
    wl, ccds, om, n = cfg4
    wm, r = wl.model, wl.model.rates
    # the adjoint keeps six rows of a task: the widest tasks exceed shared memory
    assert np.any(6 * _task_widths(W, wm, ccds, True) > SMEM_DOUBLES)
    tot, per = W.Batch(wm, ccds).logpdf(wm, per_family=True)
    rng = np.random.default_rng(0)
    pick = sorted(set(np.argsort(-n)[:6].tolist() + rng.choice(np.where(n <= 400)[0], 30, replace=False).tolist()))
    _, oper = om.logpdf([O.OracleCCD(om, wl.ale[i]) for i in pick], r.λ, r.μ, q=r.q, eta=r.η)
    assert np.sum(np.isinf(oper)) >= 2  # the largest families underflow FP64, as in the reference
    for i, o in zip(pick, oper):
        if np.isinf(o):
            assert per[i] == -np.inf, i
        else:
            assert per[i] == pytest.approx(o, rel=1e-10), i


def test_config4_gradient_small_families_against_oracle_duals(W, O, cfg4):
    wl, ccds, om, n = cfg4
    wm, r = wl.model, wl.model.rates
    small = [i for i in range(len(ccds)) if 20 <= n[i] <= 150][:8]
    g = W.gradient(wm, [ccds[i] for i in small])
    _, og = om.gradient([O.OracleCCD(om, wl.ale[i]) for i in small], r.λ, r.μ, q=r.q, eta=r.η)
    scale = np.maximum(np.abs(og), 1.0)
    assert np.max(np.abs(g - og) / scale) <= 1e-8


def test_config4_gradient_large_families_directional(W, cfg4):
    # 2,000-7,000 clades with finite log L: their adjoint tasks run from
    # device memory; the derivative along the (slightly perturbed) gradient
    # direction of the 169 parameters against central differences of the GPU
    # forward (along it the derivative is large next to the differences'
    # rounding, ~1e-10 of a total log L of ~1,400)
    wl, ccds, om, n = cfg4
    wm, r = wl.model, wl.model.rates
    cand = [i for i in np.argsort(-n) if 2000 <= n[i] <= 7000]
    fams = [ccds[i] for i in cand]
    assert np.any(6 * _task_widths(W, wm, fams, True) > SMEM_DOUBLES)
    g = W.gradient(wm, fams)
    x = np.concatenate([r.λ, r.μ, r.q, [r.η]])
    rng = np.random.default_rng(4)
    d = g / np.linalg.norm(g) + 0.1 * rng.normal(size=x.size) / np.sqrt(x.size)
    d /= np.linalg.norm(d)
    nl, nq = len(r.λ), len(r.q)

    def f(y):
        p = W.DLWGD(λ=y[:nl], μ=y[nl:2 * nl], q=y[2 * nl:2 * nl + nq], η=y[-1])
        return W.logpdf(wm(p), fams)

    h = 1e-5
    fd = (f(x + h * d) - f(x - h * d)) / (2 * h)
    assert np.isfinite(fd)
    assert float(g @ d) == pytest.approx(fd, rel=1e-6)


def test_config4_maximum_size_family(W, O, cfg4):
    # the 876-gene family of config 4's model with up to 20 NNI moves per
    # tree: ~18,000 clades, a root-task row wider than shared memory in the
    # forward too; its likelihood underflows FP64 (-Inf, as in the reference)
    from whale_gb300 import synth

    wl, _, om, _ = cfg4
    wm = wl.model
    ale = synth.simulate_families(wm, 1, 99, n_trees=500, max_nni=20, min_genes=4,
                                  target_clades=np.array([20000]), walk=True)[0]
    c = W.parse_ale_text(ale, wm)
    assert c.n_clades > 15000
    assert np.any(2 * _task_widths(W, wm, [c], False) > SMEM_DOUBLES)
    r = wm.rates
    _, oper = om.logpdf([O.OracleCCD(om, ale)], r.λ, r.μ, q=r.q, eta=r.η)
    per = W.Batch(wm, [c]).logpdf(wm, per_family=True)[1]
    assert oper[0] == -np.inf and per[0] == -np.inf
