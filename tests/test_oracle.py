"""The CPU oracle against the reference's own pinned values and properties
(test/runtests.jl).  These pin the oracle before it is trusted as the checker
of the CUDA path."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, REFERENCE, read

EX1_OTHER_ORDER = ("((MPOL:4.752,PPAT:4.752):0.292,(SMOE:4.457,((((OSAT:1.555,((ATHA:0.2774)wgd_1:0.2774,"
                   "CPAP:0.5548):1.0002):0.738,ATRI:2.293):0.6125)wgd_2:0.6125,(GBIL:3.178,PABI:3.178):0.34)"
                   ":0.939):0.587);")


def test_single_family_golden(O, ex1_tree, ex1_files, golden):
    # test/runtests.jl:15-19: maxn=5, first file in readdir order, no condition
    g = golden["single_family"]
    m = O.OracleModel(ex1_tree, g["dt"], maxn=g["maxn"])
    c = O.read_ale_files(m, ex1_files[:1])
    n = g["n_rates"]
    _, per = m.logpdf(c, np.ones(n), np.ones(n), q=g["q"], eta=g["eta"])
    assert per[0] == pytest.approx(g["logpdf"], rel=1e-12)


def test_twelve_families_golden(O, ex1_tree, ex1_files, golden):
    # test/runtests.jl:21-34: RootCondition, 12 families
    g = golden["twelve_families"]
    m = O.OracleModel(ex1_tree, g["dt"], maxn=g["maxn"], condition="root")
    cs = O.read_ale_files(m, ex1_files)
    assert len(cs) == 12
    n = g["n_rates"]
    tot, _ = m.logpdf(cs, np.ones(n), np.ones(n), q=g["q"], eta=g["eta"])
    assert tot == pytest.approx(g["logpdf"], rel=1e-12)


def test_child_order_invariance(O, ex1_files, golden):
    # the likelihood does not depend on the order of children (equal rates)
    g = golden["twelve_families"]
    m = O.OracleModel(EX1_OTHER_ORDER, g["dt"], condition="root")
    cs = O.read_ale_files(m, ex1_files)
    tot, _ = m.logpdf(cs, np.ones(17), np.ones(17), q=g["q"], eta=g["eta"])
    assert tot == pytest.approx(g["logpdf"], rel=1e-12)


def test_root_rates_have_no_effect(O, ex1_tree, ex1_files, golden):
    # test/runtests.jl:44-49
    g = golden["twelve_families"]
    m = O.OracleModel(ex1_tree, g["dt"], condition="root")
    cs = O.read_ale_files(m, ex1_files)
    lam, mu = np.ones(17), np.ones(17)
    root_id = int(m.ids[-1])
    lam[root_id - 1] = np.nan
    mu[root_id - 1] = np.nan
    tot, _ = m.logpdf(cs, lam, mu, q=g["q"], eta=g["eta"])
    assert tot == pytest.approx(g["logpdf"], rel=1e-12)


def test_gradient_finite_and_matches_fd(O, ex1_tree, ex1_files):
    # test/runtests.jl:36-39 (finite) + central differences for the dual numbers
    m = O.OracleModel(ex1_tree, 0.05, condition="root")
    cs = O.read_ale_files(m, ex1_files[:4])
    x = np.r_[np.ones(17), np.ones(17), [0.1, 0.2], 0.8]
    # off the critical line |λ - μ| <= 1e-6 (src/bdputil.jl:6-7), where the
    # reference's branch makes the dual derivative differ from differences
    x[:17] += np.linspace(-0.3, 0.3, 17) + 0.01
    tot, g = m.gradient(cs, x[:17], x[17:34], q=x[34:36], eta=x[36])
    assert np.all(np.isfinite(g))
    h = 1e-6
    fd = np.zeros_like(x)
    for i in range(x.size):
        xp, xm = x.copy(), x.copy()
        xp[i] += h
        xm[i] -= h
        fp, _ = m.logpdf(cs, xp[:17], xp[17:34], q=xp[34:36], eta=xp[36])
        fm, _ = m.logpdf(cs, xm[:17], xm[17:34], q=xm[34:36], eta=xm[36])
        fd[i] = (fp - fm) / (2 * h)
    assert np.allclose(g, fd, rtol=1e-5, atol=1e-5)


def test_discretisation_stable(O):
    # test/runtests.jl:128-144 (example-5, all branches of length 1)
    nw = read(os.path.join(GOLDEN, "example5_tree.nw")).strip()
    import re

    nw1 = re.sub(r":[0-9.eE+-]+", ":1.0", nw)
    rng = np.random.default_rng(5)
    for _ in range(3):
        vals = []
        for e in np.arange(-3.0, -0.99, 0.5):
            m = O.OracleModel(nw1, 10 ** e, condition="root")
            cs = O.read_ale_files(m, [os.path.join(GOLDEN, "example5", "OG0014587.ale")])
            n = int(m.nonwgd)
            r = rng.normal(size=n) if not vals else r
            tot, _ = m.logpdf(cs, r, r, q=[], eta=0.9)
            vals.append(tot)
        assert np.all(np.abs(np.array(vals) - vals[0]) < 0.1)


@pytest.mark.skipif(not REFERENCE or not os.path.isdir(REFERENCE), reason="WHALE_REFERENCE_DIR not set")
def test_fixtures_equal_reference_files(O, ex1_tree, golden):
    # the normalised fixtures give the same likelihood as the reference's files
    src = os.path.join(REFERENCE, "example", "example-1", "ale")
    files = [os.path.join(src, f) for f in sorted(os.listdir(src))]
    m = O.OracleModel(ex1_tree, 0.05, condition="root")
    tot, per = m.logpdf(O.read_ale_files(m, files), np.ones(17), np.ones(17), q=[0.2, 0.1], eta=0.9)
    assert tot == pytest.approx(golden["twelve_families"]["logpdf"], rel=1e-12)


@pytest.mark.skipif(not REFERENCE or not os.path.isdir(REFERENCE), reason="WHALE_REFERENCE_DIR not set")
@pytest.mark.parametrize("sub,src,tree", [("example4", "example/example-4", "example4_tree.nw"),
                                          ("landplant", "docs/data/landplant/100fams", "landplant_tree.nw")])
def test_real_data_fixtures_equal_reference_files(O, sub, src, tree):
    # the normalised fixtures give the same per-family likelihood as the files
    nw = read(os.path.join(GOLDEN, tree)).strip()
    m = O.OracleModel(nw, 0.1, condition="root")
    n = int(m.nonwgd)
    d = os.path.join(REFERENCE, src)
    orig = [os.path.join(d, f) for f in sorted(os.listdir(d)) if f.endswith(".ale")]
    mine = [os.path.join(GOLDEN, sub, os.path.basename(f)) for f in orig]
    rates = (np.full(n, np.log(0.2)), np.full(n, np.log(0.25)))
    _, a = m.logpdf(O.read_ale_files(m, orig), *rates, q=[], eta=0.7)
    _, b = m.logpdf(O.read_ale_files(m, mine), *rates, q=[], eta=0.7)
    assert np.array_equal(a, b) and np.all(np.isfinite(a))

