"""The gradient as a sampler uses it (config 3: successive leapfrog
evaluations with the log-rates moving): leapfrog trajectories of
H(θ, m) = -log p(θ) + |m|²/2 over config 1's 70 parameters, log p = Σ log L -
N·condition of 500 config-1 families.  With the exact gradient the
integrator is second order: its energy error over a fixed trajectory length
falls as ε², so halving ε divides it by about 4; it is also reversible (the
trajectory run back returns to its start).  Both hold only if every
gradient entry is the derivative of the value the library returns."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def target(W):
    from whale_gb300 import synth

    wl = synth.config1(n_families=500)
    wm = wl.model
    r = wm.rates
    nl, nq = len(r.λ), len(r.q)
    x0 = np.concatenate([r.λ, r.μ, r.q, [r.η]])

    def logp_grad(x):
        m = wm(W.DLWGD(λ=x[:nl], μ=x[nl:2 * nl], q=x[2 * nl:2 * nl + nq], η=x[-1]))
        tot, g = W.logpdf_gradient(m, ccds)
        return tot, np.concatenate([g["λ"], g["μ"], g["q"], [g["η"]]])

    ccds = wl.ccds()
    return x0, logp_grad


def _leapfrog(logp_grad, x, m, eps, n):
    lp, g = logp_grad(x)
    h0 = -lp + 0.5 * m @ m
    for _ in range(n):
        m = m + 0.5 * eps * g
        x = x + eps * m
        lp, g = logp_grad(x)
        m = m + 0.5 * eps * g
    return x, m, (-lp + 0.5 * m @ m) - h0


def test_leapfrog_energy_error_is_second_order(target):
    x0, logp_grad = target
    rng = np.random.default_rng(6)
    m0 = rng.normal(size=x0.size)
    T = 4e-3  # trajectory length: many gradient evaluations, a small move of the rates
    errs = []
    for n in (8, 16, 32):
        _, _, dh = _leapfrog(logp_grad, x0, m0, T / n, n)
        errs.append(abs(dh))
    assert all(np.isfinite(errs))
    r1, r2 = errs[0] / errs[1], errs[1] / errs[2]
    assert 3.0 < r1 < 5.5 and 3.0 < r2 < 5.5, (errs, r1, r2)


def test_leapfrog_is_reversible(target):
    x0, logp_grad = target
    rng = np.random.default_rng(7)
    m0 = rng.normal(size=x0.size)
    x1, m1, _ = _leapfrog(logp_grad, x0, m0, 2e-4, 10)
    x2, m2, _ = _leapfrog(logp_grad, x1, -m1, 2e-4, 10)
    assert np.max(np.abs(x2 - x0)) < 1e-9 * max(1.0, np.max(np.abs(x0)))
    assert np.max(np.abs(m2 + m0)) < 1e-7 * max(1.0, np.max(np.abs(m0)))
