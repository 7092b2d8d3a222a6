"""Likelihoods over several WhaleModels (src/core.jl:66-79).

``MixtureModel``: every family comes from one of K components (WhaleModels
on the same species tree and discretisation, e.g. different rates):
``logpdf = Σ_i logsumexp_j (log L_ij + log p_j - condition_j)``.
``ModelArray``: family i has its own model; ``logpdf = Σ_i log L_i`` with the
single-CCD (unconditioned) form of each term.

Both run on the batched GPU path: the components share one device batch
(packed for the first component; the batch only depends on the tree and the
slices), and gradients use the weighted adjoint (``wg_logpdf_grad_weighted``),
whose seeds are the per-family posterior weights of each component.
"""
from __future__ import annotations

from typing import Dict, List, Sequence, Tuple

import numpy as np

from .ccd import CCD
from .core import get_batch, map_gradient
from .model import WhaleModel


def _lhood(x: float) -> float:
    # ℓhood (src/core.jl:15): non-finite totals map to -Inf
    return float(x) if np.isfinite(x) else float("-inf")


def _logsumexp_rows(a: np.ndarray) -> np.ndarray:
    m = np.max(a, axis=1)
    out = np.full(a.shape[0], -np.inf)
    ok = np.isfinite(m)
    out[ok] = m[ok] + np.log(np.sum(np.exp(a[ok] - m[ok, None]), axis=1))
    return out


class MixtureModel:
    """``MixtureModel(components, prior)`` as Distributions.MixtureModel over
    WhaleModels (src/core.jl:66)."""

    def __init__(self, components: Sequence[WhaleModel], prior: Sequence[float]):
        self.components = list(components)
        self.prior = np.asarray(prior, dtype=np.float64)
        if len(self.components) == 0 or self.prior.shape != (len(self.components),):
            raise ValueError("one prior probability per component")
        if np.any(self.prior < 0) or not np.isclose(self.prior.sum(), 1.0):
            raise ValueError("prior probabilities must be non-negative and sum to 1")
        s0 = self.components[0]._struct
        for wm in self.components[1:]:
            if wm._struct.total_rows != s0.total_rows or len(wm.order) != len(self.components[0].order):
                raise ValueError("mixture components must share the species tree and slices")

    def _terms(self, xs: Sequence[CCD]) -> np.ndarray:
        """a_ij = log L_ij + log p_j - condition_j (families × components)."""
        b = get_batch(self.components[0], list(xs))
        a = np.empty((len(xs), len(self.components)))
        with np.errstate(divide="ignore"):
            logp = np.log(self.prior)
        for j, wm in enumerate(self.components):
            _, per = b.logpdf(wm, per_family=True)
            a[:, j] = per + logp[j] - wm.condition_value()
        return a


def logpdf(mm: MixtureModel, xs: Sequence[CCD]) -> float:
    """Σ_i logsumexp_j (log L_ij + log p_j - condition_j) (src/core.jl:66-75)."""
    return _lhood(np.sum(_logsumexp_rows(mm._terms(xs))))


def logpdf_gradient(mm: MixtureModel, xs: Sequence[CCD]) -> Tuple[float, List[Dict], np.ndarray]:
    """The mixture log-likelihood, the gradient w.r.t. each component's rates
    struct (as ``core.logpdf_gradient``) and w.r.t. the prior probabilities."""
    xs = list(xs)
    a = mm._terms(xs)
    lse = _logsumexp_rows(a)
    total = _lhood(np.sum(lse))
    w = np.zeros_like(a)
    ok = np.isfinite(lse)
    w[ok] = np.exp(a[ok] - lse[ok, None])  # posterior component weight of each family
    b = get_batch(mm.components[0], xs, grad=True)
    grads = []
    for j, wm in enumerate(mm.components):
        _, _, dl, dm, dq, de = b.grad_nodes_weighted(wm, w[:, j], float(np.sum(w[:, j])))
        grads.append(map_gradient(wm, dl, dm, dq, de))
    with np.errstate(divide="ignore", invalid="ignore"):
        dprior = np.where(mm.prior > 0, np.sum(w, axis=0) / mm.prior, np.inf)
    return total, grads, dprior


class ModelArray:
    """``ModelArray(models)``: family i is scored by models[i] (src/core.jl:77-78)."""

    def __init__(self, models: Sequence[WhaleModel]):
        self.models = list(models)

    def _groups(self, n: int):
        if len(self.models) != n:
            raise ValueError("one model per family")
        groups: Dict[int, Tuple[WhaleModel, List[int]]] = {}
        for i, wm in enumerate(self.models):
            groups.setdefault(id(wm), (wm, []))[1].append(i)
        return list(groups.values())


def modelarray_logpdf(ma: ModelArray, xs: Sequence[CCD]) -> float:
    """Σ_i log L(models[i], xs[i]), each term unconditioned (src/core.jl:39, :77-78)."""
    xs = list(xs)
    total = 0.0
    for wm, idx in ma._groups(len(xs)):
        _, per = get_batch(wm, [xs[i] for i in idx]).logpdf(wm, per_family=True)
        total += float(np.sum(per))
    return _lhood(total)


def modelarray_logpdf_gradient(ma: ModelArray, xs: Sequence[CCD]) -> Tuple[float, List[Tuple[WhaleModel, Dict]]]:
    """The ModelArray log-likelihood and, per distinct model, the gradient of
    the sum of its families' unconditioned log-likelihoods."""
    xs = list(xs)
    total = 0.0
    out = []
    for wm, idx in ma._groups(len(xs)):
        b = get_batch(wm, [xs[i] for i in idx], grad=True)
        _, per, dl, dm, dq, de = b.grad_nodes_weighted(wm, np.ones(len(idx)), 0.0)
        total += float(np.sum(per))
        out.append((wm, map_gradient(wm, dl, dm, dq, de)))
    return _lhood(total), out
