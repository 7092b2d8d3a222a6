"""Seeded synthetic workloads for the likelihood (species trees, WGD placement,
rates, and gene families with their amalgamated CCDs).

The reference publishes no benchmark data set; these generators make inputs
with the shapes its benchmark configurations describe: Yule species trees with
root age 1, WGD nodes on branches, branch-wise log-normal rates, families
simulated under the DL+WGD model with the root condition
(src/simulation.jl:27-133) and CCDs amalgamated from NNI-perturbed copies of
the true gene tree (the role ALEobserve plays for the reference,
src/ccd.jl:262-268).  Family simulation and amalgamation run natively
(wg_synth_family).
"""
from __future__ import annotations

import math
import os
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _native as N
from .ccd import CCD, parse_ale_text
from .model import ConstantDLWGD, DLWGD, RootCondition, WhaleModel
from .newick import Node, getleaves, insertnode, postwalk, prewalk


def yule_tree(n: int, rng: np.random.Generator, root_age: float = 1.0, prefix: str = "S") -> Node:
    """Ultrametric Yule tree with ``n`` leaves scaled to ``root_age``."""
    root = Node()
    tips = [(root, 0.0)]  # (node, birth time)
    t = 0.0
    born = {id(root): 0.0}
    lineages = [Node(parent=root), Node(parent=root)]
    for c in lineages:
        born[id(c)] = 0.0
    while len(lineages) < n:
        t += rng.exponential(1.0 / len(lineages))
        i = int(rng.integers(len(lineages)))
        x = lineages.pop(i)
        x.distance = t - born[id(x)]
        for _ in range(2):
            c = Node(parent=x)
            born[id(c)] = t
            lineages.append(c)
    t_end = t + rng.exponential(1.0 / len(lineages))
    for x in lineages:
        x.distance = t_end - born[id(x)]
    leaves = [x for x in prewalk(root) if x.isleaf()]
    for i, x in enumerate(leaves):
        x.name = f"{prefix}{i + 1}"
    scale = root_age / t_end
    for x in prewalk(root):
        if x.parent is not None:
            x.distance *= scale
    root.distance = math.nan
    return root


def place_wgds(tree: Node, k: int, rng: np.random.Generator, uniform_position: bool = True) -> List[Node]:
    """Insert ``k`` WGD nodes on distinct non-root branches, each at a uniform
    position along its branch (``insertnode!`` with a drawn distance)."""
    branches = [x for x in postwalk(tree) if x.parent is not None]
    pick = rng.choice(len(branches), size=k, replace=False)
    out = []
    for j, b in enumerate(sorted(pick)):
        n = branches[b]
        d = n.distance * (rng.uniform() if uniform_position else 0.5)
        out.append(insertnode(n, name=f"wgd_{j + 1}", dist=d))
    return out


@dataclass
class Workload:
    name: str
    model: WhaleModel
    ale: List[str]
    seed: int
    n_trees: int
    max_nni: int

    def ccds(self, threads: int = 0) -> List[CCD]:
        threads = threads or (os.cpu_count() or 4)
        with ThreadPoolExecutor(max_workers=threads) as ex:
            return list(ex.map(lambda i: parse_ale_text(self.ale[i], self.model, f"{self.name}_{i}.ale"),
                               range(len(self.ale))))


def simulate_families(wm: WhaleModel, n: int, seed: int, n_trees: int, max_nni: int, min_genes: int = 3,
                      target_clades: Optional[np.ndarray] = None, walk: bool = False, threads: int = 0,
                      indices: Optional[Sequence[int]] = None) -> List[str]:
    """ALE texts of ``n`` families simulated on ``wm`` (native, threaded);
    with ``indices``, only those families of the ``n`` (each family depends
    on its index alone)."""
    lam, mu, q, eta, _ = wm.node_rates()
    q = np.where(np.isnan(q), 0.0, q)
    lam = np.where(np.isnan(lam), 0.0, lam)
    mu = np.where(np.isnan(mu), 0.0, mu)
    names = [m.name if m.kind == N.NODE_LEAF else "" for m in wm.order]
    enc = (N.C.c_char_p * len(names))(*[s.encode() for s in names])
    L = N.lib()

    def one(i: int) -> str:
        s = np.uint64((seed * 1000003 + i * 7919 + 17) % (1 << 63))
        tgt = int(target_clades[i]) if target_clades is not None else 0
        need = N.i64()
        cap = 1 << 20
        while True:
            buf = N.C.create_string_buffer(cap)
            flags = (N.SYNTH_WALK | N.SYNTH_PUSH) if walk else 0
            N.check(L.wg_synth_family(wm._struct.h, N.dptr(lam), N.dptr(mu), N.dptr(q), eta, enc, int(s), n_trees,
                                      max_nni, min_genes, tgt, flags, buf, cap, N.C.byref(need)))
            if need.value < cap:
                return buf.value.decode()
            cap = int(need.value) + 1

    threads = threads or (os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(one, range(n) if indices is None else list(indices)))


def config0(seed: int = 0, n_families: int = 100) -> Workload:
    """9-taxon Yule tree, one WGD halfway up a fixed internal branch (q=0.2),
    ConstantDLWGD λ=0.2, μ=0.3, η=0.67, Δt=0.05; CCDs from 100 trees with
    0-3 NNIs."""
    rng = np.random.default_rng(seed)
    t = yule_tree(9, rng)
    internal = [x for x in postwalk(t) if x.parent is not None and not x.isleaf()]
    insertnode(internal[0], name="wgd_1")
    r = ConstantDLWGD(λ=0.2, μ=0.3, q=[0.2], η=0.67)
    wm = WhaleModel(r, t, 0.05, condition=RootCondition())
    ale = simulate_families(wm, n_families, seed, n_trees=100, max_nni=3)
    return Workload("cfg0", wm, ale, seed, 100, 3)


def _dlwgd_model(ntaxa: int, nwgd: int, dt: float, rng: np.random.Generator) -> WhaleModel:
    t = yule_tree(ntaxa, rng)
    wg = place_wgds(t, nwgd, rng)
    nnodes = 2 * ntaxa - 1
    lam = rng.normal(math.log(0.2), 0.5, size=nnodes)
    mu = rng.normal(math.log(0.2), 0.5, size=nnodes)
    q = rng.uniform(0.05, 0.5, size=nwgd)
    r = DLWGD(λ=lam, μ=mu, q=q, η=0.67)
    return WhaleModel(r, t, dt, condition=RootCondition())


def config1(seed: int = 1, n_families: int = 5000) -> Workload:
    """17-taxon Yule tree, Δt=0.02, 3 WGDs at uniform positions on distinct
    branches with q ~ U(0.05, 0.5), branch-wise λ, μ = exp(N(log 0.2, 0.5²)),
    η=0.67; CCDs from 200 trees with 0-5 NNIs, target clade counts
    log-uniform in [10, 2000].  To reach the target the tree sample is a
    random walk of NNI moves (each tree perturbs the previous one) that takes
    the maximum move count until the target is reached and no moves after."""
    rng = np.random.default_rng(seed)
    wm = _dlwgd_model(17, 3, 0.02, rng)
    tgt = np.exp(rng.uniform(math.log(10), math.log(2000), size=n_families)).astype(np.int64)
    ale = simulate_families(wm, n_families, seed, n_trees=200, max_nni=5, min_genes=4, target_clades=tgt,
                            walk=True)
    return Workload("cfg1", wm, ale, seed, 200, 5)


def config4_targets(seed: int = 4, n_families: int = 50000) -> np.ndarray:
    """Target clade counts of config4's families (Pareto tail, α = 0.8,
    capped at 20,000)."""
    rng = np.random.default_rng(seed)
    _dlwgd_model(40, 10, 0.01, rng)
    u = rng.uniform(size=n_families)
    return np.minimum(20000, 10.0 * np.power(1.0 - u, -1.0 / 0.8)).astype(np.int64)


def config4(seed: int = 4, n_families: int = 50000, indices: Optional[Sequence[int]] = None) -> Workload:
    """40-taxon Yule tree, Δt=0.01, 10 WGDs, rates as config1; CCDs from 500
    trees with 0-8 NNIs, heavy-tailed clade counts in [10, 20000].  With
    ``indices``, only those families of the 50,000 (identical to theirs in
    the full workload)."""
    rng = np.random.default_rng(seed)
    wm = _dlwgd_model(40, 10, 0.01, rng)
    u = rng.uniform(size=n_families)
    tgt = np.minimum(20000, 10.0 * np.power(1.0 - u, -1.0 / 0.8)).astype(np.int64)
    ale = simulate_families(wm, n_families, seed, n_trees=500, max_nni=8, min_genes=4, target_clades=tgt,
                            walk=True, indices=indices)
    return Workload("cfg4", wm, ale, seed, 500, 8)
