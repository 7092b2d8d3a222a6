"""Rates models and the species-tree model (WhaleModel).

Restates the reference's parameter structs and model construction:
  ConstantDLWGD / DLWGD, getθ, getp      src/rmodels.jl:8-66
  WhaleModel(rates, tree, Δt; minn, maxn, condition)
                                          src/model.jl:96-145 (node order:
                                          leaves, then postorder; ids: non-WGD
                                          nodes first; WGD ordinals in preorder)
  Slices shape                            src/model.jl:16-22
  (m::WhaleModel)(θ)                      src/model.jl:147-160
  setsamplingp!                           src/model.jl:248-255
  Root/NonExtinct/NoCondition             src/condition.jl:1-29
The slice tables themselves (setmodel!) and the condition are evaluated by
the native library (wg_model_set_rates / wg_model_condition).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _native as N
from .newick import Node, getleaves, postwalk


# ---------------------------------------------------------------- conditions
class SamplingCondition:
    code = N.COND_ROOT


class RootCondition(SamplingCondition):
    code = N.COND_ROOT


class NonExtinctCondition(SamplingCondition):
    code = N.COND_NONEXTINCT


class NoCondition(SamplingCondition):
    code = N.COND_NONE


class NowhereExtinctCondition(SamplingCondition):
    """Probability that every leaf keeps a copy (src/condition.jl:5-9, :31-36):
    inclusion-exclusion over the joint pgf of the leaf counts at all 2^L
    binary arguments (src/bdputil.jl:114-135), computed by the library with
    its gradient on the rates.  ``NowhereExtinctCondition(tree)`` as in the
    reference; the signs are implied by the tree, so the argument is only
    checked (at most 22 leaves)."""

    code = N.COND_NOWHERE

    def __init__(self, tree=None):
        if tree is not None and len(getleaves(tree)) > 22:
            raise ValueError("NowhereExtinctCondition over more than 22 leaves (2^leaves pgf terms)")


# ---------------------------------------------------------------- rates
def _vec(x) -> np.ndarray:
    return np.asarray(x if x is not None else [], dtype=np.float64).reshape(-1).copy()


class Params:
    """Base of the rates structs; calling with a dict of fields returns an
    updated copy (``Params(θ)``, src/rmodels.jl:8-11)."""

    _fields = ()

    def __call__(self, theta: Dict) -> "Params":
        kw = {k: getattr(self, k) for k in self._fields}
        for k, v in dict(theta).items():
            k = _ALIASES.get(k, k)
            if k not in kw:
                raise KeyError(f"unknown parameter {k!r}")
            kw[k] = v
        return type(self)(**kw)


_ALIASES = {"lam": "λ", "mu": "μ", "eta": "η"}


class ConstantDLWGD(Params):
    """Constant duplication/loss rates (natural scale), WGD retention rates q
    by WGD ordinal, geometric root prior η (src/rmodels.jl:23-38)."""

    _fields = ("λ", "μ", "q", "p", "η")

    def __init__(self, λ=None, μ=None, q=None, p=None, η=0.66, lam=None, mu=None, eta=None):
        self.λ = float(lam if λ is None else λ)
        self.μ = float(mu if μ is None else μ)
        self.q = _vec(q)
        self.p = _vec(p)
        self.η = float(η if eta is None else eta)

    def __repr__(self):
        return f"ConstantDLWGD(λ={self.λ}, μ={self.μ}, q={self.q.tolist()}, η={self.η})"


class DLWGD(Params):
    """Branch-wise duplication/loss rates on log scale, indexed by node id
    (src/rmodels.jl:47-66)."""

    _fields = ("λ", "μ", "q", "p", "η")

    def __init__(self, λ=None, μ=None, q=None, p=None, η=0.66, lam=None, mu=None, eta=None):
        self.λ = _vec(lam if λ is None else λ)
        self.μ = _vec(mu if μ is None else μ)
        self.q = _vec(q)
        self.p = _vec(p)
        self.η = float(η if eta is None else eta)

    def __repr__(self):
        return f"DLWGD(λ={self.λ.tolist()}, μ={self.μ.tolist()}, q={self.q.tolist()}, η={self.η})"


def iswgd(name: str) -> bool:
    return name.startswith("wgd")  # src/model.jl:54


# ---------------------------------------------------------------- model
@dataclass
class MNode:
    pos: int          # position in the reference order
    id: int           # node id (1-based)
    wgdid: int        # WGD ordinal (0 if not a WGD)
    name: str
    kind: int
    children: List[int]
    parent: int
    nslices: int
    distance: float
    slice_len: float
    leafP: float
    clade: List[int]  # species ids


class _Structure:
    """Native model handle shared by all re-parameterisations of one tree."""

    def __init__(self, order: List[MNode], condition: SamplingCondition):
        K = len(order)
        kind = np.array([n.kind for n in order], np.int32)
        c0 = np.array([n.children[0] if n.children else -1 for n in order], np.int32)
        c1 = np.array([n.children[1] if len(n.children) > 1 else -1 for n in order], np.int32)
        nrow = np.array([n.nslices + 1 for n in order], np.int32)
        sl = np.array([n.slice_len for n in order], np.float64)
        lp = np.array([n.leafP for n in order], np.float64)
        off = np.zeros(K + 1, np.int32)
        sp: List[int] = []
        for k, n in enumerate(order):
            sp.extend(n.clade)
            off[k + 1] = len(sp)
        spa = np.array(sp if sp else [0], np.int32)
        h = N.vp()
        N.check(N.lib().wg_model_create(K, N.iptr(kind), N.iptr(c0), N.iptr(c1), N.iptr(nrow), N.dptr(sl),
                                        N.dptr(lp), N.iptr(off), N.iptr(spa), condition.code, N.C.byref(h)))
        self.h = h
        self.K = K
        self.nrow = nrow
        self.total_rows = int(nrow.sum())
        self.version = None  # id of the parameter set currently loaded

    def __del__(self):
        if getattr(self, "h", None) and N._lib is not None:
            N._lib.wg_model_destroy(self.h)
            self.h = None


class WhaleModel:
    """Species-tree model with slice discretisation (src/model.jl:71-145)."""

    def __init__(self, rates: Params, tree: Node, Δt: float = None, minn: int = 5, maxn: int = 10000,
                 condition: Optional[SamplingCondition] = None, dt: float = None, _from: "WhaleModel" = None):
        self.rates = rates
        if _from is not None:
            self.order, self.index, self.condition = _from.order, _from.index, _from.condition
            self.Δt, self.minn, self.maxn, self.tree = _from.Δt, _from.minn, _from.maxn, _from.tree
            self._struct = _from._struct
            self.spmap = _from.spmap
            return
        self.Δt = float(dt if Δt is None else Δt)
        self.minn, self.maxn = int(minn), int(maxn)
        self.condition = condition if condition is not None else RootCondition()
        self.tree = tree
        self._build(tree)
        self._struct = _Structure(self.order, self.condition)

    # ---- construction (src/model.jl:96-145)
    def _build(self, tree: Node) -> None:
        leaves = getleaves(tree)
        counts: Dict[str, int] = {}
        for l in leaves:
            counts[l.name] = counts.get(l.name, 0) + 1
        mulgroups = {k: v for k, v in counts.items() if v > 1}
        wgdid_of: Dict[int, int] = {}
        nonwgd = 0
        wgd = 0
        post: List[Node] = []

        def walk(x: Node):
            nonlocal nonwgd, wgd
            if iswgd(x.name):
                wgd += 1
                wgdid_of[id(x)] = wgd
            else:
                nonwgd += 1
                wgdid_of[id(x)] = 0
            for c in x.children:
                walk(c)
            post.append(x)

        walk(tree)
        seen = set()
        order_nodes: List[Node] = []
        for x in leaves + post:  # union(getleaves(root), postorder)
            if id(x) not in seen:
                seen.add(id(x))
                order_nodes.append(x)
        pos_of = {id(x): k for k, x in enumerate(order_nodes)}
        ids: List[int] = []
        i, j = nonwgd + 1, 1
        mulid: Dict[str, int] = {}
        for x in order_nodes:
            if iswgd(x.name):
                ids.append(i)
                i += 1
            else:
                ids.append(j)
                if x.name in mulgroups:
                    mulid[x.name] = j
                j += 1
        self.order: List[MNode] = []
        for k, x in enumerate(order_nodes):
            t = x.distance
            if math.isnan(t):
                n = 0
            else:
                n = min(self.maxn, max(self.minn, math.ceil(t / self.Δt)))
            if iswgd(x.name):
                kind = N.NODE_WGD
            elif x.parent is None:
                kind = N.NODE_ROOT
            elif x.isleaf():
                kind = N.NODE_LEAF
            else:
                kind = N.NODE_INTERNAL
            if x.name in mulgroups:
                lp = 1.0 / mulgroups[x.name]
            else:
                lp = 1.0 if x.isleaf() else 0.0
            self.order.append(MNode(pos=k, id=ids[k], wgdid=wgdid_of[id(x)], name=x.name, kind=kind,
                                    children=[pos_of[id(c)] for c in x.children],
                                    parent=-1 if x.parent is None else pos_of[id(x.parent)],
                                    nslices=n, distance=t, slice_len=(0.0 if n == 0 else t / n), leafP=lp,
                                    clade=[]))
        for m in self.order:
            if m.kind == N.NODE_INTERNAL and len(m.children) != 2:
                raise ValueError("internal speciation nodes must be binary")
            if m.kind == N.NODE_WGD and len(m.children) != 1:
                raise ValueError("a WGD node must have exactly one child")
        # clades (setclade!, src/model.jl:32-42)
        for m in self.order:
            if m.kind == N.NODE_LEAF:
                m.clade = [mulid.get(m.name, m.id)]
        for m in self.order:  # children precede parents in the order
            if m.kind != N.NODE_LEAF:
                s = set()
                for c in m.children:
                    s.update(self.order[c].clade)
                m.clade = sorted(s)
        self.index = {m.id: m.pos for m in self.order}
        # spmap: Dict(name(l)=>id(l) for l in getleaves(root(wm))) (src/ccd.jl:128)
        self.spmap: Dict[str, int] = {}
        for m in self.order:
            if m.kind == N.NODE_LEAF:
                self.spmap[m.name] = m.id
        if self.order[-1].kind != N.NODE_ROOT:
            raise ValueError("root must be last in the node order")

    # ---- API
    def __call__(self, theta) -> "WhaleModel":
        """``(m::WhaleModel)(θ)``: same structure, new parameters."""
        rates = self.rates(theta) if isinstance(theta, dict) else theta
        return WhaleModel(rates, None, _from=self)

    def __len__(self) -> int:
        return len(self.order)

    def __getitem__(self, node_id: int) -> MNode:
        return self.order[self.index[node_id]]

    def root(self) -> MNode:
        return self.order[-1]

    def getwgds(self) -> List[MNode]:
        return [n for n in self.order if n.kind == N.NODE_WGD]

    def nonwgdchild(self, k: int) -> int:
        while self.order[k].kind == N.NODE_WGD:
            k = self.order[k].children[0]
        return k

    # ---- getθ for every node (src/rmodels.jl:14, :31-33, :55-64)
    def node_rates(self, rates: Params = None):
        r = self.rates if rates is None else rates
        K = len(self.order)
        lam = np.full(K, np.nan)
        mu = np.full(K, np.nan)
        q = np.full(K, np.nan)
        p = np.zeros(K)
        for m in self.order:
            k = m.pos
            if m.kind == N.NODE_LEAF and r.p.size > 0:
                p[k] = r.p[m.id - 1]
            if isinstance(r, ConstantDLWGD):
                lam[k], mu[k] = r.λ, r.μ
                if m.kind == N.NODE_WGD:
                    q[k] = r.q[m.wgdid - 1]
                continue
            if m.kind == N.NODE_WGD:
                c = self.order[self.nonwgdchild(k)]
                lam[k], mu[k] = math.exp(r.λ[c.id - 1]), math.exp(r.μ[c.id - 1])
                q[k] = r.q[m.wgdid - 1]
            elif m.id <= r.λ.size:
                lam[k], mu[k] = math.exp(r.λ[m.id - 1]), math.exp(r.μ[m.id - 1])
        return lam, mu, q, float(r.η), p

    def load(self) -> None:
        """Fill the native slice tables from this model's rates (setmodel!)."""
        key = (id(self.rates), _rates_key(self.rates))
        if self._struct.version == key:
            return
        lam, mu, q, eta, p = self.node_rates()
        N.check(N.lib().wg_model_set_rates(self._struct.h, N.dptr(lam), N.dptr(mu), N.dptr(q), eta, N.dptr(p)))
        self._struct.version = key

    def tables(self):
        """Slice tables (ε, ϕ, ψ) of every node, concatenated in node order."""
        self.load()
        n = self._struct.total_rows
        e, f, s = np.zeros(n), np.zeros(n), np.zeros(n)
        N.check(N.lib().wg_model_get_tables(self._struct.h, N.dptr(e), N.dptr(f), N.dptr(s)))
        return e, f, s

    def condition_value(self) -> float:
        self.load()
        out = N.dbl()
        N.check(N.lib().wg_model_condition(self._struct.h, N.C.byref(out)))
        return out.value

    def setsamplingp(self, d: Dict[str, float]) -> None:
        """``setsamplingp!`` (src/model.jl:248-255)."""
        leaves = [m for m in self.order if m.kind == N.NODE_LEAF]
        if self.rates.p.size == 0:
            self.rates.p = np.zeros(len(leaves))
        for m in leaves:
            self.rates.p[m.id - 1] = d.get(m.name, 0.0)
        self._struct.version = None

    def __repr__(self) -> str:
        lines = ["WhaleModel", "—" * 10, f"⋅Parameterization:\n{self.rates}",
                 f"⋅Condition:\n{type(self.condition).__name__}", "",
                 f"⋅Model structure:\n{len(self.order)} nodes ({sum(m.kind == N.NODE_LEAF for m in self.order)} "
                 f"leaves, {len(self.getwgds())} WGD nodes)", "node_id,wgd_id,distance,Δt,n"]
        for m in self.order:
            lines.append(f"{m.id},{m.wgdid},{m.distance:.4f},{m.slice_len:.4f},{m.nslices}")
        return "\n".join(lines)


def _rates_key(r: Params):
    parts = []
    for k in r._fields:
        v = getattr(r, k)
        parts.append(v.tobytes() if isinstance(v, np.ndarray) else repr(v))
    return tuple(parts)


def condition(wm: WhaleModel) -> float:
    """``condition(wm)`` (src/condition.jl:11-29)."""
    return wm.condition_value()
