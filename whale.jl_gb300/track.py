"""Sampling reconciled gene trees from the DP tables (backtracking,
src/track.jl:180-488).

``backtrack(wm, ccd, n=1, seed=0)`` evaluates the family with its tables kept
(``logpdf!``) and draws ``n`` reconciled trees: every latent state (species
node, clade, slice) draws the event that produced it with probability
proportional to its term in the DP recursion, in the reference's event order.
Trees come back as ``RecNode`` trees (labels ``speciation``, ``duplication``,
``wgd``, ``wgdloss``, ``sploss``, ``loss``; branch lengths from the
reference's node heights) and as extended Newick text.  Randomness is the
library's own stream: trees match the reference in distribution.
"""
from __future__ import annotations

import ctypes as C
import re
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Union

from . import _native as N
from .ccd import CCD
from .core import get_batch
from .model import WhaleModel


@dataclass
class RecNode:
    name: str
    label: str
    node: int          # species-tree node, position in ``wm.order``
    species: str       # name of that node ("" for internal nodes without a name)
    clade: int         # 0-based clade of the CCD, -1 for a loss
    slice: int         # slice where the branch leading to this node starts
    distance: float
    children: List["RecNode"] = field(default_factory=list)

    def isleaf(self) -> bool:
        return not self.children

    def postwalk(self):
        for c in self.children:
            yield from c.postwalk()
        yield self


def _parse(text: str, wm: WhaleModel) -> RecNode:
    pos = 0

    def node_from(tok: str) -> RecNode:
        name, attrs, dist = tok, {}, 0.0
        m = re.match(r"^([^\[:]*)(?:\[&&NHX:([^\]]*)\])?(?::([-+0-9.eE]+))?$", tok)
        if m:
            name = m.group(1)
            if m.group(2):
                attrs = dict(kv.split("=", 1) for kv in m.group(2).split(":"))
            if m.group(3):
                dist = float(m.group(3))
        k = int(attrs.get("node", -1))
        sp = wm.order[k].name if 0 <= k < len(wm.order) else ""
        return RecNode(name, attrs.get("label", ""), k, sp or "", int(attrs.get("clade", -1)),
                       int(attrs.get("slice", 0)), dist)

    def sub() -> RecNode:
        nonlocal pos
        children = []
        if text[pos] == "(":
            pos += 1
            while True:
                children.append(sub())
                if text[pos] == ",":
                    pos += 1
                    continue
                if text[pos] == ")":
                    pos += 1
                    break
                raise ValueError("malformed reconciled tree")
        m = re.match(r"[^(),;]*", text[pos:])
        tok = m.group(0)
        pos += len(tok)
        n = node_from(tok)
        n.children = children
        return n

    root = sub()
    if text[pos] != ";":
        raise ValueError("malformed reconciled tree")
    return root


@dataclass
class RecTree:
    newick: str
    root: RecNode


def backtrack_tables(wm: WhaleModel, ccd: CCD, tables, n: int = 1, seed: int = 0) -> List[RecTree]:
    """Sampling from DP tables already at hand (the ``logpdf!`` layout of
    ``Batch.family_tables``), on the host."""
    import numpy as np

    wm.load()
    t = np.ascontiguousarray(tables, dtype=np.float64)
    need = N.i64()
    L = N.lib()
    N.check(L.wg_backtrack_tables(wm._struct.h, ccd._h, N.dptr(t), t.size, int(n), C.c_uint64(seed), None, 0,
                                  C.byref(need)))
    buf = C.create_string_buffer(need.value)
    N.check(L.wg_backtrack_tables(wm._struct.h, ccd._h, N.dptr(t), t.size, int(n), C.c_uint64(seed), buf,
                                  need.value, C.byref(need)))
    return [RecTree(ln, _parse(ln, wm)) for ln in buf.value.decode().split("\n") if ln]


def backtrack(wm: WhaleModel, x: Union[CCD, Sequence[CCD]], n: int = 1, seed: int = 0):
    """``backtrack(wm, ccd)`` (src/track.jl:188-194): ``n`` sampled reconciled
    trees of one family (a list of RecTree); for a vector of CCDs, one such
    list per family."""
    if not isinstance(x, CCD):
        return [backtrack(wm, c, n, seed + 7919 * i) for i, c in enumerate(x)]
    wm.load()
    b = get_batch(wm, [x], tables=True)
    need = N.i64()
    L = N.lib()
    N.check(L.wg_backtrack(b.ctx.h, wm._struct.h, b.h, 0, int(n), C.c_uint64(seed), None, 0, C.byref(need)))
    buf = C.create_string_buffer(need.value)
    N.check(L.wg_backtrack(b.ctx.h, wm._struct.h, b.h, 0, int(n), C.c_uint64(seed), buf, need.value,
                           C.byref(need)))
    lines = [ln for ln in buf.value.decode().split("\n") if ln]
    return [RecTree(ln, _parse(ln, wm)) for ln in lines]


# ---- TreeTracker (src/track.jl:11-82) and tree summaries (src/rectree.jl) ----

LABELS = ("loss", "wgd", "wgdloss", "duplication", "sploss", "speciation")  # src/track.jl:468


@dataclass
class TrackSummary:
    """``RecSummary`` (src/rectree.jl:4-8) of one family's sampled trees.

    trees: the distinct reconciled trees, most frequent first, as
    (frequency, RecTree); credibility: for each of them, per node in
    postorder, the fraction of all samples holding that node (the
    reference's ``cred``); events: per label (LABELS), the expected number of
    such events on every species node (``wm.order`` positions), i.e. the
    frequency-weighted event counts of the distinct trees (the mean over the
    samples); counts: the same counts per distinct tree."""
    fname: str
    trees: List[tuple]
    credibility: List[List[float]]
    events: dict
    counts: List[dict]


def _node_key(n: RecNode, sister: Optional[RecNode]):
    # src/track.jl:111-113: a loss is its branch and its sister's clade; any
    # other node its clade, branch and its children's (clade, branch) pairs
    if n.label == "loss":
        return (-1, n.node, sister.clade if sister is not None else -2)
    return (n.clade, n.node, frozenset((c.clade, c.node) for c in n.children))


def _node_keys(root: RecNode):
    out = []

    def walk(n: RecNode, sister: Optional[RecNode]):
        for i, c in enumerate(n.children):
            s = n.children[1 - i] if len(n.children) == 2 else None
            walk(c, s)
        out.append(_node_key(n, sister))

    walk(root, None)
    return out


def sumtrees(trees: Sequence[RecTree], ccd: CCD, wm: WhaleModel) -> TrackSummary:
    """``sumtrees`` (src/rectree.jl:123-143): distinct trees (by the set of
    their node keys, as ``nodehash``), their frequencies, node credibilities
    and event counts per species node."""
    import numpy as np

    n = len(trees)
    if n == 0:
        raise ValueError("no trees to summarise")
    keys = [_node_keys(t.root) for t in trees]
    tkeys = [frozenset(k) for k in keys]
    clade_count = {}
    for k in keys:
        for x in k:
            clade_count[x] = clade_count.get(x, 0) + 1
    first, count = {}, {}
    for i, tk in enumerate(tkeys):
        first.setdefault(tk, i)
        count[tk] = count.get(tk, 0) + 1
    order = sorted(count, key=lambda tk: (-count[tk], first[tk]))
    K = len(wm.order)
    events = {lab: np.zeros(K) for lab in LABELS}
    out_trees, cred, counts = [], [], []
    for tk in order:
        t = trees[first[tk]]
        f = count[tk] / n
        c = {lab: np.zeros(K, dtype=np.int64) for lab in LABELS}
        for node in t.root.postwalk():
            if node.label in c and 0 <= node.node < K:
                c[node.label][node.node] += 1
        for lab in LABELS:
            events[lab] += f * c[lab]
        out_trees.append((f, t))
        cred.append([clade_count[x] / n for x in keys[first[tk]]])
        counts.append(c)
    return TrackSummary(getattr(ccd, "fname", ""), out_trees, cred, events, counts)


def _draw_seed(seed: int, j: int, f: int) -> int:
    return (seed * 0x9E3779B97F4A7C15 + j * 0xBF58476D1CE4E5B9 + f * 0x94D049BB133111EB + 1) % (1 << 64)


def track_tables(tables_of, wm: WhaleModel, ccds: Sequence[CCD], draws: Sequence, n: int, fun=None, seed: int = 0,
                 summary: bool = True, threads: int = 0):
    """``track`` with the DP tables from ``tables_of(model, f)`` (family f's
    tables under ``model``, in the ``logpdf!`` layout).  Per pick, the
    families' tables are fetched in turn, then sampled on ``threads`` host
    threads (0: every core); every tree has its own seed, so the trees do not
    depend on the thread count."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np

    if len(draws) == 0:
        raise ValueError("no posterior draws")
    rng = np.random.default_rng(seed)
    picks = rng.integers(len(draws), size=int(n))
    trees = [[] for _ in ccds]
    nt = max(1, min(threads or (os.cpu_count() or 1), len(ccds)))
    with ThreadPoolExecutor(max_workers=nt) as pool:
        for j, i in enumerate(picks):
            m = fun(wm, draws[i]) if fun is not None else wm(draws[i])
            tabs = [tables_of(m, f) for f in range(len(ccds))]
            m.load()  # before the threads: they only read the model

            def sample(f, m=m, tabs=tabs, j=j):
                return backtrack_tables(m, ccds[f], tabs[f], n=1, seed=_draw_seed(seed, j, f))

            for f, t in enumerate(pool.map(sample, range(len(ccds)))):
                trees[f] += t
    if not summary:
        return trees
    return [sumtrees(t, c, wm) for t, c in zip(trees, ccds)]


def sample_device(b, wm: WhaleModel, families: Sequence[int], seeds: Sequence[int]):
    """One reconciled tree per (family, seed) sampled on the device from the
    tables of the batch's last fetched evaluation (wg_track_device); each
    equals ``backtrack_tables(..., n=1, seed)`` on the same tables.  Returns
    the node arrays (per tree an (n, 4) int32 array: clade, species node,
    slice, parent)."""
    import numpy as np

    fam = np.ascontiguousarray(families, dtype=np.int32)
    sd = np.ascontiguousarray(seeds, dtype=np.uint64)
    off = np.zeros(fam.size + 1, dtype=np.int64)
    L = N.lib()
    N.check(L.wg_track_device(b.ctx.h, wm._struct.h, b.h, int(fam.size), N.iptr(fam),
                              sd.ctypes.data_as(C.POINTER(C.c_uint64)), N.lptr(off)))
    nodes = np.zeros((max(int(off[-1]), 1), 4), dtype=np.int32)
    N.check(L.wg_track_nodes(b.h, nodes.ctypes.data_as(N.P_i32), nodes.shape[0]))
    return [nodes[off[i]:off[i + 1]] for i in range(fam.size)]


def tree_of_nodes(wm: WhaleModel, ccd: CCD, nodes) -> RecTree:
    """A sampled tree's node arrays as a RecTree (wg_tree_newick)."""
    import numpy as np

    a = np.ascontiguousarray(nodes, dtype=np.int32)
    L = N.lib()
    need = N.i64()
    N.check(L.wg_tree_newick(wm._struct.h, ccd._h, a.ctypes.data_as(N.P_i32), a.shape[0], None, 0, C.byref(need)))
    buf = C.create_string_buffer(need.value)
    N.check(L.wg_tree_newick(wm._struct.h, ccd._h, a.ctypes.data_as(N.P_i32), a.shape[0], buf, need.value,
                             C.byref(need)))
    text = buf.value.decode()
    return RecTree(text, _parse(text, wm))


def track(wm: WhaleModel, ccds: Sequence[CCD], draws: Sequence, n: int, fun=None, seed: int = 0,
          summary: bool = True, threads: int = 0, device: bool = True):
    """``track(TreeTracker(wm, ccds, draws, fun), n)`` (src/track.jl:11-82):
    ``n`` reconciled trees per family from the posterior predictive, each
    under a draw picked uniformly from ``draws`` (``fun(wm, draw)`` gives the
    model of a draw, by default ``wm(draw)``), summarised per family
    (``sumtrees``) unless ``summary`` is false.

    The loops run the other way round from the reference's, as its own
    comment (src/track.jl:18-21) says would be faster: for each of the ``n``
    picks, one batched ``logpdf!`` of every family on the device, then one
    tree per family from its tables on ``threads`` host threads (0: every
    core).  All families of a pick share
    its draw (the reference picks per family): each family's trees have the
    same distribution.  The same seed gives the same trees.

    With ``device`` (the default) every pick's trees are sampled on the GPU,
    one thread per family, from the tables in device memory
    (wg_track_device); only the sampled node arrays come back.  Otherwise
    each family's tables are downloaded and sampled on host threads.  Both
    give the same trees."""
    wm.load()
    b = get_batch(wm, list(ccds), tables=True)
    if device:
        import numpy as np

        if len(draws) == 0:
            raise ValueError("no posterior draws")
        picks = np.random.default_rng(seed).integers(len(draws), size=int(n))
        trees = [[] for _ in ccds]
        fams = list(range(len(ccds)))
        for j, i in enumerate(picks):
            m = fun(wm, draws[i]) if fun is not None else wm(draws[i])
            b.logpdf(m)
            arrs = sample_device(b, m, fams, [_draw_seed(seed, j, f) for f in fams])
            for f, a in enumerate(arrs):
                trees[f].append(tree_of_nodes(m, ccds[f], a))
        if not summary:
            return trees
        return [sumtrees(t, c, wm) for t, c in zip(trees, ccds)]
    state = {"model": None}

    def tables_of(m, f):
        if state["model"] is not m:
            b.logpdf(m)
            state["model"] = m
        return b.last_tables(f)[1]

    return track_tables(tables_of, wm, ccds, draws, n, fun=fun, seed=seed, summary=summary, threads=threads)


def pair_labels(wm: WhaleModel) -> List[str]:
    """Event labels of ``getpairs`` (src/rectree.jl:52-62): per species node
    (its id), ``<id>_duplication`` and ``<id>_wgd``, ``<id>_wgdloss`` for a WGD
    node or ``<id>_speciation`` otherwise."""
    out = []
    for m in wm.order:
        out.append(f"{m.id}_duplication")
        out += [f"{m.id}_wgd", f"{m.id}_wgdloss"] if m.kind == N.NODE_WGD else [f"{m.id}_speciation"]
    return out


def _leaves(n: RecNode):
    return [x for x in n.postwalk() if x.isleaf()]


def getpairs(summaries: Sequence[TrackSummary], wm: WhaleModel, digits: int = 3):
    """``getpairs`` (src/rectree.jl:52-97): for every pair of surviving genes
    of a family, the posterior probability that the pair's split node in the
    reconciled tree is each event on each species node (``pair_labels``),
    rounded to ``digits`` as the reference does.  One (family, pairs, labels,
    pp) tuple per summary: pp[p, l] for pair p (``"a__b"``, names sorted) and
    label l; each row sums to 1 up to the rounding."""
    import numpy as np

    labels = pair_labels(wm)
    lab_ix = {l: i for i, l in enumerate(labels)}
    out = []
    for s in summaries:
        first = [x for x in _leaves(s.trees[0][1].root) if x.label != "loss"]
        pairs = ["__".join(sorted([first[i].name, first[j].name])) for i in range(len(first)) for j in range(i)]
        pix = {p: i for i, p in enumerate(pairs)}
        pp = np.zeros((len(pairs), len(labels)))
        for f, t in s.trees:
            for n in t.root.postwalk():
                if len(n.children) != 2:
                    continue
                a = [x for x in _leaves(n.children[0]) if x.label != "loss"]
                b = [x for x in _leaves(n.children[1]) if x.label != "loss"]
                if not a or not b:
                    continue
                col = lab_ix.get(f"{wm.order[n.node].id}_{n.label}")
                if col is None:
                    raise ValueError(f"pair split at a {n.label!r} node")
                for x in a:
                    for y in b:
                        pp[pix["__".join(sorted([x.name, y.name]))], col] += f
        out.append((s.fname, pairs, labels, np.round(pp, digits)))
    return out
