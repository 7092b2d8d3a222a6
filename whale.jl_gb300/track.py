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
