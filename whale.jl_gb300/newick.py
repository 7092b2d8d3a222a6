"""Species trees in Newick form, with the node operations the reference's
model construction relies on (NewickTree 0.3.1, Manifest.toml:1061-1065):
``readnw``, ``nwstr``, ``postwalk``/``prewalk``, ``getleaves``, ``getlca``,
``insertnode`` (``insertnode!``) and child indexing ``t[0][1]``.

Conventions restated from NewickTree's behaviour as the reference uses it:
children keep their textual order; a node without a branch length has
distance NaN (the root of ``extree`` for instance); ``insertnode`` puts a new
node halfway up the branch above ``n`` (docs/lit/wgd-turing.jl:22-24) and the
new node is appended to the parent's children.
"""
from __future__ import annotations

import math
from typing import Iterator, List, Optional


class Node:
    __slots__ = ("name", "distance", "parent", "children")

    def __init__(self, name: str = "", distance: float = math.nan, parent: Optional["Node"] = None):
        self.name = name
        self.distance = distance
        self.parent = parent
        self.children: List[Node] = []
        if parent is not None:
            parent.children.append(self)

    def isleaf(self) -> bool:
        return not self.children

    def isroot(self) -> bool:
        return self.parent is None

    def __getitem__(self, i: int) -> "Node":
        return self.children[i]

    def __len__(self) -> int:
        return len(self.children)

    def __repr__(self) -> str:
        return f"Node({self.name!r}, {self.distance})"


def readnw(s: str) -> Node:
    """Parse a Newick string (names, branch lengths, unary nodes, [comments])."""
    s = s.strip()
    pos = 0

    def skip():
        nonlocal pos
        while pos < len(s) and s[pos].isspace():
            pos += 1

    def subtree(parent):
        nonlocal pos
        node = Node(parent=parent)
        skip()
        if pos < len(s) and s[pos] == "(":
            pos += 1
            while True:
                subtree(node)
                skip()
                if pos < len(s) and s[pos] == ",":
                    pos += 1
                    continue
                if pos < len(s) and s[pos] == ")":
                    pos += 1
                    break
                raise ValueError(f"newick: expected ',' or ')' at {pos}")
        skip()
        start = pos
        while pos < len(s) and s[pos] not in ":,);[":
            pos += 1
        node.name = s[start:pos].strip()
        skip()
        if pos < len(s) and s[pos] == "[":
            end = s.index("]", pos)
            pos = end + 1
        skip()
        if pos < len(s) and s[pos] == ":":
            pos += 1
            start = pos
            while pos < len(s) and s[pos] not in ",);[":
                pos += 1
            node.distance = float(s[start:pos])
        return node

    root = subtree(None)
    skip()
    if pos < len(s) and s[pos] == ";":
        pos += 1
    return root


def _fmt(x: float) -> str:
    return repr(float(x))


def nwstr(n: Node, dist: bool = True) -> str:
    """Newick string of the subtree at ``n`` (unary nodes kept)."""

    def rec(x: Node) -> str:
        s = ""
        if x.children:
            s = "(" + ",".join(rec(c) for c in x.children) + ")"
        s += x.name
        if dist and not math.isnan(x.distance):
            s += ":" + _fmt(x.distance)
        return s

    return rec(n) + ";"


def postwalk(n: Node) -> List[Node]:
    out: List[Node] = []

    def rec(x):
        for c in x.children:
            rec(c)
        out.append(x)

    rec(n)
    return out


def prewalk(n: Node) -> List[Node]:
    out: List[Node] = []

    def rec(x):
        out.append(x)
        for c in x.children:
            rec(c)

    rec(n)
    return out


def getleaves(n: Node) -> List[Node]:
    return [x for x in prewalk(n) if x.isleaf()]


def getroot(n: Node) -> Node:
    while n.parent is not None:
        n = n.parent
    return n


def getlca(t: Node, a: str, b: str) -> Node:
    """Lowest common ancestor of the leaves named ``a`` and ``b``."""
    leaves = {x.name: x for x in getleaves(t)}
    x, y = leaves[a], leaves[b]
    anc = set()
    while x is not None:
        anc.add(id(x))
        x = x.parent
    while id(y) not in anc:
        y = y.parent
    return y


def insertnode(n: Node, name: str = "", dist: Optional[float] = None) -> Node:
    """``insertnode!``: insert a node on the branch above ``n`` at ``dist``
    below the parent (default halfway).  The new node takes over ``n`` as its
    only child and is appended to the parent's children."""
    if n.parent is None:
        raise ValueError("cannot insert a node above the root")
    p = n.parent
    d = n.distance / 2.0 if dist is None else float(dist)
    new = Node(name=name, distance=d, parent=p)
    p.children.remove(n)
    n.parent = new
    new.children.append(n)
    n.distance = n.distance - d
    return new


def copytree(n: Node) -> Node:
    return readnw(nwstr(n))


# The reference's 9-taxon example tree (src/Whale.jl:34-37).
EXTREE = ("((MPOL:4.752,PPAT:4.752):0.292,(SMOE:4.457,(((OSAT:1.555,(ATHA:0.5548,CPAP:0.5548):1.0002):0"
          ".738,ATRI:2.293):1.225,(GBIL:3.178,PABI:3.178):0.34):0.939):0.587);")


def extree() -> Node:
    return readnw(EXTREE)


def addbranchwgds(tree: Node, tips: bool = False) -> int:
    """``addbranchwgds!`` (src/model.jl:231-239): a WGD halfway up every
    internal branch (and tip branch with ``tips``)."""
    nwgd = 0
    for n in postwalk(tree):
        if n.isroot() or (not tips and n.isleaf()):
            continue
        nwgd += 1
        insertnode(n, name=f"wgd_{nwgd}")
    return nwgd


def iter_nodes(t: Node) -> Iterator[Node]:
    yield from prewalk(t)
