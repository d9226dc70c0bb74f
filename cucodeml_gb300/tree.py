"""Unrooted binary trees in codeml's node numbering.

codeml reads a Newick tree (ReadTreeN, treesub.c:2883-3110) and numbers nodes
as follows, which this module reproduces so that parameter vectors line up:

* tips 0..ns-1 are the species in sequence-file order (matched by name);
* internal nodes are numbered ns, ns+1, ... in the order their '(' appears,
  so the root is node ns (the outermost parenthesis, a trifurcation for an
  unrooted tree);
* every non-root node gets a branch index `ibranch` in the order it is first
  met while reading, i.e. a pre-order walk (also what NodeToBranch produces,
  treesub.c:2683-2701); the first `nbranch` entries of codeml's x[] are the
  branch lengths in this order.
* `#1` after a clade or name sets the foreground label (nodes[].label), every
  other non-root node has label 0 (treesub.c:3142).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Tree:
    ns: int
    father: np.ndarray            # [nnode] int, -1 for the root
    sons: list                    # [nnode] list of son node ids
    branch: np.ndarray            # [nnode] branch length above node (root: 0)
    label: np.ndarray             # [nnode] 0 background, 1 foreground (root: 0)
    ibranch: np.ndarray           # [nnode] pre-order branch index (root: -1)
    root: int
    names: list = field(default_factory=list)

    @property
    def nnode(self) -> int:
        return len(self.father)

    @property
    def nbranch(self) -> int:
        return self.nnode - 1

    def branch_nodes(self) -> np.ndarray:
        """node id of branch ib, for ib in 0..nbranch-1."""
        out = np.empty(self.nbranch, dtype=np.int64)
        for n in range(self.nnode):
            if self.ibranch[n] >= 0:
                out[self.ibranch[n]] = n
        return out

    def x_branch_lengths(self) -> np.ndarray:
        """Branch lengths in codeml's x[] order (by ibranch)."""
        return self.branch[self.branch_nodes()].copy()

    def set_from_x(self, xb: np.ndarray) -> None:
        self.branch[self.branch_nodes()] = np.asarray(xb, dtype=np.float64)

    def foreground_node(self) -> int:
        fg = np.nonzero(self.label == 1)[0]
        return int(fg[0]) if len(fg) else -1

    def to_newick(self, lengths: bool = True, digits: int = 12) -> str:
        def rec(n: int) -> str:
            s = self.names[n] if n < self.ns else "(" + ",".join(rec(c) for c in self.sons[n]) + ")"
            if n != self.root and self.label[n] == 1:
                s += " #1"
            if lengths and n != self.root:
                s += ":" + format(float(self.branch[n]), f".{digits}g")
            return s
        return rec(self.root) + ";"

    def postorder(self) -> list:
        order = []

        def rec(n):
            for c in self.sons[n]:
                rec(c)
            order.append(n)
        rec(self.root)
        return order


def parse_newick(text: str, names: list) -> Tree:
    """Parse a Newick string with codeml's node numbering (see module doc)."""
    ns = len(names)
    name_to_id = {nm: i for i, nm in enumerate(names)}
    nmax = 2 * ns - 1
    father = [-1] * nmax
    sons = [[] for _ in range(nmax)]
    branch = [0.0] * nmax
    label = [-1.0] * nmax
    ibranch = [-1] * nmax
    nnode = ns
    nbranch = 0
    cfather = -1
    inodeb = 0
    root = -1
    i = 0
    delim = "(),:#;"
    while i < len(text):
        ch = text[i]
        if ch == ";":
            break
        if ch in ", \t\r\n":
            i += 1
            continue
        if ch == "(":
            cnode = nnode
            nnode += 1
            if cfather >= 0:
                sons[cfather].append(cnode)
                father[cnode] = cfather
                ibranch[cnode] = nbranch
                nbranch += 1
            else:
                root = cnode
            cfather = cnode
            i += 1
        elif ch == ")":
            inodeb = cfather
            cfather = father[cfather]
            i += 1
        elif ch in ":#":
            j = i + 1
            while j < len(text) and text[j] == " ":
                j += 1
            k = j
            while k < len(text) and (text[k].isdigit() or text[k] in "+-.eE"):
                k += 1
            val = float(text[j:k])
            if ch == ":":
                branch[inodeb] = val
            else:
                label[inodeb] = val
            i = k
        else:
            j = i
            while j < len(text) and text[j] not in delim and text[j] not in "\n":
                j += 1
            nm = text[i:j].strip()
            cnode = name_to_id[nm]
            father[cnode] = cfather
            sons[cfather].append(cnode)
            ibranch[cnode] = nbranch
            nbranch += 1
            inodeb = cnode
            i = j
    lab = np.array(label[:nnode])
    lab[lab < 0] = 0
    lab[root] = 0
    return Tree(ns=ns, father=np.array(father[:nnode]), sons=sons[:nnode],
                branch=np.array(branch[:nnode]), label=lab.astype(np.int64),
                ibranch=np.array(ibranch[:nnode]), root=root, names=list(names))


def random_tree(ns: int, rng: np.random.Generator, mean_blen: float = 0.1) -> Tree:
    """Uniform random unrooted binary tree by random sequential joining.

    Start from the 3-taxon star; taxon k is attached to a uniformly chosen
    existing edge.  Branch lengths ~ Exp(mean_blen); one uniformly chosen
    branch carries the foreground label #1.  The result is written to Newick
    rooted at the internal node of the first star and re-read, so node ids
    follow codeml's numbering.
    """
    if ns < 3:
        raise ValueError("need at least 3 taxa")
    names = [f"S{i + 1}" for i in range(ns)]
    # adjacency over labels: tips 0..ns-1, internal ns..2ns-3
    adj = {0: [ns], 1: [ns], 2: [ns], ns: [0, 1, 2]}
    edges = [(ns, 0), (ns, 1), (ns, 2)]
    nxt = ns + 1
    for k in range(3, ns):
        a, b = edges[int(rng.integers(len(edges)))]
        m = nxt
        nxt += 1
        adj[a][adj[a].index(b)] = m
        adj[b][adj[b].index(a)] = m
        adj[m] = [a, b, k]
        adj[k] = [m]
        edges.remove((a, b))
        edges += [(a, m), (m, b), (m, k)]
    # root at node ns, orient edges away from it
    rootlab = ns
    children = {}
    stack = [(rootlab, -1)]
    order = []
    while stack:
        v, p = stack.pop()
        order.append(v)
        children[v] = [u for u in adj[v] if u != p]
        for u in reversed(children[v]):
            stack.append((u, v))
    blen = {v: float(rng.exponential(mean_blen)) for v in order if v != rootlab}
    nonroot = [v for v in order if v != rootlab]
    fg = nonroot[int(rng.integers(len(nonroot)))]

    def rec(v):
        s = names[v] if v < ns else "(" + ",".join(rec(u) for u in children[v]) + ")"
        if v == rootlab:
            return s
        if v == fg:
            s += " #1"
        return s + ":" + repr(blen[v])
    return parse_newick(rec(rootlab) + ";", names)
