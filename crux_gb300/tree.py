"""Unrooted trees as rings of half-edges, with Newick input.

Host-side restatement of pkg/Crux/Tree/__init__.pyx and pkg/Crux/Newick.pyx,
kept exact where the likelihood depends on it: ring order fixes the
post-order step plan, so ``Edge.attach`` inserts a ring before the node's
head ring and makes it the head (__init__.pyx:811-848), ``Edge.detach``
advances the head if it pointed at the removed ring (:850-876), the Newick
parser appends children at the ring tail (Newick.pyx:177-191),
``Tree.deroot`` splices out a degree-2 root adding a float32-rounded length
(:397-437, ``cdef float removedLength`` at :404) and ``Tree.canonize``
re-orders every ring by per-subtree minimum taxon index starting from the
minimum taxon (:439-473, :960-1002).
"""
import re

import numpy as np


class Ring:
    __slots__ = ("node", "edge", "other", "next", "prev", "aux")

    def __init__(self, edge=None, other=None):
        self.node = None
        self.edge = edge
        self.other = other
        self.next = self
        self.prev = self
        self.aux = None

    def __iter__(self):
        """This ring and its siblings, in ring order."""
        r = self
        while True:
            yield r
            r = r.next
            if r is self:
                return

    def siblings(self):
        """The other rings of this node, in ring order."""
        r = self.next
        while r is not self:
            nxt = r.next
            yield r
            r = nxt

    def _minTaxon(self, taxaMap):
        ret = self.node
        for r in self.siblings():
            m = r.other._minTaxon(taxaMap)
            if ret.taxon is None or \
                    taxaMap.indGet(m.taxon) < taxaMap.indGet(ret.taxon):
                ret = m
        return ret

    def _canonize(self, taxaMap):
        node = self.node
        ret = node
        if node.degree_calc() > 1:
            rings = []
            for r in list(self.siblings()):
                m = r.other._canonize(taxaMap)
                if ret.taxon is None or \
                        taxaMap.indGet(m.taxon) < taxaMap.indGet(ret.taxon):
                    ret = m
                rings.append((taxaMap.indGet(m.taxon), r))
            rings.sort(key=lambda x: x[0])
            for _, r in reversed(rings):
                other = r.other.node
                e = r.edge
                e.detach()
                e.attach(node, other)
            node.ring = self
        return ret


class Node:
    __slots__ = ("tree", "ring", "taxon", "aux", "_degree")

    def __init__(self, tree=None):
        self.tree = tree
        self.ring = None
        self.taxon = None
        self.aux = None
        self._degree = None

    def degree_calc(self):
        if self.ring is None:
            return 0
        return sum(1 for _ in self.ring)

    def getDegree(self):
        # Cached: only Edge.attach and Edge.detach change a degree, and they
        # clear the cache of both end nodes.
        d = self._degree
        if d is None:
            d = self._degree = self.degree_calc()
        return d

    @property
    def degree(self):
        return self.getDegree()

    def getTaxon(self):
        return self.taxon


class Edge:
    __slots__ = ("tree", "ring", "length", "aux")

    def __init__(self, tree=None):
        self.tree = tree
        self.ring = Ring(self, None)
        self.ring.other = Ring(self, self.ring)
        self.length = 0.0
        self.aux = None

    def attach(self, nodeA, nodeB):
        assert self.ring.node is None and self.ring.other.node is None
        assert nodeA is not nodeB
        for ring, node in ((self.ring, nodeA), (self.ring.other, nodeB)):
            ring.node = node
            node._degree = None
            head = node.ring
            if head is not None:
                tail = head.prev
                ring.next = head
                ring.prev = tail
                head.prev = ring
                tail.next = ring
            node.ring = ring
        if self.tree is not None:
            self.tree.sn += 1

    def detach(self):
        for ring in (self.ring, self.ring.other):
            node = ring.node
            node._degree = None
            nxt = ring.next
            if nxt is ring:
                node.ring = None
            else:
                if node.ring is ring:
                    node.ring = nxt
                prv = ring.prev
                nxt.prev = prv
                prv.next = nxt
                ring.next = ring
                ring.prev = ring
            ring.node = None
        if self.tree is not None:
            self.tree.sn += 1


class Tree:
    """Tree with a base node; unrooted after ``deroot``."""

    def __init__(self, newick=None, rooted=True):
        self.sn = 0
        self.rooted = rooted
        self.base = None
        self.aux = None
        if newick is not None:
            NewickParser(self).parse(newick)
            if not self.rooted:
                self.rooted = True
                self.deroot()

    # -- traversal --------------------------------------------------------
    def _walk(self):
        nodes, edges = [], []
        if self.base is None:
            return nodes, edges
        nodes.append(self.base)
        stack = []
        if self.base.ring is not None:
            for r in reversed(list(self.base.ring)):
                stack.append(r)
        while stack:
            r = stack.pop()
            edges.append(r.edge)
            child = r.other
            nodes.append(child.node)
            for s in reversed(list(child.siblings())):
                stack.append(s)
        return nodes, edges

    @property
    def nodes(self):
        return self._walk()[0]

    @property
    def edges(self):
        return self._walk()[1]

    @property
    def ntaxa(self):
        return sum(1 for n in self.nodes if n.taxon is not None)

    def getTaxa(self):
        return sorted(n.taxon for n in self.nodes if n.taxon is not None)

    def getBase(self):
        return self.base

    def setBase(self, node):
        self.base = node
        self.sn += 1

    def clearAux(self):
        self.aux = None
        self.sn += 1
        for n in self.nodes:
            n.aux = None
            if n.ring is not None:
                for r in n.ring:
                    r.aux = None
                    r.edge.aux = None

    # -- structural edits -------------------------------------------------
    def deroot(self):
        """Remove the root (__init__.pyx:397-437)."""
        if not self.rooted:
            return
        self.rooted = False
        ring = self.base.ring
        if ring is None:
            self.base = None
            return
        ring = ring.other
        node = ring.node
        edge = ring.edge
        edge.detach()
        if node.degree_calc() == 2:
            ring = node.ring
            self.base = ring.other.node
            edge = ring.edge
            removed = float(np.float32(edge.length))
            edge.detach()
            ring = node.ring
            edge = ring.edge
            node = ring.other.node
            edge.detach()
            edge.attach(self.base, node)
            edge.length = edge.length + removed
            self.base.ring = self.base.ring.next
        else:
            self.base = node

    def canonize(self, taxaMap):
        """Repeatable ring order keyed by taxon index (__init__.pyx:439-473)."""
        if self.rooted:
            base = self.base
        else:
            node = self.base
            if node is None or node.ring is None:
                return
            ring = node.ring
            base = ring._minTaxon(taxaMap)
            other = ring.other._minTaxon(taxaMap)
            if base.taxon is None or \
                    taxaMap.indGet(other.taxon) < taxaMap.indGet(base.taxon):
                base = other
            self.base = base
        ring = base.ring
        if ring is None:
            return
        ring.other._canonize(taxaMap)

    def dup(self):
        """Independent copy with the same ring order (__init__.pyx:130-172)."""
        new = Tree()
        new.rooted = self.rooted

        def rec(node, prev):
            nn = Node(new)
            nn.taxon = node.taxon
            if node.ring is not None:
                deg = node.degree_calc()
                r = node.ring
                for _ in range(deg):
                    if r is not prev:
                        o = r.other
                        child = rec(o.node, o)
                        e = Edge(new)
                        e.length = r.edge.length
                        e.attach(nn, child)
                    r = r.next
            return nn

        if self.base is not None:
            new.base = rec(self.base, None)
        return new

    # -- pickling (__init__.pyx:53-63, 626-647, 801-809) ---------------------
    def __reduce__(self):
        """Pickled as flat tables, not as the linked ring structure (whose
        recursion a deep tree would overflow): every node's taxon and its
        rings in ring order from its head ring, every edge's length, the
        base.  Unpickling rebuilds the same ring order, which fixes the
        post-order step plan; aux data (CL caches) is dropped, as the
        reference's __setstate__ drops it."""
        nodes, edges = self._walk()
        nid = {id(n): i for i, n in enumerate(nodes)}
        eid = {id(e): i for i, e in enumerate(edges)}
        rings = []
        for n in nodes:
            rs = []
            if n.ring is not None:
                for r in n.ring:
                    rs.append((eid[id(r.edge)], 0 if r is r.edge.ring else 1))
            rings.append(rs)
        state = (self.rooted, nid[id(self.base)] if self.base is not None else -1,
                 [n.taxon for n in nodes], rings, [e.length for e in edges])
        return (_tree_from_state, (state,))

    def render(self, lengths=True, fmt="%.7e"):
        """Newick text of an unrooted tree (for diagnostics)."""
        out = []

        def rrender(node, via, noLength):
            did = False
            if node.ring is not None:
                for r in node.ring:
                    if r.edge is not via:
                        out.append("," if did else "(")
                        did = True
                        rrender(r.other.node, r.edge, False)
                if did:
                    out.append(")")
            if node.taxon is not None:
                out.append(node.taxon.replace(" ", "_"))
            if lengths and node.degree_calc() > 0 and not noLength:
                out.append((":" + fmt) % via.length)

        n = self.base
        if n is not None:
            if n.degree_calc() == 1 and n.ring.other.node.degree_calc() > 1:
                rrender(n.ring.other.node, None, True)
            else:
                rrender(n, None, True)
        out.append(";")
        return "".join(out)


_TOKEN = re.compile(r"""
    (?P<ws>\s+)
  | (?P<comment>\[[^\]]*\])
  | (?P<lp>\()
  | (?P<rp>\))
  | (?P<comma>,)
  | (?P<colon>:)
  | (?P<semi>;)
  | (?P<qlabel>'(?:[^']|'')*')
  | (?P<word>[^\s()\[\]':;,]+)
""", re.X)


def _tree_from_state(state):
    """Rebuild a Tree pickled by Tree.__reduce__."""
    rooted, base, taxa, rings, lengths = state
    t = Tree()
    t.rooted = rooted
    nodes = []
    for taxon in taxa:
        n = Node(t)
        n.taxon = taxon
        nodes.append(n)
    edges = []
    for length in lengths:
        e = Edge(t)
        e.length = length
        edges.append(e)
    for n, rs in zip(nodes, rings):
        objs = [edges[e].ring if end == 0 else edges[e].ring.other for e, end in rs]
        for i, r in enumerate(objs):
            r.node = n
            r.next = objs[(i + 1) % len(objs)]
            r.prev = objs[i - 1]
        n.ring = objs[0] if objs else None
    t.base = nodes[base] if base >= 0 else None
    return t


class NewickParser:
    """Recursive-descent Newick reader (Newick.pyx:170-286)."""

    def __init__(self, tree):
        self.tree = tree

    def parse(self, text):
        self.toks = []
        pos = 0
        while pos < len(text):
            m = _TOKEN.match(text, pos)
            if m is None:
                raise SyntaxError("Invalid Newick token at %d" % pos)
            pos = m.end()
            kind = m.lastgroup
            if kind in ("ws", "comment"):
                continue
            self.toks.append((kind, m.group(kind)))
            if kind == "semi":
                break
        self.i = 0
        self._tree()

    def _peek(self):
        return self.toks[self.i] if self.i < len(self.toks) else ("eoi", "")

    def _get(self):
        t = self._peek()
        self.i += 1
        return t

    def _label(self):
        kind, val = self._peek()
        if kind == "word":
            self.i += 1
            return val.replace("_", " ")
        if kind == "qlabel":
            self.i += 1
            return val[1:-1].replace("''", "'")
        return None

    def _brlen(self):
        if self._peek()[0] == "colon":
            self.i += 1
            kind, val = self._get()
            if kind != "word":
                raise SyntaxError("Unexpected token: %r" % val)
            return float(val)
        return float("nan")

    def _subtree(self):
        desc = self._descendants()
        label = self._label()
        brlen = self._brlen()
        if brlen != brlen:
            brlen = 0.0
        node = desc if desc is not None else Node(self.tree)
        if label is not None:
            node.taxon = label
        return node, brlen

    def _subtree_list(self):
        ret = Node(self.tree)
        while True:
            sub, brlen = self._subtree()
            e = Edge(self.tree)
            e.length = brlen
            e.attach(ret, sub)
            ret.ring = ret.ring.next
            if self._peek()[0] != "comma":
                return ret
            self.i += 1

    def _descendants(self):
        if self._peek()[0] != "lp":
            return None
        self.i += 1
        ret = self._subtree_list()
        kind, val = self._get()
        if kind != "rp":
            raise SyntaxError("Unexpected token: %r" % val)
        return ret

    def _tree(self):
        desc = self._descendants()
        label = self._label()
        brlen = self._brlen()
        kind, val = self._get()
        if kind != "semi":
            raise SyntaxError("Unexpected token: %r" % val)
        root = Node(self.tree)
        self.tree.base = root
        if desc is not None:
            node = desc
            if label is not None:
                node.taxon = label
        elif label is not None:
            node = Node(self.tree)
            node.taxon = label
        elif brlen == brlen:
            node = Node(self.tree)
        else:
            return
        e = Edge(self.tree)
        if brlen == brlen:
            e.length = brlen
        e.attach(root, node)
