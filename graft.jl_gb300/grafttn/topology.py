"""Tree topologies (host metadata).

Mirrors lib/GraftFoundation/src/Trees/topology.jl:22-160 and geometries.jl:13-95: a rooted
tree given as top-down ``(parent, child)`` edges; child order is leg order; every edge
points towards the root.  Node indices are 0-based here (the reference is 1-based);
the root is node 0.
"""
from __future__ import annotations


class TreeTopology:
    def __init__(self, root, edges):
        self.ids = [root]
        self.index = {root: 0}
        self.parent = [-1]
        self.children = [[]]
        for p, c in edges:
            if p not in self.index:
                raise ValueError(f"parent {p} unknown when adding edge {p} => {c} (edges must be given top-down)")
            if c in self.index:
                raise ValueError(f"node {c} added twice")
            self.ids.append(c)
            self.index[c] = len(self.ids) - 1
            self.parent.append(self.index[p])
            self.children.append([])
            self.children[self.index[p]].append(self.index[c])
        self.root = 0
        self.depth = [0] * len(self.ids)
        for i in range(1, len(self.ids)):
            self.depth[i] = self.depth[self.parent[i]] + 1

    def __eq__(self, other):
        return (isinstance(other, TreeTopology) and self.ids == other.ids
                and self.parent == other.parent and self.children == other.children)

    def __hash__(self):
        return hash((tuple(self.ids), tuple(self.parent)))

    @property
    def nnodes(self):
        return len(self.ids)

    def nodeindex(self, n):
        return n if isinstance(n, int) else self.index[n]

    def nchildren(self, i):
        return len(self.children[i])

    def isroot(self, i):
        return self.parent[i] < 0

    def neighbors(self, i):
        """Children in leg order, then the parent (topology.jl:67-72)."""
        ns = list(self.children[i])
        if self.parent[i] >= 0:
            ns.append(self.parent[i])
        return ns

    def childslot(self, p, c):
        try:
            return self.children[p].index(c)
        except ValueError:
            raise ValueError(f"{self.ids[c]} is not a child of {self.ids[p]}") from None

    def edges(self):
        return [(i, self.parent[i]) for i in range(self.nnodes) if self.parent[i] >= 0]

    def postorder(self):
        out = []
        stack = [(self.root, False)]
        while stack:
            i, done = stack.pop()
            if done:
                out.append(i)
                continue
            stack.append((i, True))
            for c in reversed(self.children[i]):
                stack.append((c, False))
        return out

    def path_to_root(self, a):
        p = [a]
        while self.parent[p[-1]] >= 0:
            p.append(self.parent[p[-1]])
        return p

    def path_between(self, a, b):
        pa, pb = self.path_to_root(a), self.path_to_root(b)
        inb = set(pb)
        lca_pos = next(i for i, x in enumerate(pa) if x in inb)
        lca = pa[lca_pos]
        return pa[: lca_pos + 1] + list(reversed(pb[: pb.index(lca)]))

    def subtree_nodes(self, n, avoiding):
        """The nodes reached from n without crossing to `avoiding` (n first), as a tuple;
        the topology never changes after construction, so each answer is computed once."""
        memo = self.__dict__.setdefault("_subtree_memo", {})
        key = (n, avoiding)
        got = memo.get(key)
        if got is None:
            acc, stack = [], [(n, avoiding)]
            while stack:
                i, frm = stack.pop()
                acc.append(i)
                for m in self.neighbors(i):
                    if m != frm:
                        stack.append((m, i))
            got = memo[key] = (tuple(acc), frozenset(acc))
        return got[0]

    def in_subtree(self, x, n, avoiding):
        """Whether x is among subtree_nodes(n, avoiding) (a set lookup after the first call)."""
        self.subtree_nodes(n, avoiding)
        return x in self._subtree_memo[(n, avoiding)][1]


def mps_topology(n):
    ids = [f"site{i}" for i in range(1, n + 1)]
    return TreeTopology(ids[-1], [(ids[i + 1], ids[i]) for i in range(n - 2, -1, -1)])


def star_topology(nbranches, branchlength):
    edges = []
    for b in range(1, nbranches + 1):
        prev = "center"
        for l in range(1, branchlength + 1):
            node = f"b{b}_{l}"
            edges.append((prev, node))
            prev = node
    return TreeTopology("center", edges)


def binary_topology(depth):
    edges = []
    for d in range(1, depth + 1):
        for k in range(1, 2 ** d + 1):
            edges.append((f"n{d-1}_{(k + 1) // 2}", f"n{d}_{k}"))
    return TreeTopology("n0_1", edges)


def kary_topology(k, depth):
    """Complete k-ary tree (the 85-site 4-ary depth-3 tree of the TDVP1_CBE workload)."""
    edges = []
    for d in range(1, depth + 1):
        for j in range(1, k ** d + 1):
            edges.append((f"k{d-1}_{(j - 1) // k + 1}", f"k{d}_{j}"))
    return TreeTopology("k0_1", edges)


def fork_topology(nteeth, toothlength):
    if nteeth < 1:
        raise ValueError("fork_topology needs at least one flavor spine node")
    edges = [(f"spine{s-1}", f"spine{s}") for s in range(2, nteeth + 1)]
    for s in range(1, nteeth + 1):
        prev = f"spine{s}"
        for l in range(1, toothlength + 1):
            node = f"tooth{s}_{l}"
            edges.append((prev, node))
            prev = node
    return TreeTopology("spine1", edges)
