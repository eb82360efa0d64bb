"""CPU oracle for the tree-tensor-network effective-Hamiltonian path (TEST INFRASTRUCTURE).

This module is the checker, not the product: only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` import it.  It is a
plain numpy/scipy (complex128) restatement of GraftTN/Graft.jl's algorithms for the
eff_h1 / eff_h2 / eff_h0 Krylov maps, the environment updates, the two-site merge/split,
the gauge moves, the Lanczos ground-state solve of ``dmrg2!`` and the Krylov exponential
of ``TDVP1``.  Each function cites the reference file:line it follows (paths are relative
to the reference project root).

Parity status.  The reference is Julia (no toolchain here) and its arithmetic lives in
unvendored packages (TensorKit 0.17.1, TensorOperations 5.6.2, KrylovKit 0.10.4,
MatrixAlgebraKit 0.6.9).  It ships no golden vectors for this path; it pins the path with
known-answer gates instead, and this oracle is pinned by the same gates
(``tests/test_oracle.py``): DMRG vs exact diagonalisation <= 1e-10
(test/runtests.jl:687-700), eff_h1 Rayleigh closure <= 1e-12 (:654-672), two-site
merge/split round trip <= 1e-12 (:674-685), TTNO == dense H <= 1e-12 (:362-393),
full-rank TDVP1 == exact propagation (:895-959), planned map == unplanned ncon and
Hermitian (test/contraction_planning.jl:111-160).  Bitwise parity of initial states is
impossible (TensorKit's Xoshiro fill order); random states here use numpy PCG64.

Layout.  A tensor is a C-ordered numpy array whose axes follow the reference's flat leg
order: TTNS node ``(children..., phys, parent)`` (lib/GraftNetworks/src/Networks/ttns.jl:1-12),
TTNO node ``(children..., P_out, P_in, parent)`` (ttno.jl:1-9), environment
``(ket, op, bra)`` (lib/GraftContractions/src/Contractions/envcache.jl:919-999).  The root's
parent leg has dimension 1 and is closed by an all-ones cap (Backend.jl:144-150).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla

# ---------------------------------------------------------------------------
# trees (lib/GraftFoundation/src/Trees/topology.jl:22-160, geometries.jl:13-95)
# ---------------------------------------------------------------------------


class TreeTopology:
    """Rooted tree; ``edges`` are ``(parent, child)`` pairs given top-down
    (topology.jl:31-50).  Node 0 is the root; child order is leg order."""

    def __init__(self, root, edges):
        self.ids = [root]
        self.index = {root: 0}
        self.parent = [-1]
        self.children = [[]]
        for p, c in edges:
            if p not in self.index:
                raise ValueError(f"parent {p} unknown when adding edge {p} => {c}")
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

    @property
    def nnodes(self):
        return len(self.ids)

    def nchildren(self, i):
        return len(self.children[i])

    def neighbors(self, i):
        """Children in leg order, then the parent (topology.jl:67-72)."""
        ns = list(self.children[i])
        if self.parent[i] >= 0:
            ns.append(self.parent[i])
        return ns

    def childslot(self, p, c):
        return self.children[p].index(c)

    def edges(self):
        """``(child, parent)`` pairs (topology.jl:84)."""
        return [(i, self.parent[i]) for i in range(self.nnodes) if self.parent[i] >= 0]

    def postorder(self):
        out = []

        def rec(i):
            for c in self.children[i]:
                rec(c)
            out.append(i)
        rec(self.root)
        return out

    def path_to_root(self, a):
        p = [a]
        while self.parent[p[-1]] >= 0:
            p.append(self.parent[p[-1]])
        return p

    def path_between(self, a, b):
        """Unique path a -> b, inclusive (topology.jl:132-140)."""
        pa, pb = self.path_to_root(a), self.path_to_root(b)
        inb = set(pb)
        lca_pos = next(i for i, x in enumerate(pa) if x in inb)
        lca = pa[lca_pos]
        up = pa[: lca_pos + 1]
        down = list(reversed(pb[: pb.index(lca)]))
        return up + down

    def subtree_nodes(self, n, avoiding):
        acc, stack = [], [(n, avoiding)]
        while stack:
            i, frm = stack.pop()
            acc.append(i)
            for m in self.neighbors(i):
                if m != frm:
                    stack.append((m, i))
        return acc


def mps_topology(n):
    """Chain rooted at the last site (geometries.jl:13-17)."""
    ids = [f"site{i}" for i in range(1, n + 1)]
    return TreeTopology(ids[-1], [(ids[i + 1], ids[i]) for i in range(n - 2, -1, -1)])


def star_topology(nbranches, branchlength):
    """Centre plus ``nbranches`` chains (geometries.jl:26-37)."""
    edges = []
    for b in range(1, nbranches + 1):
        prev = "center"
        for l in range(1, branchlength + 1):
            node = f"b{b}_{l}"
            edges.append((prev, node))
            prev = node
    return TreeTopology("center", edges)


def binary_topology(depth):
    """Perfect binary tree, root at depth 0 (geometries.jl:45-53)."""
    edges = []
    for d in range(1, depth + 1):
        for k in range(1, 2 ** d + 1):
            edges.append((f"n{d-1}_{(k + 1) // 2}", f"n{d}_{k}"))
    return TreeTopology("n0_1", edges)


def kary_topology(k, depth):
    """Complete k-ary tree built through ``TreeTopology(root, edges)``
    (the reference has no k-ary builder: geometries.jl:134)."""
    edges = []
    for d in range(1, depth + 1):
        for j in range(1, k ** d + 1):
            edges.append((f"k{d-1}_{(j - 1) // k + 1}", f"k{d}_{j}"))
    return TreeTopology("k0_1", edges)


# ---------------------------------------------------------------------------
# operators (lib/GraftSymbolic/src/Symbolic/Symbolic.jl:177-185) and Hamiltonians
# ---------------------------------------------------------------------------


def spin_ops():
    X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
    Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
    Z = np.array([[1, 0], [0, -1]], dtype=np.complex128)
    Sp = np.array([[0, 1], [0, 0]], dtype=np.complex128)
    Sm = np.array([[0, 0], [1, 0]], dtype=np.complex128)
    I = np.eye(2, dtype=np.complex128)
    return dict(X=X, Y=Y, Z=Z, Sp=Sp, Sm=Sm, I=I)


@dataclass
class NNHamiltonian:
    """Nearest-neighbour tree Hamiltonian: ``onsite[n]`` one-body matrices and
    ``bonds[(child, parent)]`` lists of ``(coeff, O_child, O_parent)`` two-body terms.
    This is the OpSum subset the hot-path configs use (test/runtests.jl:20-31)."""
    topo: TreeTopology
    d: int = 2
    onsite: dict = field(default_factory=dict)
    bonds: dict = field(default_factory=dict)


def tfi(topo, J=1.0, g=0.7):
    """-J ZZ on every edge, -g X on every site (test/runtests.jl:20-31)."""
    S = spin_ops()
    H = NNHamiltonian(topo)
    for c, p in topo.edges():
        H.bonds[(c, p)] = [(-J, S["Z"], S["Z"])]
    for i in range(topo.nnodes):
        H.onsite[i] = -g * S["X"]
    return H


def heisenberg(topo, J=1.0):
    """J (XX + YY + ZZ) with Pauli matrices on every edge (the literal reading of the
    dense Heisenberg workload; 4x the S.S convention)."""
    S = spin_ops()
    H = NNHamiltonian(topo)
    for c, p in topo.edges():
        H.bonds[(c, p)] = [(J, S["X"], S["X"]), (J, S["Y"], S["Y"]), (J, S["Z"], S["Z"])]
    return H


def xxz(topo, couplings, delta=0.7):
    """sum_e theta_e (XX + YY + delta ZZ) (the XXZ workload with per-edge couplings)."""
    S = spin_ops()
    H = NNHamiltonian(topo)
    for e in topo.edges():
        th = couplings[e]
        H.bonds[e] = [(th, S["X"], S["X"]), (th, S["Y"], S["Y"]), (th * delta, S["Z"], S["Z"])]
    return H


def dense_hamiltonian(H: NNHamiltonian):
    """Dense matrix on all sites, site 0 slowest (GraftTestUtils.jl:433-453 up to
    the kron order, which is fixed here to match ``to_dense``)."""
    n, d = H.topo.nnodes, H.d
    dim = d ** n

    def embed(ops):
        mats = [np.eye(d, dtype=np.complex128)] * n
        mats = list(mats)
        for site, m in ops:
            mats[site] = m
        out = mats[0]
        for m in mats[1:]:
            out = np.kron(out, m)
        return out
    Hd = np.zeros((dim, dim), dtype=np.complex128)
    for i, h in H.onsite.items():
        Hd += embed([(i, h)])
    for (c, p), terms in H.bonds.items():
        for coeff, oc, op in terms:
            Hd += coeff * embed([(c, oc), (p, op)])
    return Hd


def sparse_hamiltonian(H: NNHamiltonian):
    """The same matrix as ``dense_hamiltonian`` in scipy CSR form (site 0 slowest), for
    systems too large for a dense matrix."""
    import scipy.sparse as sp
    n, d = H.topo.nnodes, H.d

    def embed(ops):
        out = sp.identity(1, dtype=np.complex128, format="csr")
        for i in range(n):
            out = sp.kron(out, sp.csr_matrix(ops.get(i, np.eye(d, dtype=np.complex128))), format="csr")
        return out
    Hs = sp.csr_matrix((d ** n, d ** n), dtype=np.complex128)
    for i, h in H.onsite.items():
        Hs = Hs + embed({i: h})
    for (c, p), terms in H.bonds.items():
        for coeff, oc, op in terms:
            Hs = Hs + coeff * embed({c: oc, p: op})
    return Hs


def sparse_ground_energy(Hs):
    """Lowest eigenvalue of a sparse Hermitian matrix (implicitly restarted Lanczos)."""
    import scipy.sparse.linalg as spla
    return float(spla.eigsh(Hs, k=1, which="SA", tol=1e-13)[0][0])


def exact_groundstate(Hd):
    """(GraftTestUtils.jl:468-471)"""
    w, v = np.linalg.eigh((Hd + Hd.conj().T) / 2)
    return w[0], v[:, 0]


def exact_evolve(Hd, v, dz):
    """exp(dz H) v (GraftTestUtils.jl:474-475)."""
    return sla.expm(dz * Hd) @ v


# ---------------------------------------------------------------------------
# TTNO: finite-state construction for nearest-neighbour trees
# ---------------------------------------------------------------------------

VAC, DONE = 0, 1


def ttno_nn(H: NNHamiltonian):
    """TTNO node tensors ``W[n]`` with legs ``(children..., P_out, P_in, parent)``.

    Edge (c -> p) bond states: 0 = identity so far, 1 = a complete term below,
    2 + t = term t of that edge opened at c (awaiting its partner at p).  The root's
    parent leg is the single 'complete' state.  This replaces the state-diagram builder
    (lib/GraftTTNOBuild/src/statediagram.jl:713) for the nearest-neighbour Hamiltonians
    of the hot-path workloads; ``tests/test_oracle.py`` checks it against the dense H
    like test/runtests.jl:362-393 does for ``ttno_from_opsum``.
    """
    t, d = H.topo, H.d
    I = np.eye(d, dtype=np.complex128)

    def bonddim(c):
        return 2 + len(H.bonds.get((c, t.parent[c]), []))

    Ws = []
    for n in range(t.nnodes):
        kids = t.children[n]
        isroot = t.parent[n] < 0
        wp = 1 if isroot else bonddim(n)
        shape = [bonddim(c) for c in kids] + [d, d, wp]
        W = np.zeros(shape, dtype=np.complex128)
        K = len(kids)
        vac = [VAC] * K

        def put(kidstates, pstate, op):
            if isroot:
                if pstate != DONE:
                    return
                pstate = 0
            W[tuple(kidstates) + (slice(None), slice(None), pstate)] += op
        put(vac, VAC, I)
        if n in H.onsite:
            put(vac, DONE, H.onsite[n])
        for i, c in enumerate(kids):
            st = list(vac)
            st[i] = DONE
            put(st, DONE, I)
            for tix, (coeff, oc, op) in enumerate(H.bonds.get((c, n), [])):
                st = list(vac)
                st[i] = 2 + tix
                put(st, DONE, coeff * op)
        if not isroot:
            for tix, (coeff, oc, op) in enumerate(H.bonds.get((n, t.parent[n]), [])):
                put(vac, 2 + tix, oc)
        Ws.append(W)
    return Ws


def ttno_to_dense(topo, Ws):
    """Contract a TTNO to a dense matrix, site 0 slowest (GraftTestUtils.jl:271-300)."""
    N = topo.nnodes
    labels = []
    for n in range(N):
        lab = [c + 1 for c in topo.children[n]] + [-(n + 1), -(N + n + 1)]
        lab.append(-(2 * N + 1) if topo.parent[n] < 0 else n + 1)
        labels.append(lab)
    res = ncon(Ws, labels)
    d = Ws[0].shape[-2]
    return res.reshape(d ** N, d ** N)


# ---------------------------------------------------------------------------
# contraction helper: the reference's pairwise plan executor restated
# (lib/GraftPlanning/src/Planning/executor.jl:16-45, 240 ncon_reference)
# ---------------------------------------------------------------------------


def ncon(tensors, labels, conj=None, order=None):
    """Contract ``tensors`` with ncon labels (positive = summed, -k = output axis k-1).
    ``order`` is the sequence of operand indices absorbed pairwise into the running
    intermediate (the env-first ``preferred_slots`` order of effective.jl:683,971-975);
    default: operands in list order."""
    n = len(tensors)
    conj = conj or [False] * n
    order = list(order) if order is not None else list(range(n))
    ts = [np.conj(t) if c else t for t, c in zip(tensors, conj)]
    cur = ts[order[0]]
    cl = list(labels[order[0]])
    # self traces are not used on this path
    for j in order[1:]:
        t, tl = ts[j], list(labels[j])
        shared = [l for l in cl if l > 0 and l in tl]
        ax_a = [cl.index(l) for l in shared]
        ax_b = [tl.index(l) for l in shared]
        cur = np.tensordot(cur, t, axes=(ax_a, ax_b))
        cl = [l for l in cl if l not in shared] + [l for l in tl if l not in shared]
    assert all(l < 0 for l in cl), f"unresolved labels {cl}"
    perm = sorted(range(len(cl)), key=lambda i: -cl[i])
    return cur.transpose(perm) if cl else cur


# ---------------------------------------------------------------------------
# TTNS (ttns.jl, GraftTestUtils.jl:48-92)
# ---------------------------------------------------------------------------


class TTNS:
    def __init__(self, topo, tensors, center):
        self.topo = topo
        self.tensors = list(tensors)
        self.center = center

    def copy(self):
        return TTNS(self.topo, [a.copy() for a in self.tensors], self.center)

    def physleg(self, n):
        return self.topo.nchildren(n)

    def parentleg(self, n):
        return self.topo.nchildren(n) + 1


def stateleg(topo, u, w):
    """Leg of node u's state tensor pointing to neighbour w (envcache.jl:852-853)."""
    return topo.nchildren(u) + 1 if topo.parent[u] == w else topo.childslot(u, w)


def opleg(topo, u, w):
    """Leg of node u's operator tensor pointing to neighbour w (envcache.jl:856-857)."""
    return topo.nchildren(u) + 2 if topo.parent[u] == w else topo.childslot(u, w)


def left_orth(A):
    """QR across (all legs but last) | last leg (MatrixAlgebraKit left_orth default)."""
    sh = A.shape
    M = A.reshape(-1, sh[-1])
    Q, R = np.linalg.qr(M, mode="reduced")
    return Q.reshape(sh[:-1] + (Q.shape[1],)), R


def _others(N, k):
    return [j for j in range(N) if j != k]


def orth_factor_leg(A, k):
    """(Backend.jl:602-609) QR of A permuted to (others, k); Q has the new bond at k."""
    N = A.ndim
    t = np.moveaxis(A, k, -1)
    Q, C = left_orth(t)
    return np.moveaxis(Q, -1, k), C


def absorb_on_leg(A, C, k):
    """A'[.., y@k, ..] = sum_e C[y, e] A[.., e@k, ..] (Backend.jl:533-543)."""
    t = np.tensordot(C, A, axes=([1], [k]))  # (y, others...)
    return np.moveaxis(t, 0, k)


def move_center_edge(psi: TTNS, m):
    """One gauge step of the centre to neighbour m (ttns.jl:181-203)."""
    t = psi.topo
    n = psi.center
    A = psi.tensors[n]
    if t.parent[n] == m:
        Q, C = left_orth(A)
        psi.tensors[n] = Q
        psi.tensors[m] = absorb_on_leg(psi.tensors[m], C, t.childslot(m, n))
    else:
        k = t.childslot(n, m)
        Q, C = orth_factor_leg(A, k)
        psi.tensors[n] = Q
        psi.tensors[m] = np.tensordot(psi.tensors[m], C.T, axes=([psi.tensors[m].ndim - 1], [0]))
    psi.center = m


def move_center(psi: TTNS, target, on_edge=None):
    """(ttns.jl:126-132)  ``on_edge(n, m)`` is called after every step (cache invalidation)."""
    path = psi.topo.path_between(psi.center, target)
    for i in range(1, len(path)):
        n = psi.center
        move_center_edge(psi, path[i])
        if on_edge is not None:
            on_edge(n, path[i])


def canonicalize(psi: TTNS, center=None):
    """Leaf->root QR sweep then a centre move (GraftTestUtils.jl:48-63)."""
    t = psi.topo
    for n in t.postorder():
        if n == t.root:
            continue
        Q, C = left_orth(psi.tensors[n])
        psi.tensors[n] = Q
        p = t.parent[n]
        psi.tensors[p] = absorb_on_leg(psi.tensors[p], C, t.childslot(p, n))
    psi.center = t.root
    move_center(psi, t.root if center is None else center)
    return psi


def randn_c(rng, shape):
    """Complex normal with unit total variance (Julia randn(ComplexF64) convention)."""
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / math.sqrt(2.0)


def random_ttns(rng, topo, d, bond, center=None):
    """(GraftTestUtils.jl:71-92) randn per node, canonicalize, normalize.  ``bond`` is
    an int or a dict child-node -> dim."""
    def edim(c):
        return bond if isinstance(bond, int) else bond[c]
    ts = []
    for n in range(topo.nnodes):
        shape = [edim(c) for c in topo.children[n]] + [d, 1 if topo.parent[n] < 0 else edim(n)]
        ts.append(randn_c(rng, shape))
    psi = TTNS(topo, ts, topo.root)
    canonicalize(psi, center)
    nrm = np.linalg.norm(psi.tensors[psi.center])
    psi.tensors[psi.center] = psi.tensors[psi.center] / nrm
    return psi


def to_dense(psi: TTNS):
    """State vector, site 0 slowest (GraftTestUtils.jl:245-269)."""
    t = psi.topo
    labels = []
    for n in range(t.nnodes):
        lab = [c + 1 for c in t.children[n]] + [-(n + 1)]
        lab.append(-(t.nnodes + 1) if t.parent[n] < 0 else n + 1)
        labels.append(lab)
    res = ncon(psi.tensors, labels)
    return res.reshape(-1)


def bond_dims(psi):
    return [psi.tensors[c].shape[-1] for c in range(psi.topo.nnodes) if psi.topo.parent[c] >= 0]


# ---------------------------------------------------------------------------
# environments (envcache.jl:919-999, 1010-1101) and the effective maps
# (effective.jl:627-686 h1, 739-749 h0, 878-976 h2)
# ---------------------------------------------------------------------------


def env_spec(topo, u, v, A, W, B_conj=True):
    """Label graph of the sandwich at u with legs towards v open: operands in the
    reference order (ket, envs of neighbours != v ..., root cap?, W, conj(bra)).
    Returns (labels, conj, env_neighbours, has_cap).  Output legs (ket, op, bra)."""
    K = topo.nchildren(u)
    aidx = [0] * A.ndim
    bidx = [0] * A.ndim
    widx = [0] * W.ndim
    nxt = [0]

    def fresh():
        nxt[0] += 1
        return nxt[0]
    pin, pout = fresh(), fresh()
    aidx[K] = pin
    widx[K + 1] = pin
    widx[K] = pout
    bidx[K] = pout
    env_labels, env_nb = [], []
    for w in topo.neighbors(u):
        la = stateleg(topo, u, w)
        if w == v:
            aidx[la] = -1
            widx[opleg(topo, u, w)] = -2
            bidx[la] = -3
        else:
            e = [fresh(), fresh(), fresh()]
            aidx[la] = e[0]
            widx[opleg(topo, u, w)] = e[1]
            bidx[la] = e[2]
            env_labels.append(e)
            env_nb.append(w)
    cap_labels = None
    if topo.parent[u] < 0:
        ka, ko, kb = fresh(), fresh(), fresh()
        aidx[-1] = ka
        bidx[-1] = kb
        widx[-1] = ko
        cap_labels = [kb, ko, ka]
    labels = [aidx] + env_labels + ([cap_labels] if cap_labels else []) + [widx, bidx]
    conj = [False] * (len(labels) - 1) + [True]
    return labels, conj, env_nb, cap_labels is not None


def root_cap(dtype=np.complex128):
    return np.ones((1, 1, 1), dtype=dtype)


def build_env(topo, psi_tensors, Ws, u, v, envs):
    """E(u->v)[ket, op, bra] (envcache.jl:919-999)."""
    A = psi_tensors[u]
    W = Ws[u]
    labels, conj, env_nb, has_cap = env_spec(topo, u, v, A, W)
    ops = [A] + [envs[(w, u)] for w in env_nb] + ([root_cap()] if has_cap else []) + [W, A]
    return ncon(ops, labels, conj)


class EnvCache:
    """Directed-edge environment cache with invalidation (envcache.jl:61-109, 812-844)."""

    def __init__(self, topo):
        self.topo = topo
        self.envs = {}

    def invalidate_edge(self, n, m):
        """Drop every env whose contracted side contains n or m (envcache.jl:830)."""
        self.invalidate_node(n)
        self.invalidate_node(m)

    def invalidate_node(self, n):
        t = self.topo
        drop = []
        for (u, v) in self.envs:
            if n in t.subtree_nodes(u, v):
                drop.append((u, v))
        for k in drop:
            del self.envs[k]

    def env(self, psi, Ws, u, v):
        """Lazy recursive build of E(u->v) (envcache.jl:1440-1476)."""
        key = (u, v)
        if key not in self.envs:
            for w in self.topo.neighbors(u):
                if w != v:
                    self.env(psi, Ws, w, u)
            self.envs[key] = build_env(self.topo, psi.tensors, Ws, u, v, self.envs)
        return self.envs[key]


def h1_spec(topo, n, x_ndim, w_ndim):
    """Labels of the one-site map (effective.jl:627-686).  Operand order
    (x, W, env(w->n) for w in neighbours..., cap?); returns (labels, order)."""
    K = topo.nchildren(n)
    Nx = x_ndim
    xidx = [0] * Nx
    widx = [0] * w_ndim
    labels = [xidx, widx]
    nxt = [0]

    def fresh():
        nxt[0] += 1
        return nxt[0]
    pin = fresh()
    xidx[K] = pin
    widx[K + 1] = pin
    widx[K] = -(K + 1)
    children, parents, caps = [], [], []
    for w in topo.neighbors(n):
        lx = stateleg(topo, n, w)
        kk, oo = fresh(), fresh()
        xidx[lx] = kk
        widx[opleg(topo, n, w)] = oo
        labels.append([kk, oo, -(lx + 1)])
        (parents if topo.parent[n] == w else children).append(len(labels) - 1)
    if topo.parent[n] < 0:
        ka, ko = fresh(), fresh()
        xidx[-1] = ka
        widx[-1] = ko
        labels.append([ka, ko, -Nx])
        caps.append(len(labels) - 1)
    order = [0] + children + [1] + parents + caps
    return labels, order


def two_site_tensor(psi, n, m):
    """Θ legs: A_n codomain legs, then A_m flat legs except slot k (effective.jl:827-843)."""
    t = psi.topo
    assert t.parent[n] == m
    k = t.childslot(m, n)
    A, B = psi.tensors[n], psi.tensors[m]
    return np.tensordot(A, B, axes=([A.ndim - 1], [k]))


def split_two_site(psi, theta, n, m, maxdim=None, atol=0.0, rtol=0.0, discarded_weight=0.0,
                   center_on="n"):
    """Truncated SVD back into A_n, A_m (effective.jl:852-876, Backend.jl:466-505)."""
    t = psi.topo
    k = t.childslot(m, n)
    pn = psi.tensors[n].ndim - 1
    sh = theta.shape
    M = theta.reshape(int(np.prod(sh[:pn])), -1)
    U, S, Vh = np.linalg.svd(M, full_matrices=False)
    r = truncation_rank(S, maxdim, atol, rtol, discarded_weight)
    U, S, Vh = U[:, :r], S[:r], Vh[:r]
    if center_on == "n":
        An, Rm = U * S, Vh
    else:
        An, Rm = U, S[:, None] * Vh
    An = An.reshape(sh[:pn] + (r,))
    Rm = Rm.reshape((r,) + sh[pn:])
    # move the new bond (axis 0) into slot k
    psi.tensors[n] = An
    psi.tensors[m] = np.moveaxis(Rm, 0, k)
    psi.center = n if center_on == "n" else m
    return float(np.sqrt(np.sum(np.linalg.svd(M, compute_uv=False)[r:] ** 2)))


def truncation_rank(S, maxdim=None, atol=0.0, rtol=0.0, discarded_weight=0.0):
    """Rank kept by TruncationScheme (Backend.jl:466-483): truncrank & trunctol & truncerror."""
    r = len(S)
    if maxdim is not None:
        r = min(r, maxdim)
    if atol > 0 or rtol > 0:
        thr = max(atol, rtol * (S[0] if len(S) else 0.0))
        r = min(r, int(np.sum(S > thr)))
    if discarded_weight > 0:
        tot = np.sqrt(np.sum(S ** 2))
        tail = np.sqrt(np.cumsum((S ** 2)[::-1])[::-1])  # tail[i] = norm of S[i:]
        rr = len(S)
        for i in range(len(S)):
            if tail[i] <= discarded_weight * tot:
                rr = i
                break
        r = min(r, rr)
    return max(r, 1)


def h2_spec(topo, n, m, theta_ndim, wn_ndim, wm_ndim, pn):
    """Labels of the two-site map (effective.jl:878-976).  Operand order
    (Θ, Wn, Wm, env(w->n) for children w of n..., env(w->m) for w != n..., cap?)."""
    t = topo
    k = t.childslot(m, n)
    Kn, Km = t.nchildren(n), t.nchildren(m)
    Nx = theta_ndim
    xidx = [0] * Nx
    wnidx = [0] * wn_ndim
    wmidx = [0] * wm_ndim
    labels = [xidx, wnidx, wmidx]
    nxt = [0]

    def fresh():
        nxt[0] += 1
        return nxt[0]

    def mpos(j):  # 0-based leg j of A_m -> position in Θ
        return pn + (j if j < k else j - 1)
    ob = fresh()
    wnidx[-1] = ob
    wmidx[k] = ob
    pin = fresh()
    xidx[Kn] = pin
    wnidx[Kn + 1] = pin
    wnidx[Kn] = -(Kn + 1)
    pin = fresh()
    xidx[mpos(Km)] = pin
    wmidx[Km + 1] = pin
    wmidx[Km] = -(mpos(Km) + 1)
    envn, envmc, envmp, caps = [], [], [], []
    for w in t.neighbors(n):
        if w == m:
            continue
        lx = t.childslot(n, w)
        kk, oo = fresh(), fresh()
        xidx[lx] = kk
        wnidx[lx] = oo
        labels.append([kk, oo, -(lx + 1)])
        envn.append((w, len(labels) - 1))
    for w in t.neighbors(m):
        if w == n:
            continue
        if t.parent[m] == w:
            lw, lx = wm_ndim - 1, Nx - 1
        else:
            lw = t.childslot(m, w)
            lx = mpos(lw)
        kk, oo = fresh(), fresh()
        xidx[lx] = kk
        wmidx[lw] = oo
        labels.append([kk, oo, -(lx + 1)])
        (envmp if t.parent[m] == w else envmc).append((w, len(labels) - 1))
    if t.parent[m] < 0:
        ka, ko = fresh(), fresh()
        xidx[Nx - 1] = ka
        wmidx[-1] = ko
        labels.append([ka, ko, -Nx])
        caps.append(len(labels) - 1)
    order = [0] + [s for _, s in envn] + [1] + [s for _, s in envmc] + [2] + [s for _, s in envmp] + caps
    env_keys = [(w, n) for w, _ in envn] + [(w, m) for w, _ in envmc] + [(w, m) for w, _ in envmp]
    return labels, order, env_keys


class EffMap:
    """y = H_eff x for a fixed label graph and statics (types.jl:410-445)."""

    def __init__(self, labels, order, statics, shape):
        self.labels = labels
        self.order = order
        self.statics = statics       # operands 1.. in label order
        self.shape = shape

    def __call__(self, x):
        return ncon([x] + self.statics, self.labels, None, self.order)


def eff_h1(cache, psi, Ws, n):
    """(effective.jl:709-730)"""
    t = psi.topo
    x = psi.tensors[n]
    labels, order = h1_spec(t, n, x.ndim, Ws[n].ndim)
    statics = [Ws[n]] + [cache.env(psi, Ws, w, n) for w in t.neighbors(n)]
    if t.parent[n] < 0:
        statics.append(root_cap())
    return EffMap(labels, order, statics, x.shape)


def eff_h2(cache, psi, Ws, n, m):
    """(effective.jl:986-1034)"""
    t = psi.topo
    pn = psi.tensors[n].ndim - 1
    Nx = pn + psi.tensors[m].ndim - 1
    labels, order, env_keys = h2_spec(t, n, m, Nx, Ws[n].ndim, Ws[m].ndim, pn)
    statics = [Ws[n], Ws[m]] + [cache.env(psi, Ws, w, u) for (w, u) in env_keys]
    if t.parent[m] < 0:
        statics.append(root_cap())
    shape = psi.tensors[n].shape[:-1] + tuple(
        s for j, s in enumerate(psi.tensors[m].shape) if j != t.childslot(m, n))
    return EffMap(labels, order, statics, shape)


def eff_h0(cache, psi, Ws, n, m):
    """Link map y = E(n->m) C E(m->n) (effective.jl:739-797)."""
    En = cache.env(psi, Ws, n, m)
    Em = cache.env(psi, Ws, m, n)
    labels = [[1, 2], [1, 3, -1], [2, 3, -2]]
    return EffMap(labels, [0, 1, 2], [En, Em], (En.shape[0], Em.shape[0]))


def expect(psi, Ws):
    """<psi|H|psi> / <psi|psi> closed at the centre through eff_h1 (expectation.jl:32-40;
    the closure identity of test/runtests.jl:654-672)."""
    cache = EnvCache(psi.topo)
    c = psi.center
    x = psi.tensors[c]
    y = eff_h1(cache, psi, Ws, c)(x)
    return np.vdot(x, y) / np.vdot(x, x)


# ---------------------------------------------------------------------------
# Krylov solvers (KrylovKit 0.10.4 eigsolve / exponentiate as called at
# lib/GraftGroundState/src/GroundState/GroundState.jl:25-39 and
# lib/GraftEvolution/src/Evolution/Evolution.jl:54-68)
# ---------------------------------------------------------------------------


def _projected(m, k, a, b, s):
    """Projected matrix of a thick-restarted Lanczos basis: kept Ritz values a[:k] coupled to
    column k by the arrow s, then the Lanczos tridiagonal (a, b)."""
    T = np.zeros((m, m))
    T[np.arange(m), np.arange(m)] = a[:m]
    for i in range(k, m - 1):
        T[i, i + 1] = T[i + 1, i] = b[i]
    if k < m:
        T[:k, k] = s[:k]
        T[k, :k] = s[:k]
    return T


def lanczos_min(apply, x0, krylovdim=20, tol=1e-12, maxiter=100):
    """Lowest eigenpair of a Hermitian map as KrylovKit 0.10's Lanczos eigsolve computes it
    for the reference's groundstate_eigsolve_backend (GroundState.jl:25-39): full
    re-orthogonalisation (two classical Gram-Schmidt passes), convergence checked after
    every step on the absolute residual |beta_m q_m| <= tol, and thick restarts that keep
    the lowest (3 krylovdim + 2) / 5 Ritz vectors (Wu and Simon's thick-restart Lanczos).
    Returns (E, v, info)."""
    shape = x0.shape
    n = x0.size
    kd = min(krylovdim, n)
    V = np.zeros((kd + 1, n), dtype=np.complex128)
    V[0] = x0.reshape(-1) / np.linalg.norm(x0)
    a = np.zeros(kd)
    b = np.zeros(kd)
    s = np.zeros(kd)
    k = 0
    matvecs = 0
    theta, resid, v = None, np.inf, V[0]
    for it in range(maxiter):
        m, brk = kd, False
        for j in range(k, kd):
            w = apply(V[j].reshape(shape)).reshape(-1)
            matvecs += 1
            hj = 0.0
            for _ in range(2):
                h = V[: j + 1].conj() @ w
                w = w - V[: j + 1].T @ h
                hj += h[j].real
            a[j] = hj
            b[j] = np.linalg.norm(w)
            if b[j] < 1e-14 * max(1.0, abs(a[j])):
                m, brk = j + 1, True
                break
            V[j + 1] = w / b[j]
            if j + 1 >= 2 or kd == 1:
                ev, Q = np.linalg.eigh(_projected(j + 1, k, a, b, s))
                if abs(b[j] * Q[j, 0]) <= tol:
                    m = j + 1
                    break
        ev, Q = np.linalg.eigh(_projected(m, k, a, b, s))
        theta = ev[0]
        resid = 0.0 if brk else abs(b[m - 1] * Q[m - 1, 0])
        converged = brk or resid <= tol or m == n
        keep = max(0, min((3 * kd + 2) // 5, m - 1))
        if converged or it == maxiter - 1 or keep == 0:
            v = V[:m].T @ Q[:, 0]
            v = v / np.linalg.norm(v)
            if converged or it == maxiter - 1:
                return theta, v.reshape(shape), dict(iters=it + 1, matvecs=matvecs, resid=resid)
            V[0] = v
            k = 0
            continue
        # thick restart: V[:keep] <- V[:m] Q[:, :keep], the residual direction V[m] follows
        V[:keep] = (V[:m].T @ Q[:, :keep]).T
        V[keep] = V[m]
        s[:keep] = b[m - 1] * Q[m - 1, :keep]
        a[:keep] = ev[:keep]
        k = keep
    return theta, v.reshape(shape), dict(iters=maxiter, matvecs=matvecs, resid=resid)


def krylov_expm(apply, dz, x, krylovdim=30, tol=1e-12, max_substeps=64, hermitian=True):
    """exp(dz H) x (KrylovKit's exponentiate as Evolution.jl:54-68 calls it): Lanczos for a
    Hermitian map, Arnoldi otherwise, with the exact small exponential and sub-stepping when
    the a-posteriori error estimate exceeds tol."""
    if not hermitian:
        return _arnoldi_expm(apply, dz, x, krylovdim, tol, max_substeps)
    shape = x.shape
    y = x.reshape(-1).astype(np.complex128)
    remaining = 1.0
    frac = 1.0
    steps = 0
    while remaining > 1e-15:
        step = min(frac, remaining)
        beta0 = np.linalg.norm(y)
        if beta0 == 0:
            return y.reshape(shape)
        n = y.size
        kd = min(krylovdim, n)
        V = np.zeros((kd + 1, n), dtype=np.complex128)
        V[0] = y / beta0
        a = np.zeros(kd)
        b = np.zeros(kd)
        m = kd
        for j in range(kd):
            w = apply(V[j].reshape(shape)).reshape(-1)
            a[j] = np.vdot(V[j], w).real
            for _ in range(2):
                w = w - V[: j + 1].T @ (V[: j + 1].conj() @ w)
            b[j] = np.linalg.norm(w)
            if b[j] < 1e-14 * max(1.0, abs(a[j])):
                m = j + 1
                break
            V[j + 1] = w / b[j]
        T = np.diag(a[:m]) + np.diag(b[: m - 1], 1) + np.diag(b[: m - 1], -1)
        evals, Q = np.linalg.eigh(T)
        c = Q @ (np.exp(dz * step * evals) * Q[0].conj())
        err = beta0 * abs(b[m - 1] * c[m - 1]) if m == kd else 0.0
        if err > tol and steps < max_substeps:
            frac = step / 2
            steps += 1
            continue
        y = beta0 * (V[:m].T @ c)
        remaining -= step
    return y.reshape(shape)


def _arnoldi_expm(apply, dz, x, krylovdim=30, tol=1e-12, max_substeps=64):
    """Arnoldi form of krylov_expm for a map that is not Hermitian: two classical
    Gram-Schmidt passes, the Hessenberg projection H_m, exp(dz H_m) e_1 by scipy's expm,
    error estimate beta |h(m+1,m)| |(exp(dz H_m) e_1)_m|."""
    shape = x.shape
    y = x.reshape(-1).astype(np.complex128)
    remaining = 1.0
    frac = 1.0
    steps = 0
    while remaining > 1e-15:
        step = min(frac, remaining)
        beta0 = np.linalg.norm(y)
        if beta0 == 0:
            return y.reshape(shape)
        n = y.size
        kd = min(krylovdim, n)
        V = np.zeros((kd + 1, n), dtype=np.complex128)
        V[0] = y / beta0
        Hm = np.zeros((kd + 1, kd), dtype=np.complex128)
        m = kd
        for j in range(kd):
            w = apply(V[j].reshape(shape)).reshape(-1)
            for _ in range(2):
                h = V[: j + 1].conj() @ w
                w = w - V[: j + 1].T @ h
                Hm[: j + 1, j] += h
            Hm[j + 1, j] = np.linalg.norm(w)
            if Hm[j + 1, j].real < 1e-13 * max(1.0, np.max(np.abs(Hm[: j + 1, j]))):
                m = j + 1
                break
            V[j + 1] = w / Hm[j + 1, j].real
        c = sla.expm(dz * step * Hm[:m, :m])[:, 0]
        err = beta0 * abs(Hm[m, m - 1]) * abs(c[m - 1]) if m == kd else 0.0
        if err > tol and steps < max_substeps:
            frac = step / 2
            steps += 1
            continue
        y = beta0 * (V[:m].T @ c)
        remaining -= step
    return y.reshape(shape)


# ---------------------------------------------------------------------------
# solvers: dmrg2! (GroundState.jl:102-143) and TDVP1 (tdvp.jl:171-301)
# ---------------------------------------------------------------------------


def dmrg2(psi, Ws, maxdim=None, nsweeps=10, tol=1e-10, krylovdim=20, atol=0.0, lanczos_tol=1e-12):
    t = psi.topo
    cache = EnvCache(t)
    energies = []
    bonds = [n for n in t.postorder() if t.parent[n] >= 0]
    sched = [(n, "m") for n in bonds] + [(n, "n") for n in reversed(bonds)]
    for sweep in range(nsweeps):
        E = float("nan")
        for n, center_on in sched:
            m = t.parent[n]
            move_center(psi, n, cache.invalidate_edge)
            theta = two_site_tensor(psi, n, m)
            h2 = eff_h2(cache, psi, Ws, n, m)
            E, v, _ = lanczos_min(h2, theta, krylovdim=krylovdim, tol=lanczos_tol)
            cache.invalidate_edge(n, m)
            split_two_site(psi, v, n, m, maxdim=maxdim, atol=atol, center_on=center_on)
        energies.append(float(E))
        if len(energies) >= 2 and abs(energies[-1] - energies[-2]) < tol:
            break
    return psi, energies


def dmrg1(psi, Ws, nsweeps=10, tol=1e-10, krylovdim=20, lanczos_tol=1e-12):
    """Single-site DMRG with fixed bond dimensions (GroundState.jl:51-84): postorder then
    reverse postorder, the local ground state of eff_h1 at every node."""
    t = psi.topo
    cache = EnvCache(t)
    energies = []
    order = t.postorder()
    for sweep in range(nsweeps):
        E = float("nan")
        for n in list(order) + list(reversed(order)):
            move_center(psi, n, cache.invalidate_edge)
            h1 = eff_h1(cache, psi, Ws, n)
            E, v, _ = lanczos_min(h1, psi.tensors[n], krylovdim=krylovdim, tol=lanczos_tol)
            psi.tensors[n] = v
            cache.invalidate_node(n)
        energies.append(float(E))
        if len(energies) >= 2 and abs(energies[-1] - energies[-2]) < tol:
            break
    return psi, energies


def _svd_keep(M, maxdim=None, atol=0.0, rtol=0.0):
    """Left singular vectors kept by TruncationScheme(maxdim, atol, rtol)."""
    U, S, _ = np.linalg.svd(M, full_matrices=False)
    r = truncation_rank(S, maxdim, atol, rtol)
    return U[:, :r], S[:r]


EXPAND_SCHEMES = ("exact", "directqr", "rsvd", "rangefinder")


def predictor_probe(rng, rest, budget):
    """Gaussian probe block (rest x budget, complex, unit variance) for the randomised
    predictor schemes (expansion.jl:372-446).  The reference draws it from a caller-owned
    Xoshiro stream, which cannot be reproduced here; this restatement draws the real parts,
    then the imaginary parts, from a numpy Generator, the convention the device path shares."""
    return (rng.standard_normal((rest, budget)) + 1j * rng.standard_normal((rest, budget))) / np.sqrt(2.0)


def predictor_basis(P, cap, scheme="exact", rng=None, oversample=8, poweriter=0):
    """Child predictor basis of the (n-side legs) x (rest) matrix P (_child_predictor_basis,
    expansion.jl:240-370): exact = its leading cap left singular vectors; directqr = Q of its
    compact QR; rsvd = the leading cap left singular vectors of Y = (P P^H)^q P Omega;
    rangefinder = Q of QR(P Omega) after q QR-stabilised power steps.  Omega has
    min(rest, cap + oversample) columns."""
    if scheme == "exact":
        U, _ = _svd_keep(P, cap)
        return U
    if scheme == "directqr":
        Q, _ = np.linalg.qr(P, mode="reduced")
        return Q
    if scheme not in ("rsvd", "rangefinder"):
        raise ValueError(f"expand: scheme must be one of {EXPAND_SCHEMES}")
    if rng is None:
        raise ValueError(f"expand: scheme={scheme} requires an explicit rng")
    budget = min(P.shape[1], cap + oversample)
    Om = predictor_probe(rng, P.shape[1], budget)
    if scheme == "rsvd":
        Y = P @ Om
        for _ in range(poweriter):
            Y = P @ (P.conj().T @ Y)
        U, _ = _svd_keep(Y, cap)
        return U
    Q, _ = np.linalg.qr(P @ Om, mode="reduced")
    for _ in range(poweriter):
        Z, _ = np.linalg.qr(P.conj().T @ Q, mode="reduced")
        Q, _ = np.linalg.qr(P @ Z, mode="reduced")
    return Q


def factorized_rangefinder_enrichment(Am, P, room, rng, oversample=8, poweriter=0, enr_atol=1e-12,
                                      enr_rtol=1e-10):
    """Enrichment of the factorised range finder (_factorized_rangefinder_enrich_split,
    expansion.jl:134-216) for the n-side matrix A_n and the predictor P = mixing * H2 Theta:
    kept Q = QR(A_n); N = orthonormal complement of range(Q); the range finder (:280-326)
    on the complement-side operator N^H P (probes of min(rest, room + oversample) columns,
    poweriter QR-stabilised steps) gives S; the left singular vectors of S^H N^H P kept by
    (maxdim = room, atol, rtol) give L; the enrichment is E = N S L.  Returns (Q, E), E None
    when nothing is added."""
    Q, _ = np.linalg.qr(Am, mode="reduced")
    full, _ = np.linalg.qr(np.concatenate([Q, np.eye(Am.shape[0])], axis=1), mode="reduced")
    N = full[:, Q.shape[1]:Am.shape[0]]
    if room <= 0 or N.shape[1] == 0:
        return Q, None
    NP = N.conj().T @ P
    sk = min(P.shape[1], room + oversample)
    S, _ = np.linalg.qr(NP @ predictor_probe(rng, P.shape[1], sk), mode="reduced")
    for _ in range(poweriter):
        Z, _ = np.linalg.qr(NP.conj().T @ S, mode="reduced")
        S, _ = np.linalg.qr(NP @ Z, mode="reduced")
    L, _ = _svd_keep(S.conj().T @ NP, room, enr_atol, enr_rtol)
    if L.shape[1] == 0:
        return Q, None
    return Q, N @ (S @ L)


def expand_exact(psi, Ws, cache, n, m, maxdim, max_add=8, mixing=1.0, enr_rtol=1e-10, enr_atol=1e-12):
    """expand with the exact predictor scheme."""
    return expand(psi, Ws, cache, n, m, maxdim, max_add, mixing, enr_rtol, enr_atol, scheme="exact")


def expand(psi, Ws, cache, n, m, maxdim, max_add=8, mixing=1.0, enr_rtol=1e-10, enr_atol=1e-12,
           scheme="exact", rng=None, oversample=8, poweriter=0, factorized=False):
    """3S subspace expansion of the bond n -> m (expand!, unfactorised branch,
    expansion.jl:40-131, 240-370, 488-512): the predictor basis P of mixing * H2 Theta
    (n-side legs x rest, predictor_basis with cap = min(maxdim, D + max_add)); the
    directions of P outside range(A_n) (left singular vectors of N^H P with N the
    complement of range(A_n), at most cap - D, atol / rtol enrichment tolerances) are
    appended to A_n; the factor U of [A_n E] (at most cap columns) replaces A_n and
    R = U^H A_n is absorbed into A_m.  factorized with scheme rangefinder takes the factorised
    range finder's enrichment instead, and U = [Q E] with no final SVD."""
    if scheme not in EXPAND_SCHEMES:
        raise ValueError(f"expand: scheme must be one of {EXPAND_SCHEMES}")
    if scheme in ("rsvd", "rangefinder") and rng is None:
        raise ValueError(f"expand: scheme={scheme} requires an explicit rng")
    t = psi.topo
    olddim = psi.tensors[n].shape[-1]
    cap = min(maxdim, olddim + max_add)
    if cap <= olddim or mixing == 0:
        return
    move_center(psi, n, cache.invalidate_edge)
    A = psi.tensors[n]
    sh = A.shape
    Am = A.reshape(-1, sh[-1])
    theta = two_site_tensor(psi, n, m)
    P = (mixing * eff_h2(cache, psi, Ws, n, m)(theta)).reshape(Am.shape[0], -1)
    if factorized and scheme == "rangefinder":
        Q, E = factorized_rangefinder_enrichment(Am, P, cap - olddim, rng, oversample, poweriter, enr_atol,
                                                 enr_rtol)
        if E is None:
            return
        U = np.concatenate([Q, E], axis=1)
        R = U.conj().T @ Am
        psi.tensors[n] = U.reshape(sh[:-1] + (U.shape[1],))
        psi.tensors[m] = absorb_on_leg(psi.tensors[m], R, t.childslot(m, n))
        psi.center = m
        cache.invalidate_edge(n, m)
        return
    P = predictor_basis(P, cap, scheme, rng, oversample, poweriter)
    room = min(max_add, cap - olddim)
    expanded = Am
    if room > 0 and Am.shape[0] > Am.shape[1]:
        U, S, _ = np.linalg.svd(Am, full_matrices=True)
        rank = int(np.sum(S > 1e-14 * max(S[0], 1e-300))) if S.size else 0
        N = U[:, rank:]
        if N.shape[1] > 0:
            Um, _ = _svd_keep(N.conj().T @ P, room, enr_atol, enr_rtol)
            if Um.shape[1] > 0:
                expanded = np.concatenate([Am, N @ Um], axis=1)
    U, _ = _svd_keep(expanded, cap)
    if U.shape[1] == olddim:
        return
    R = U.conj().T @ Am
    psi.tensors[n] = U.reshape(sh[:-1] + (U.shape[1],))
    psi.tensors[m] = absorb_on_leg(psi.tensors[m], R, t.childslot(m, n))
    psi.center = m
    cache.invalidate_edge(n, m)


def dmrg1_3s(psi, Ws, maxdim=100, nsweeps=10, tol=1e-10, krylovdim=20, mixing=1.0, max_add=8,
             enr_rtol=1e-10, enr_atol=1e-12, lanczos_tol=1e-12, expand_scheme="exact", rng=None,
             rsvd_oversample=8, rsvd_poweriter=0):
    """Single-site DMRG with subspace expansion after every sweep (GroundState.jl:166-248):
    dmrg1's local updates, then expand with expand_scheme on every bond in postorder, with
    factorized=true as the reference passes it (so rangefinder is the factorised range
    finder); the randomised schemes draw their probes from rng, bond by bond."""
    if expand_scheme not in EXPAND_SCHEMES:
        raise ValueError(f"dmrg1_3s: expand_scheme must be one of {EXPAND_SCHEMES}")
    if expand_scheme in ("rsvd", "rangefinder") and rng is None:
        raise ValueError(f"dmrg1_3s: expand_scheme={expand_scheme} requires an explicit rng")
    t = psi.topo
    cache = EnvCache(t)
    energies = []
    order = t.postorder()
    bonds = [n for n in order if t.parent[n] >= 0]
    for sweep in range(nsweeps):
        E = float("nan")
        for n in list(order) + list(reversed(order)):
            move_center(psi, n, cache.invalidate_edge)
            h1 = eff_h1(cache, psi, Ws, n)
            E, v, _ = lanczos_min(h1, psi.tensors[n], krylovdim=krylovdim, tol=lanczos_tol)
            psi.tensors[n] = v
            cache.invalidate_node(n)
        alpha = mixing(sweep + 1) if callable(mixing) else mixing
        if alpha != 0:
            for n in bonds:
                expand(psi, Ws, cache, n, t.parent[n], maxdim, max_add, alpha, enr_rtol, enr_atol,
                       expand_scheme, rng, rsvd_oversample, rsvd_poweriter, factorized=True)
        energies.append(float(E))
        if len(energies) >= 2 and abs(energies[-1] - energies[-2]) < tol:
            break
    return psi, energies


def tdvp1_step(psi, Ws, dz, cache=None, krylovdim=30, tol=1e-12, hermitian=True):
    """Order-2 TDVP1 step (tdvp.jl:171-195): forward half sweep with the turning site
    evolved by the full dz, then the reverse half sweep skipping that site."""
    cache = cache or EnvCache(psi.topo)
    _tdvp1_sweep(psi, Ws, dz / 2, cache, rev=False, terminal_dz=dz, krylovdim=krylovdim, tol=tol,
                 hermitian=hermitian)
    _tdvp1_sweep(psi, Ws, dz / 2, cache, rev=True, skip_initial=True, krylovdim=krylovdim, tol=tol,
                 hermitian=hermitian)
    return cache


def _tdvp1_sweep(psi, Ws, dz, cache, rev, terminal_dz=None, skip_initial=False, krylovdim=30, tol=1e-12,
                 hermitian=True):
    """(tdvp.jl:197-249)"""
    t = psi.topo
    order = t.postorder()
    if rev:
        order = order[::-1]
    move_center(psi, order[0], cache.invalidate_edge)
    for i, n in enumerate(order):
        assert psi.center == n
        if not (skip_initial and i == 0):
            sdz = terminal_dz if (terminal_dz is not None and i == len(order) - 1) else dz
            h1 = eff_h1(cache, psi, Ws, n)
            A = krylov_expm(h1, sdz, psi.tensors[n], krylovdim=krylovdim, tol=tol, hermitian=hermitian)
            psi.tensors[n] = A
            cache.invalidate_node(n)
        if i == len(order) - 1:
            break
        seg = t.path_between(n, order[i + 1])
        for j in range(1, len(seg)):
            u, v = seg[j - 1], seg[j]
            if (t.parent[u] == v) != rev:
                _evolve_link_and_move(psi, Ws, u, v, dz, cache, krylovdim, tol, hermitian)
            else:
                move_center(psi, v, cache.invalidate_edge)


def _evolve_link_and_move(psi, Ws, u, v, dz, cache, krylovdim, tol, hermitian=True):
    """(tdvp.jl:257-301) QR split, backward link evolution with eff_h0, absorb."""
    t = psi.topo
    if t.parent[u] == v:
        Q, C = left_orth(psi.tensors[u])
        psi.tensors[u] = Q
        cache.invalidate_node(u)
        k0 = eff_h0(cache, psi, Ws, u, v)
        C = krylov_expm(k0, -dz, C, krylovdim=krylovdim, tol=tol, hermitian=hermitian)
        psi.tensors[v] = absorb_on_leg(psi.tensors[v], C, t.childslot(v, u))
    else:
        k = t.childslot(u, v)
        Q, Cd = orth_factor_leg(psi.tensors[u], k)
        psi.tensors[u] = Q
        C = Cd.T
        cache.invalidate_node(u)
        k0 = eff_h0(cache, psi, Ws, v, u)
        C = krylov_expm(k0, -dz, C, krylovdim=krylovdim, tol=tol, hermitian=hermitian)
        psi.tensors[v] = np.tensordot(psi.tensors[v], C, axes=([psi.tensors[v].ndim - 1], [0]))
    psi.center = v
    cache.invalidate_node(v)


def tdvp2_step(psi, Ws, dz, cache=None, maxdim=None, atol=0.0, krylovdim=30, tol=1e-12):
    """Order-2 TDVP2 step with the fused turning bond (tdvp.jl:307-329): forward half sweep
    whose last bond is evolved by the full dz and split onto the child, then the reverse
    half sweep that skips that bond."""
    cache = cache or EnvCache(psi.topo)
    opts = dict(maxdim=maxdim, atol=atol, krylovdim=krylovdim, tol=tol)
    _tdvp2_sweep(psi, Ws, dz / 2, cache, rev=False, terminal_dz=dz, opts=opts)
    _tdvp2_sweep(psi, Ws, dz / 2, cache, rev=True, skip_initial=True, opts=opts)
    return cache


def _tdvp2_sweep(psi, Ws, dz, cache, rev, terminal_dz=None, skip_initial=False, opts=None):
    """(tdvp.jl:340-388) Two-site forward evolution of every bond (postorder child nodes);
    a backward one-site evolution of the parent between consecutive bonds, before the
    bond in reverse, after it forward; none at the turning bond."""
    t = psi.topo
    bonds = [n for n in t.postorder() if t.parent[n] >= 0]
    last = len(bonds) - 1
    idx = range(last, -1, -1) if rev else range(last + 1)
    for j in idx:
        if rev and skip_initial and j == last:
            continue
        n = bonds[j]
        m = t.parent[n]
        move_center(psi, m, cache.invalidate_edge)
        if rev:
            if j != last:
                _tdvp2_site_backward(psi, Ws, m, dz, cache, opts)
            _tdvp2_bond_forward(psi, Ws, n, m, dz, "n", cache, opts)
        else:
            term = terminal_dz is not None and j == last
            _tdvp2_bond_forward(psi, Ws, n, m, terminal_dz if term else dz, "n" if term else "m", cache, opts)
            if j != last:
                _tdvp2_site_backward(psi, Ws, m, dz, cache, opts)


def _tdvp2_bond_forward(psi, Ws, n, m, dz, center_on, cache, opts):
    """(tdvp.jl:390-410)"""
    theta = two_site_tensor(psi, n, m)
    h2 = eff_h2(cache, psi, Ws, n, m)
    theta = krylov_expm(h2, dz, theta, krylovdim=opts["krylovdim"], tol=opts["tol"])
    cache.invalidate_edge(n, m)
    split_two_site(psi, theta, n, m, maxdim=opts["maxdim"], atol=opts["atol"], center_on=center_on)


def _tdvp2_site_backward(psi, Ws, m, dz, cache, opts):
    """(tdvp.jl:412-431)"""
    assert psi.center == m
    h1 = eff_h1(cache, psi, Ws, m)
    psi.tensors[m] = krylov_expm(h1, -dz, psi.tensors[m], krylovdim=opts["krylovdim"], tol=opts["tol"])
    cache.invalidate_node(m)


# ---------------------------------------------------------------------------
# cost model: algorithmic flops of the env-first plan (complex MAC = 8 flop)
# ---------------------------------------------------------------------------


def plan_macs(shapes, labels, order):
    """Complex MACs of the pairwise plan: sum over steps of prod(free A) * prod(contracted)
    * prod(free B) (the dense counterpart of Backend.jl:328-368 per-block m*k*n)."""
    dims = {}
    for sh, lab in zip(shapes, labels):
        for s, l in zip(sh, lab):
            dims[l] = s
    cl = list(labels[order[0]])
    macs = 0
    for j in order[1:]:
        tl = labels[j]
        shared = [l for l in cl if l > 0 and l in tl]
        fa = [l for l in cl if l not in shared]
        fb = [l for l in tl if l not in shared]
        macs += (math.prod(dims[l] for l in fa) * math.prod(dims[l] for l in shared)
                 * math.prod(dims[l] for l in fb))
        cl = fa + fb
    return macs


# ---------------------------------------------------------------------------
# TDVP1_CBE with PredictorCBE (lib/GraftEvolution/src/Evolution/cbe.jl:132-148,240-259,
# 308-352,418-589,741-806; factor frames lib/GraftContractions/src/Contractions/
# two_site_factor_frame.jl:118-160,308-426), dense exact-SVD path
# ---------------------------------------------------------------------------


def _left_null(Q):
    """Orthonormal complement of Q's columns (MatrixAlgebraKit left_null)."""
    m, r = Q.shape
    if r >= m:
        return np.zeros((m, 0), dtype=Q.dtype)
    full, _ = np.linalg.qr(np.concatenate([Q, randn_c(np.random.default_rng(0), (m, m - r))], axis=1))
    N = full[:, r:]
    N = N - Q @ (Q.conj().T @ N)
    N, _ = np.linalg.qr(N)
    return N


def _edge_frames(psi, u, v):
    """(active matrix ext_u x edge, partner matrix ext_v x edge, restore info) with the
    active endpoint u (cbe.jl:270-295)."""
    t = psi.topo
    Au, Av = psi.tensors[u], psi.tensors[v]
    if t.parent[u] == v:
        ku = Au.ndim - 1                   # u's parent leg
        kv = t.childslot(v, u)
    else:
        ku = t.childslot(u, v)
        kv = Av.ndim - 1
    act = np.moveaxis(Au, ku, -1)
    par = np.moveaxis(Av, kv, -1)
    return act.reshape(-1, act.shape[-1]), par.reshape(-1, par.shape[-1]), ku, kv, act.shape, par.shape


def _site_half(cache, psi, Ws, site, peer, X, k_site):
    """Half of the two-site sandwich at `site` (two_site_factor_frame.jl:308-403): X (the
    site tensor in its original leg order; its leg k_site faces `peer`) contracted with W and
    the environments of every neighbour except `peer`.  Result legs: (the external legs in
    original order..., edge ket, edge op)."""
    t = psi.topo
    W = Ws[site]
    N = X.ndim
    order = [j for j in range(N) if j != k_site] + [k_site]
    out_pos = {raw: j for j, raw in enumerate(order)}     # raw leg -> output position
    K = t.nchildren(site)
    xidx = [0] * N
    widx = [0] * W.ndim
    labels = [xidx, widx]
    nxt = [0]

    def fresh():
        nxt[0] += 1
        return nxt[0]
    xidx[k_site] = -N
    widx[opleg(t, site, peer)] = -(N + 1)
    pin = fresh()
    xidx[K] = pin
    widx[K + 1] = pin
    widx[K] = -(out_pos[K] + 1)
    statics = [W]
    for w in t.neighbors(site):
        if w == peer:
            continue
        raw = stateleg(t, site, w)
        kk, oo = fresh(), fresh()
        xidx[raw] = kk
        widx[opleg(t, site, w)] = oo
        labels.append([kk, oo, -(out_pos[raw] + 1)])
        statics.append(cache.env(psi, Ws, w, site))
    if t.parent[site] < 0:
        raw = N - 1
        ka, ko = fresh(), fresh()
        xidx[raw] = ka
        widx[-1] = ko
        labels.append([ka, ko, -(out_pos[raw] + 1)])
        statics.append(root_cap())
    return ncon([X] + statics, labels)


def cbe_split(psi, Ws, cache, u, v, dz, maxdim, max_add=16, spawn_threshold=1e-10, neigs=2):
    """PredictorCBE split of the active endpoint u towards v (cbe.jl:741-806): returns
    (U as the new site tensor of u in its original leg order, the link R for the backward
    step in (new, edge) orientation of an up move or (edge, new) of a down move)."""
    t = psi.topo
    act, par, ku, kv, ashape, pshape = _edge_frames(psi, u, v)
    Q, link = np.linalg.qr(act)
    r = Q.shape[1]
    room = max(0, maxdim - r)
    budget = min(room, max_add, neigs)
    E = np.zeros((Q.shape[0], 0), dtype=Q.dtype)
    if budget > 0 and dz != 0:
        Na, Np = _left_null(Q), _left_null(par)
        if Na.shape[1] > 0 and Np.shape[1] > 0:
            Xq = np.moveaxis(Q.reshape(ashape[:-1] + (r,)), -1, ku)
            Xp = psi.tensors[v]
            S = _site_half(cache, psi, Ws, u, v, Xq, ku)          # ext_u..., a, o
            T = _site_half(cache, psi, Ws, v, u, Xp, kv)          # ext_v..., b, o
            S = S.reshape(-1, S.shape[-2], S.shape[-1])
            T = T.reshape(-1, T.shape[-2], T.shape[-1])
            # M = Na^H S link T^T conj(Np)  (biprojected core, contract_biprojected_two_site)
            SL = np.einsum("xao,ab->xbo", S, link)
            M = np.einsum("xi,xbo,ybo,yj->ij", Na.conj(), SL, T, Np.conj())
            Uu, sv, _ = np.linalg.svd(M, full_matrices=False)
            cutoff = spawn_threshold * max(np.linalg.norm(act), 1e-300) / abs(dz)
            keep = [i for i in range(min(budget, len(sv))) if sv[i] >= cutoff]
            E = Na @ Uu[:, keep]
    Unew = np.concatenate([Q, E], axis=1)
    R = Unew.conj().T @ act
    Ut = np.moveaxis(Unew.reshape(ashape[:-1] + (Unew.shape[1],)), -1, ku)
    return Ut, R


def tdvp1_cbe_step(psi, Ws, dz, cache=None, maxdim=16, max_add=16, spawn_threshold=1e-10, neigs=2,
                   krylovdim=30, tol=1e-12, enabled=True):
    """Order-2 TDVP1_CBE step: the TDVP1 sweep with the link split replaced by the
    PredictorCBE expansion (tdvp.jl:171-301 with cbe.jl:775-806)."""
    cache = cache or EnvCache(psi.topo)
    opts = dict(maxdim=maxdim, max_add=max_add, spawn_threshold=spawn_threshold, neigs=neigs, enabled=enabled)
    _tdvp1_cbe_sweep(psi, Ws, dz / 2, cache, False, dz, False, krylovdim, tol, opts)
    _tdvp1_cbe_sweep(psi, Ws, dz / 2, cache, True, None, True, krylovdim, tol, opts)
    return cache


def _tdvp1_cbe_sweep(psi, Ws, dz, cache, rev, terminal_dz, skip_initial, krylovdim, tol, opts):
    t = psi.topo
    order = t.postorder()
    if rev:
        order = order[::-1]
    move_center(psi, order[0], cache.invalidate_edge)
    for i, n in enumerate(order):
        if not (skip_initial and i == 0):
            sdz = terminal_dz if (terminal_dz is not None and i == len(order) - 1) else dz
            h1 = eff_h1(cache, psi, Ws, n)
            psi.tensors[n] = krylov_expm(h1, sdz, psi.tensors[n], krylovdim=krylovdim, tol=tol)
            cache.invalidate_node(n)
        if i == len(order) - 1:
            break
        seg = t.path_between(n, order[i + 1])
        for j in range(1, len(seg)):
            u, v = seg[j - 1], seg[j]
            if (t.parent[u] == v) != rev:
                _cbe_link_and_move(psi, Ws, u, v, dz, cache, krylovdim, tol, opts)
            else:
                move_center(psi, v, cache.invalidate_edge)


def _cbe_link_and_move(psi, Ws, u, v, dz, cache, krylovdim, tol, opts):
    t = psi.topo
    if not opts["enabled"]:
        return _evolve_link_and_move(psi, Ws, u, v, dz, cache, krylovdim, tol)
    Ut, R = cbe_split(psi, Ws, cache, u, v, dz, opts["maxdim"], opts["max_add"], opts["spawn_threshold"],
                      opts["neigs"])
    psi.tensors[u] = Ut
    cache.invalidate_node(u)
    if t.parent[u] == v:
        k0 = eff_h0(cache, psi, Ws, u, v)
        C = krylov_expm(k0, -dz, R, krylovdim=krylovdim, tol=tol)
        psi.tensors[v] = absorb_on_leg(psi.tensors[v], C, t.childslot(v, u))
    else:
        k0 = eff_h0(cache, psi, Ws, v, u)
        C = krylov_expm(k0, -dz, R.T, krylovdim=krylovdim, tol=tol)
        psi.tensors[v] = np.tensordot(psi.tensors[v], C, axes=([psi.tensors[v].ndim - 1], [0]))
    psi.center = v
    cache.invalidate_node(v)
