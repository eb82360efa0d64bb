"""U(1) block-sparse test networks (shared by the CPU planner test and the GPU tests):
the two-site map of an edge of a binary tree with Sz-conserving Heisenberg TTNO tensors
and random charge-conserving environments."""
import numpy as np

import grafttn as G
from grafttn import blocksparse as B
from grafttn import contractions as GC

PHYS = {0: 1, 1: 1}


def subtree_sites(topo, c):
    return len(topo.subtree_nodes(c, topo.parent[c]))


def h2_u1_case(depth, n_name, D, seed=11):
    """(plan inputs, dense oracle inputs) for eff_h2 on edge n -> parent(n) of
    binary_topology(depth); bond sectors follow the subtree charge counts scaled to D."""
    topo = G.binary_topology(depth)
    n = topo.index[n_name]
    m = topo.parent[n]
    k = topo.childslot(m, n)
    rng = np.random.default_rng(seed)
    bond = {c: B.binomial_sectors(subtree_sites(topo, c), D) for c in range(1, topo.nnodes)}
    terms = B.u1_heisenberg_terms()
    H = G.NNHamiltonian(topo)
    for e in topo.edges():
        H.bonds[e] = list(terms)
    Wd = G.ttno_tensors(H)
    oleg_out, operm = B.op_leg(+1)
    oleg_in, _ = B.op_leg(-1)

    def w_block(u):
        W = Wd[u]
        K = topo.nchildren(u)
        for ax in list(range(K)) + [K + 2]:
            if topo.parent[u] < 0 and ax == K + 2:
                continue
            W = np.take(W, operm, axis=ax)
        legs = [oleg_out] * K + [B.U1Leg(PHYS, 1), B.U1Leg(PHYS, -1)]
        legs.append(oleg_in if topo.parent[u] >= 0 else B.U1Leg({0: 1}, -1))
        T = B.BlockTensor(legs)
        return T, T.from_dense(W)
    # Θ legs: n's children, phys_n, m's other children, phys_m, m's parent
    xlegs = [B.U1Leg(bond[c], 1) for c in topo.children[n]] + [B.U1Leg(PHYS, 1)]
    xlegs += [B.U1Leg(bond[c], 1) for c in topo.children[m] if c != n] + [B.U1Leg(PHYS, 1)]
    xlegs.append(B.U1Leg(bond[m], -1) if topo.parent[m] >= 0 else B.U1Leg({0: 1}, -1))
    xs = B.BlockTensor(xlegs)
    pn = topo.nchildren(n) + 1
    Wn_t, Wn_d = w_block(n)
    Wm_t, Wm_d = w_block(m)
    labels, order, envs = GC.h2_spec(topo, n, m, len(xlegs), len(Wn_t.legs), len(Wm_t.legs), pn)
    statics = [(Wn_t, labels[1], Wn_d), (Wm_t, labels[2], Wm_d)]
    for (w, u), lab in zip(envs, labels[3:]):
        if w == topo.parent[u]:            # environment from above: ket +, op +, bra -
            sec = bond[u]
            legs = [B.U1Leg(sec, 1), oleg_out, B.U1Leg(sec, -1)]
        else:                               # environment of a child subtree: ket -, op -, bra +
            sec = bond[w]
            legs = [B.U1Leg(sec, -1), oleg_in, B.U1Leg(sec, 1)]
        T = B.BlockTensor(legs)
        statics.append((T, lab, T.random(rng) / np.sqrt(max(1, legs[0].total))))
    if topo.parent[m] < 0:
        raise ValueError("pick an edge below the root's children")
    x = xs.random(rng)
    x /= np.linalg.norm(x)
    del k
    return xs, labels, order, statics, x


def dense_reference(xs, labels, order, statics, x):
    from oracle import ttn_oracle as O
    dense = [xs.to_dense(x)] + [T.to_dense(d) for T, _, d in statics]
    return O.ncon(dense, labels, None, order)
