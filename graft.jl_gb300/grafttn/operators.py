"""Spin operators, nearest-neighbour tree Hamiltonians and their TTNO tensors (host side).

The TTNO is a static input of the hot path (the reference builds it with
``ttno_from_opsum``, lib/GraftTTNOBuild/src/statediagram.jl:713).  For the
nearest-neighbour Hamiltonians of the workloads the operator bond of edge (c -> p)
carries: 0 = nothing placed yet, 1 = a finished term below, 2 + t = term t of that edge
opened at c.  Node tensor legs follow the reference (lib/GraftNetworks/src/Networks/ttno.jl:1-9):
``(children..., P_out, P_in, parent)``; the root's parent leg keeps only the finished state.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .topology import TreeTopology


def spin_ops():
    """Pauli X, Y, Z, raising/lowering and identity on C^2 (Symbolic.jl:177-185)."""
    c = np.complex128
    return dict(
        X=np.array([[0, 1], [1, 0]], dtype=c),
        Y=np.array([[0, -1j], [1j, 0]], dtype=c),
        Z=np.array([[1, 0], [0, -1]], dtype=c),
        Sp=np.array([[0, 1], [0, 0]], dtype=c),
        Sm=np.array([[0, 0], [1, 0]], dtype=c),
        N=np.array([[0, 0], [0, 1]], dtype=c),
        I=np.eye(2, dtype=c),
    )


@dataclass
class NNHamiltonian:
    """One-body ``onsite[n]`` and two-body ``bonds[(child, parent)] = [(coeff, O_c, O_p)]``."""
    topo: TreeTopology
    d: int = 2
    onsite: dict = field(default_factory=dict)
    bonds: dict = field(default_factory=dict)
    hermitian: bool = True


def tfi(topo, J=1.0, g=0.7):
    """Transverse-field Ising: -J ZZ on every edge, -g X on every site."""
    S = spin_ops()
    H = NNHamiltonian(topo)
    for c, p in topo.edges():
        H.bonds[(c, p)] = [(-J, S["Z"], S["Z"])]
    for i in range(topo.nnodes):
        H.onsite[i] = -g * S["X"]
    return H


def heisenberg(topo, J=1.0):
    """J (XX + YY + ZZ) with Pauli matrices on every edge."""
    S = spin_ops()
    H = NNHamiltonian(topo)
    for e in topo.edges():
        H.bonds[e] = [(J, S["X"], S["X"]), (J, S["Y"], S["Y"]), (J, S["Z"], S["Z"])]
    return H


def xxz(topo, couplings, delta=0.7):
    """sum_e theta_e (XX + YY + delta ZZ); ``couplings`` maps (child, parent) -> theta_e."""
    S = spin_ops()
    H = NNHamiltonian(topo)
    for e in topo.edges():
        th = couplings[e]
        H.bonds[e] = [(th, S["X"], S["X"]), (th, S["Y"], S["Y"]), (th * delta, S["Z"], S["Z"])]
    return H


def edge_term_hamiltonian(topo, edge, terms, d=2):
    """Hamiltonian holding only the two-body terms of one edge (the derivative dH/dtheta_e
    of a Hamiltonian linear in its couplings)."""
    H = NNHamiltonian(topo, d)
    H.bonds[edge] = list(terms)
    return H


def ttno_tensors(H: NNHamiltonian):
    """Host TTNO node tensors for a nearest-neighbour tree Hamiltonian."""
    t, d = H.topo, H.d
    eye = np.eye(d, dtype=np.complex128)
    out = []
    for n in range(t.nnodes):
        kids = t.children[n]
        root = t.parent[n] < 0
        up_terms = [] if root else H.bonds.get((n, t.parent[n]), [])
        wdims = [2 + len(H.bonds.get((c, n), [])) for c in kids]
        wp = 1 if root else 2 + len(up_terms)
        W = np.zeros(wdims + [d, d, wp], dtype=np.complex128)
        done = 0 if root else 1

        def slot(states, up):
            return tuple(states) + (slice(None), slice(None), up)
        zero = [0] * len(kids)
        if not root:
            W[slot(zero, 0)] += eye
            for ti, (_, oc, _) in enumerate(up_terms):
                W[slot(zero, 2 + ti)] += oc
        if n in H.onsite:
            W[slot(zero, done)] += H.onsite[n]
        for i, c in enumerate(kids):
            st = list(zero)
            st[i] = 1
            W[slot(st, done)] += eye
            for ti, (coeff, _, op) in enumerate(H.bonds.get((c, n), [])):
                st = list(zero)
                st[i] = 2 + ti
                W[slot(st, done)] += coeff * op
        out.append(W)
    return out
