"""Host logic of the U(1) networks (no GPU): bond sectors and the truncation rule applied to
all sectors' singular values together (the rule of the dense split, Backend.jl:466-483)."""
import math

import numpy as np

import grafttn as G
from grafttn import u1 as U


def test_bond_sectors_exact_and_capped():
    topo = G.mps_topology(8)
    sec = U.bond_sectors(topo, 4, 10 ** 6)
    for c, s in sec.items():
        ns = len(topo.subtree_nodes(c, topo.parent[c]))
        for q, d in s.items():
            assert d == min(math.comb(ns, q), math.comb(8 - ns, 4 - q))
    capped = U.bond_sectors(topo, 4, 8)
    for c, s in capped.items():
        assert sum(s.values()) <= 8 and all(d >= 1 for d in s.values())
        assert set(s) <= set(sec[c])


def test_trunc_rank_rule():
    s = np.array([3.0, 2.0, 1.0, 0.5, 1e-3, 1e-9])
    assert U.trunc_rank(s, None, 0, 0, 0) == 6
    assert U.trunc_rank(s, 3, 0, 0, 0) == 3
    assert U.trunc_rank(s, None, 0.7, 0, 0) == 3
    assert U.trunc_rank(s, None, 0, 1e-4, 0) == 5
    # relative discarded weight: the tail {1e-3, 1e-9} has norm ~1e-3 <= 1e-3 * |s|
    assert U.trunc_rank(s, None, 0, 0, 1e-3) == 4
    assert U.trunc_rank(np.array([1e-20]), None, 1.0, 0, 0) == 1
