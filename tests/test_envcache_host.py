"""Host bookkeeping of the device environment cache (no GPU): the reference's invalidation
rule (envcache.jl:812-844) drops exactly the environments whose contracted side contains a
touched node, checked against a side computed independently by a walk over the tree, on
several topologies; the byte accounting follows the drops."""
import pytest
import torch

import grafttn as G
from grafttn.contractions import EnvCache


def side(topo, u, v):
    """Nodes on u's side of the edge u - v."""
    seen, stack = {u}, [u]
    while stack:
        x = stack.pop()
        for w in topo.neighbors(x):
            if (x, w) == (u, v) or w in seen:
                continue
            seen.add(w)
            stack.append(w)
    return seen


def filled_cache(topo):
    cache = EnvCache(topo)
    for u in range(topo.nnodes):
        for v in topo.neighbors(u):
            E = torch.zeros(3 + u, dtype=torch.complex128)
            cache.envs[(u, v)] = E
            cache.bytes += E.numel() * E.element_size()
    return cache


TOPOLOGIES = {"bin3": lambda: G.binary_topology(3), "star32": lambda: G.star_topology(3, 2),
              "fork22": lambda: G.fork_topology(2, 2), "kary32": lambda: G.kary_topology(3, 2),
              "mps5": lambda: G.mps_topology(5)}


@pytest.mark.parametrize("which", sorted(TOPOLOGIES))
def test_invalidate_node_drops_exactly_the_envs_that_saw_it(which):
    topo = TOPOLOGIES[which]()
    for n in range(topo.nnodes):
        cache = filled_cache(topo)
        keys = set(cache.envs)
        cache.invalidate_node(n)
        kept = {k for k in keys if n not in side(topo, *k)}
        assert set(cache.envs) == kept, (which, n)
        assert cache.bytes == sum(E.numel() * E.element_size() for E in cache.envs.values())
        # the env pointing into n from every neighbour survives: its side excludes n
        for w in topo.neighbors(n):
            assert (w, n) in cache.envs


@pytest.mark.parametrize("which", sorted(TOPOLOGIES))
def test_invalidate_edge_is_both_endpoints(which):
    topo = TOPOLOGIES[which]()
    for n in range(topo.nnodes):
        m = topo.parent[n]
        if m < 0:
            continue
        cache = filled_cache(topo)
        cache.invalidate_edge(n, m)
        kept = {k for k in filled_cache(topo).envs if n not in side(topo, *k) and m not in side(topo, *k)}
        assert set(cache.envs) == kept
        # the two envs across the edge are rebuilt; those pointing into n or m from their
        # other neighbours stay valid
        assert (n, m) not in cache.envs and (m, n) not in cache.envs
        for a, b in ((n, m), (m, n)):
            for w in topo.neighbors(a):
                if w != b:
                    assert (w, a) in cache.envs


@pytest.mark.parametrize("topo", [G.mps_topology(7), G.binary_topology(3), G.kary_topology(3, 2),
                                  G.star_topology(3, 2)])
def test_subtree_sets_match_a_tree_walk(topo):
    """The remembered subtree of (u, away from v) is u's side of the edge, on every call."""
    for _ in range(2):  # the second pass reads the remembered answers
        for u in range(topo.nnodes):
            for v in topo.neighbors(u):
                ref = side(topo, u, v)
                got = topo.subtree_nodes(u, v)
                assert got[0] == u and set(got) == ref and len(got) == len(ref)
                for x in range(topo.nnodes):
                    assert topo.in_subtree(x, u, v) == (x in ref)
