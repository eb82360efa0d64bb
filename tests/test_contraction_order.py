"""Host logic of the contraction-order choice (grafttn/contractions.py; no GPU): the cost
of a chain, the dynamic programme's optimality over left-deep chains, and the rule that
keeps the reference's env-first order unless another chain is clearly cheaper."""
import itertools

import pytest

import grafttn as G
from grafttn import contractions as GC


def h1_network(topo, n, D, w, d=2):
    """Shapes and labels of the one-site map of node n with every bond D and TTNO bond w,
    in the reference's operand order (x, W, envs..., cap?)."""
    K = topo.nchildren(n)
    x_rank, w_rank = K + 2, K + 3
    labels, order, envs = GC.h1_spec(topo, n, x_rank, w_rank)
    xs = [D] * K + [d] + [D if topo.parent[n] >= 0 else 1]
    ws = [w] * K + [d, d] + [w if topo.parent[n] >= 0 else 1]
    shapes = [tuple(xs), tuple(ws)]
    for lab in labels[2:]:
        dims = []
        for l in lab:
            if l < 0:
                dims.append(xs[-l - 1])
            else:
                pos = [i for i, q in enumerate(labels[0]) if q == l]
                dims.append(xs[pos[0]] if pos else ws[labels[1].index(l)])
        shapes.append(tuple(dims))
    return shapes, labels, order


def test_chain_cost_of_a_matrix_chain():
    # A (2x3) B (3x4) C (4x5): 2*3*4 + 2*4*5 complex MACs, largest intermediate 2*5
    labels = [[-1, 1], [1, 2], [2, -2]]
    shapes = [(2, 3), (3, 4), (4, 5)]
    assert GC.chain_cost(shapes, labels, [0, 1, 2]) == (2 * 3 * 4 + 2 * 4 * 5, 10)
    # absorbing C first is an outer product: 2*3*4*5 then a contraction over 3*4
    assert GC.chain_cost(shapes, labels, [0, 2, 1])[0] == 2 * 3 * 4 * 5 + 2 * 5 * 3 * 4


@pytest.mark.parametrize("case", ["kary_root", "kary_mid", "bin_mid", "star_centre", "mps_mid"])
def test_best_order_is_the_cheapest_left_deep_chain(case):
    topo, n, D, w = {
        "kary_root": (G.kary_topology(4, 2), 0, 5, 3),
        "kary_mid": (G.kary_topology(4, 2), 1, 6, 5),
        "bin_mid": (G.binary_topology(3), 1, 8, 5),
        "star_centre": (G.star_topology(4, 1), 0, 4, 3),
        "mps_mid": (G.mps_topology(6), 2, 16, 5),
    }[case]
    shapes, labels, order = h1_network(topo, n, D, w)
    best = GC.best_order(shapes, labels, 0)
    assert sorted(best) == list(range(len(labels))) and best[0] == 0
    brute = min(GC._objective(shapes, labels, [0] + list(p))
                for p in itertools.permutations(range(1, len(labels))))
    assert GC._objective(shapes, labels, best) == brute
    assert GC._objective(shapes, labels, best) <= GC._objective(shapes, labels, order)


def test_choose_order_keeps_env_first_unless_clearly_cheaper():
    # a chain node (degree 2): env-first is already optimal and is kept
    shapes, labels, order = h1_network(G.mps_topology(6), 2, 64, 5)
    assert GC.choose_order(shapes, labels, order) == order
    # the root of a 4-ary tree at a wide TTNO bond: absorbing every environment before W
    # grows the running tensor by w per leg, and a cheaper chain replaces it
    # (here W moves ahead of the last two environments, 6.2x cheaper)
    shapes, labels, order = h1_network(G.kary_topology(4, 2), 0, 8, 5)
    chosen = GC.choose_order(shapes, labels, order)
    assert chosen != order
    assert chosen.index(1) < order.index(1)
    assert 3 * GC._objective(shapes, labels, chosen) < 2 * GC._objective(shapes, labels, order)
    # more than 13 operands: the given order, without a search
    many = [[-1, 1]] + [[i, i + 1] for i in range(1, 14)] + [[14, -2]]
    shp = [(2, 2)] * len(many)
    assert GC.choose_order(shp, many, list(range(len(many)))) == list(range(len(many)))


def test_best_order_keeps_the_open_legs():
    # the chosen chain ends with exactly the network's open legs
    shapes, labels, order = h1_network(G.kary_topology(3, 2), 1, 3, 3)
    best = GC.best_order(shapes, labels, 0)
    cur = list(labels[best[0]])
    for j in best[1:]:
        L = labels[j]
        sh = [l for l in cur if l > 0 and l in L]
        cur = [l for l in L if l not in sh] + [l for l in cur if l not in sh]
    assert sorted(cur) == sorted(l for lab in labels for l in lab if l < 0)


def test_choose_order_is_remembered_per_network():
    """A repeated question gets the same answer, and callers get their own copy."""
    shapes, labels, order = h1_network(G.kary_topology(4, 2), 0, 8, 5)
    first = GC.choose_order(shapes, labels, order)
    first.append(99)  # a caller's edit must not leak into the remembered answer
    again = GC.choose_order([tuple(s) for s in shapes], [list(l) for l in labels], list(order))
    assert again == first[:-1]
    assert again == GC.best_order(shapes, labels, order[0])
