"""U(1) block-sparse planner on the host: the block-map descriptors, executed by a numpy
interpreter, reproduce the dense contraction of the embedded tensors (no GPU needed)."""
import numpy as np
import pytest

from grafttn import blocksparse as B
from u1_cases import dense_reference, h2_u1_case


def test_ttno_blocks_are_charge_conserving():
    xs, labels, order, statics, x = h2_u1_case(2, "n2_1", 8)
    for T, lab, d in statics[:2]:
        dense = T.to_dense(d)
        assert np.allclose(T.from_dense(dense), d)


@pytest.mark.parametrize("group", [False, True])
@pytest.mark.parametrize("depth,node,D", [(2, "n2_1", 8), (3, "n2_2", 16), (3, "n3_1", 12)])
def test_block_plan_matches_dense(depth, node, D, group):
    xs, labels, order, statics, x = h2_u1_case(depth, node, D)
    plan = B.BlockPlan(xs, labels[0], statics, order, group=group)
    y = B.execute_numpy(plan, x)
    ref = dense_reference(xs, labels, order, statics, x)
    got = plan.y.to_dense(y)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)
    # the output has the input's block structure (the map conserves charge)
    assert [b[0] for b in plan.y.blocks] == [b[0] for b in xs.blocks]
    assert plan.flops > 0 and len(plan.steps) == len(plan.groups)
    # the groups partition the absorbed operands in chain order
    assert [j for g in plan.groups for j in g] == list(order[1:])
    if not group:
        assert len(plan.steps) == len(order) - 1


def test_contract_statics_matches_dense():
    xs, labels, order, statics, x = h2_u1_case(3, "n2_2", 16)
    a, b = statics[2], statics[0]   # an environment and the TTNO site tensor it touches
    c = B.contract_statics(a, b)
    shared = [l for l in a[1] if l > 0 and l in b[1]]
    assert shared
    ia = [a[1].index(l) for l in shared]
    ib = [b[1].index(l) for l in shared]
    ref = np.tensordot(a[0].to_dense(a[2]), b[0].to_dense(b[2]), axes=(ia, ib))
    assert np.allclose(c[0].to_dense(c[2]), ref, atol=1e-13)
    assert c[1] == [l for l in a[1] if l not in shared] + [l for l in b[1] if l not in shared]


def test_u1_oracle_matches_dense_and_planner():
    from oracle import u1_oracle as U
    xs, labels, order, statics, x = h2_u1_case(3, "n2_2", 16)
    blocks = [U.blocks_from_flat(xs, x)] + [U.blocks_from_flat(T, d) for T, _, d in statics]
    plan = B.BlockPlan(xs, labels[0], statics, order)
    y_or = U.flat_from_blocks(plan.y, U.ncon_blocks(blocks, labels, order))
    ref = dense_reference(xs, labels, order, statics, x)
    assert np.linalg.norm(plan.y.to_dense(y_or) - ref) <= 1e-12 * np.linalg.norm(ref)
    assert np.linalg.norm(B.execute_numpy(plan, x) - y_or) <= 1e-12 * np.linalg.norm(y_or)
