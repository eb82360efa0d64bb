"""U(1) block-sparse eff_h2 maps on the GPU (grouped per-charge launches, CUDA graph)
against the dense oracle of the embedded tensors."""
import numpy as np
import pytest

from grafttn import blocksparse as B
from u1_cases import dense_reference, h2_u1_case

pytestmark = pytest.mark.gpu

RTOL = {"fp64": 1e-12, "fp32": 2e-5, "bf16x6": 1e-5, "bf16x3": 1e-3, "fp16x3": 1e-5}


@pytest.mark.parametrize("group", [True, False])
@pytest.mark.parametrize("prec", ["fp64", "bf16x6", "bf16x3", "fp32", "fp16x3"])
@pytest.mark.parametrize("depth,node,D", [(3, "n2_2", 16), (4, "n3_1", 64)])
def test_block_map_matches_dense(ctx, prec, depth, node, D, group):
    xs, labels, order, statics, x = h2_u1_case(depth, node, D)
    plan = B.BlockPlan(xs, labels[0], statics, order, group=group)
    ref = dense_reference(xs, labels, order, statics, x)
    bm = B.BlockEffectiveMap(ctx, plan, prec)
    y = ctx.download(bm(ctx.upload(x)))
    got = plan.y.to_dense(y)
    assert np.linalg.norm(got - ref) <= RTOL[prec] * np.linalg.norm(ref)
    bm.close()


@pytest.mark.parametrize("prec", ["fp64", "bf16x6", "fp16x3"])
def test_block_map_d128_skinny_and_tc(ctx, prec):
    """Depth-5 binary tree at D = 128: coupled-charge problems of every kind (tcgen05,
    skinny N < 16, narrow K < 16 block moves) in one map."""
    xs, labels, order, statics, x = h2_u1_case(5, "n3_1", 128)
    plan = B.BlockPlan(xs, labels[0], statics, order)
    ref = dense_reference(xs, labels, order, statics, x)
    bm = B.BlockEffectiveMap(ctx, plan, prec)
    got = plan.y.to_dense(ctx.download(bm(ctx.upload(x))))
    assert np.linalg.norm(got - ref) <= RTOL[prec] * np.linalg.norm(ref)
    bm.close()


def test_block_map_graph_replay(ctx):
    xs, labels, order, statics, x = h2_u1_case(4, "n3_1", 64, seed=12)
    plan = B.BlockPlan(xs, labels[0], statics, order)
    ref = plan.y.from_dense(dense_reference(xs, labels, order, statics, x), check_zero=False)
    bm = B.BlockEffectiveMap(ctx, plan, "bf16x6", graph=True)
    dx = ctx.upload(x)
    dy = ctx.empty((plan.y.size,))
    for _ in range(3):  # eager + capture, then replays
        bm.apply_into(dx, dy)
        ctx.sync()
        assert np.linalg.norm(ctx.download(dy) - ref) <= 1e-5 * np.linalg.norm(ref)
    bm.close()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-14), ("bf16x6", 1e-6), ("fp16x3", 1e-6)])
def test_block_map_bands_match_staged_products(ctx, prec, tol, monkeypatch):
    """The few-column problems read straight from the running tensor (fused row bands) give
    the products of the staged-operand path (GTN_BLOCK_BANDS=0) and the dense oracle."""
    xs, labels, order, statics, x = h2_u1_case(5, "n3_1", 128, seed=5)
    plan = B.BlockPlan(xs, labels[0], statics, order)
    ref = dense_reference(xs, labels, order, statics, x)
    outs, launches = [], []
    for flag in ("1", "0"):
        monkeypatch.setenv("GTN_BLOCK_BANDS", flag)
        bm = B.BlockEffectiveMap(ctx, plan, prec)
        l0 = ctx.launches
        outs.append(ctx.download(bm(ctx.upload(x))))
        launches.append(ctx.launches - l0)
        bm.close()
    assert np.linalg.norm(outs[0] - outs[1]) <= tol * np.linalg.norm(outs[1])
    got = plan.y.to_dense(outs[0])
    assert np.linalg.norm(got - ref) <= RTOL[prec] * np.linalg.norm(ref)
    assert launches[0] <= launches[1]
