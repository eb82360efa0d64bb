"""The one-pass split (row maxima shared through cluster shared memory, then the slice
planes) against the two-kernel path it replaces (row maxima, then the split): the planes,
and so the map outputs, are bit-identical.  Covers table-driven maps and one-shot
contractions, fp16x3 and the FP64-grade digit planes, views whose unit-stride index is a
row or a column, clusters of two to sixteen CTAs, row and column tails, and rows too long
for the clusters (the two-kernel path runs)."""
import os
import sys

import numpy as np
import pytest

from grafttn import _lib
from grafttn.contractions import EffectiveMap
from oracle import ttn_oracle as O

pytestmark = pytest.mark.gpu


def crandn(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def with_fused(flag, fn):
    old = os.environ.get("GTN_FUSED_SPLIT")
    os.environ["GTN_FUSED_SPLIT"] = "1" if flag else "0"
    try:
        return fn()
    finally:
        if old is None:
            del os.environ["GTN_FUSED_SPLIT"]
        else:
            os.environ["GTN_FUSED_SPLIT"] = old


@pytest.mark.parametrize("prec,tol", [("fp16x3", 3e-5), ("fp64e", 1e-12)])
def test_fused_split_map_bit_identical(ctx, prec, tol):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import bench
    xs, labels, order, statics, theta = bench.workload_arrays(bench.WORKLOAD, seed=5, bond_dim=48)
    ref = O.EffMap(labels, order, statics, xs)(theta)
    hm = EffectiveMap(ctx, xs, labels, order, [ctx.upload(s) for s in statics], prec)
    x = ctx.upload(theta)
    y1 = with_fused(True, lambda: ctx.download(hm(x)))
    n1 = ctx.launches
    y0 = with_fused(False, lambda: ctx.download(hm(x)))
    n0 = ctx.launches - n1
    n1b = ctx.launches
    with_fused(True, lambda: ctx.download(hm(x)))
    assert ctx.launches - n1b < n0  # one launch per split instead of two
    assert np.array_equal(y0, y1)
    assert np.linalg.norm(y1 - ref) / np.linalg.norm(ref) < tol
    hm.close()


@pytest.mark.parametrize("prec", ["fp16x3", "fp64e"])
@pytest.mark.parametrize("M,K,N,k_major", [
    (1000, 200, 70, True),     # a small cluster per row block, rows contiguous along k
    (1000, 200, 70, False),    # the unit-stride index is the row
    (517, 3000, 40, True),     # a wide cluster, tails in M and K
    (517, 3000, 40, False),
    (300, 7001, 33, True),     # the widest clusters
    (300, 7001, 33, False),    # longer than the clusters hold with 16-row blocks: two kernels
    (64, 20000, 24, True),     # longer than sixteen CTAs hold: the two-kernel path
])
def test_fused_split_contract_bit_identical(ctx, prec, M, K, N, k_major):
    rng = np.random.default_rng(M + K)
    A = crandn(rng, (M, K))
    A[3] *= 1e-6
    A[5] *= 1e6
    B = crandn(rng, (K, N))
    code = _lib.PRECISIONS[prec]
    if k_major:
        a, lab = ctx.upload(A), [[-1, 1], [1, -2]]
    else:
        a, lab = ctx.upload(np.ascontiguousarray(A.T)), [[1, -1], [1, -2]]
    b = ctx.upload(B)
    y1 = with_fused(True, lambda: ctx.download(ctx.contract([a, b], lab, None, None, code)))
    y0 = with_fused(False, lambda: ctx.download(ctx.contract([a, b], lab, None, None, code)))
    assert np.array_equal(y0, y1)
    ref = A @ B
    scale = np.abs(A) @ np.abs(B)
    bound = 1e-13 if prec == "fp64e" else 1e-4
    assert (np.abs(y1 - ref) / scale).max() < bound
