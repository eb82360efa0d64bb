"""Tile shapes of the tcgen05 steps: every kernel variant (one-SM tiles 128 x 32 ... 128 x 256,
two CTAs per SM, 256 x 256 tiles on an SM pair with cta_group::2 MMAs, and the persistent
kernel with double-buffered accumulators) against numpy, on shapes with M and 2N tails; and
the measured choice: tuned once per problem class, cached, reused by later launches of the
class, with the same results."""
import numpy as np
import pytest

from grafttn import _lib

pytestmark = pytest.mark.gpu

RTOL = {"bf16x6": 2e-5, "fp16x3": 2e-5, "bf16x3": 2e-3}


def crandn(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def contract(ctx, A, B, prec):
    return ctx.download(ctx.contract([ctx.upload(A), ctx.upload(B)], [[-1, 1], [1, -2]], None, None,
                                     _lib.PRECISIONS[prec]))


@pytest.fixture
def restore_tuning():
    old = _lib.tc_tuning(None)
    yield
    _lib.tc_tuning(old, clear=True)


# (M, K, N): 2N > 128 with long K (the SM-pair candidates); M = 257 leaves one valid row in
# the second pair, 2N = 600 leaves 88 valid B' rows in the last tile and none in its odd CTA
@pytest.mark.parametrize("mkn", [(700, 2000, 300), (257, 1000, 129), (1024, 1536, 512)])
@pytest.mark.parametrize("prec", ["fp16x3", "bf16x6", "bf16x3"])
def test_tc_variants_match_numpy(ctx, restore_tuning, mkn, prec):
    M, K, N = mkn
    rng = np.random.default_rng(M + K + N)
    A, B = crandn(rng, (M, K)), crandn(rng, (K, N))
    ref = A @ B
    outs = {}
    for v in ("ps256", "pair256", "ps128x2", "persist128", "persist256"):
        _lib.tc_tuning(v)
        outs[v] = contract(ctx, A, B, prec)
        assert rel(outs[v], ref) < RTOL[prec], (v, rel(outs[v], ref))
    # the variants sum the same products per output element: they agree far below the map error
    for v in ("pair256", "ps128x2", "persist128", "persist256"):
        assert rel(outs[v], outs["ps256"]) < 1e-6, v
    ctx.sync()


def test_measured_choice_is_cached_and_reused(ctx, restore_tuning):
    rng = np.random.default_rng(9)
    M, K, N = 2048, 2048, 384
    A, B = crandn(rng, (M, K)), crandn(rng, (K, N))
    _lib.tc_tuning("measured", clear=True)
    y1 = contract(ctx, A, B, "fp16x3")
    rep1 = _lib.tc_tune_report()
    assert len(rep1) >= 1 and all("chosen=" in l for l in rep1), rep1
    # the same problem class again (other values): no new measurement, the same choice
    A2 = crandn(rng, (M, K))
    y2 = contract(ctx, A2, B, "fp16x3")
    assert _lib.tc_tune_report() == rep1
    y1b = contract(ctx, A, B, "fp16x3")
    assert np.array_equal(y1, y1b)  # the cached variant reproduces the tuned launch bitwise
    assert rel(y1, A @ B) < RTOL["fp16x3"] and rel(y2, A2 @ B) < RTOL["fp16x3"]
    # the chosen variant's result equals that variant forced
    chosen = rep1[0].split("chosen=")[1].split()[0]
    _lib.tc_tuning(chosen)
    assert np.array_equal(contract(ctx, A, B, "fp16x3"), y1)
