"""Batched independent eff_h1 maps with uneven bond dimensions: grouped launches (one per
step and kernel kind) and the CUDA-graph replay match the single-map applications and the
oracle."""
import numpy as np
import pytest

from grafttn.contractions import EffectiveMap, MapBatch, apply_batched
from oracle import ttn_oracle as O

pytestmark = pytest.mark.gpu

RTOL = {"fp64": 1e-12, "fp32": 2e-5, "bf16x6": 1e-5, "bf16x3": 1e-3, "fp16x3": 1e-5}


def h1_instance(rng, dims, w=5, d=2):
    """A one-site map of a node with children dims[:-1] and parent dims[-1] (XXZ-like random
    TTNO tensor, Hermitian random environments), as the reference's eff_h1 label graph."""
    K = len(dims) - 1
    t = O.mps_topology(3) if K == 1 else O.binary_topology(2)
    n = 1                                   # a node with K children and a parent
    x_shape = tuple(dims[:-1]) + (d, dims[-1])
    W = O.randn_c(rng, (w,) * K + (d, d, w))
    envs = []
    for D in dims:
        e = O.randn_c(rng, (D, w, D)) / np.sqrt(D)
        envs.append((e + e.conj().transpose(2, 1, 0)) / 2)
    labels, order = O.h1_spec(t, n, len(x_shape), W.ndim)
    return x_shape, labels, order, [W] + envs


def make_batch(ctx, rng, count, dmin, dmax, prec):
    maps, xs, refs = [], [], []
    for i in range(count):
        if i % 2 == 0:
            dims = [int(rng.integers(dmin, dmax + 1)), int(rng.integers(dmin, dmax + 1))]
        else:
            cap = min(dmax, 48)
            dims = [int(rng.integers(dmin, cap + 1)) for _ in range(3)]
        x_shape, labels, order, statics = h1_instance(rng, dims)
        x = O.randn_c(rng, x_shape)
        refs.append(O.EffMap(labels, order, statics, x_shape)(x))
        maps.append(EffectiveMap(ctx, x_shape, labels, order, [ctx.upload(s) for s in statics], prec))
        xs.append(ctx.upload(x))
    return maps, xs, refs


@pytest.mark.parametrize("prec", ["fp64", "bf16x6", "bf16x3", "fp32", "fp16x3"])
def test_batched_h1_matches_single_and_oracle(ctx, prec):
    rng = np.random.default_rng(31)
    maps, xs, refs = make_batch(ctx, rng, 12, 4, 96, prec)
    ys = apply_batched(maps, xs)
    for m, x, y, ref in zip(maps, xs, ys, refs):
        yb = ctx.download(y)
        ys1 = ctx.download(m(x))
        assert np.linalg.norm(yb - ref) / np.linalg.norm(ref) < RTOL[prec]
        # grouped launches compute each map exactly like its single application
        assert np.linalg.norm(yb - ys1) <= 1e-6 * np.linalg.norm(ys1) if prec != "fp64" else np.allclose(yb, ys1, rtol=0, atol=1e-12 * np.abs(ys1).max())
    for m in maps:
        m.close()


@pytest.mark.parametrize("prec", ["bf16x6", "fp16x3"])
def test_batch_graph_replay_64_instances(ctx, prec):
    rng = np.random.default_rng(32)
    maps, xs, refs = make_batch(ctx, rng, 64, 16, 256, prec)
    ys = [ctx.empty(m.y_shape) for m in maps]
    b = MapBatch(maps, xs, ys, graph=True)
    for _ in range(3):             # eager, capture + launch, replay
        b.run()
        ctx.sync()
        for y, ref in zip(ys, refs):
            assert np.linalg.norm(ctx.download(y) - ref) / np.linalg.norm(ref) < RTOL[prec]
    b.close()
    for m in maps:
        m.close()
