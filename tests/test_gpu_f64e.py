"""The FP64-grade tensor-core precision (GTN_PREC_FP64E): digit-plane GEMMs against numpy
at about 1e-14 relative to sum |a||b| (tails in M, N and K, rows 1e16 apart), the
benchmark's edge-class map against the oracle, and environment updates against FP64."""
import os
import sys

import numpy as np
import pytest

import grafttn as G
from grafttn import _lib
from grafttn.contractions import EffectiveMap, EnvCache
from oracle import ttn_oracle as O

pytestmark = pytest.mark.gpu


def crandn(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


@pytest.mark.parametrize("mkn", [(130, 200, 70), (257, 1000, 129), (64, 96, 300), (700, 2000, 33)])
def test_f64e_gemm_matches_numpy(ctx, mkn):
    M, K, N = mkn
    rng = np.random.default_rng(M + K)
    A, B = crandn(rng, (M, K)), crandn(rng, (K, N))
    A[5] *= 1e-8
    A[7] *= 1e8
    ref = A @ B
    got = ctx.download(ctx.contract([ctx.upload(A), ctx.upload(B)], [[-1, 1], [1, -2]], None, None,
                                    _lib.PREC_FP64E))
    scale = np.abs(A) @ np.abs(B)
    err = np.abs(got - ref) / scale
    assert err.max() < 1e-13, err.max()


def test_f64e_headline_edge_class_matches_oracle(ctx):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import bench
    xs, labels, order, statics, theta = bench.workload_arrays(bench.WORKLOAD, seed=7, bond_dim=64)
    ref = O.EffMap(labels, order, statics, xs)(theta)
    hm = EffectiveMap(ctx, xs, labels, order, [ctx.upload(s) for s in statics], "fp64e")
    kinds = {k for k, _, _ in hm.apply_profiled(ctx.upload(theta), ctx.empty(hm.y_shape))}
    assert "tc_gemm" in kinds
    y = ctx.download(hm(ctx.upload(theta)))
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-12
    hm.close()


def test_f64e_environments_match_fp64(ctx):
    topo = G.mps_topology(12)
    H = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    psi = G.random_ttns(np.random.default_rng(3), topo, 2, 64, ctx=ctx)
    c64, ce = EnvCache(topo), EnvCache(topo, precision="fp64e")
    for u in range(topo.nnodes):
        for v in topo.neighbors(u):
            a, b = ctx.download(c64.env(psi, H, u, v)), ctx.download(ce.env(psi, H, u, v))
            assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(a), (u, v)
