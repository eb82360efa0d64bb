"""The headline workload's edge class against the oracle, through the C ABI.

The benchmark times eff_h2 on the depth-3 -> depth-2 edge of the 63-site binary tree
(Θ legs [8, 8, 2, D', 2, D], Heisenberg TTNO w = 5, Hermitian environments).  These tests
build the same map at bond 64 (Θ = [8, 8, 2, 64, 2, 64], a size the numpy oracle applies in
about a second) and compare every precision with the oracle's env-first ncon
(test/contraction_planning.jl:111-160: planned == unplanned), once through device buffers
and once through gtn_map_apply_host, the call the Julia binding makes per matvec."""
import os
import sys

import numpy as np
import pytest

import grafttn as G
from grafttn.contractions import EffectiveMap
from oracle import ttn_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

pytestmark = pytest.mark.gpu

HEADLINE = "heisenberg_bin63_d3d2_D1024_eff_h2"


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def headline_small():
    import bench
    x_shape, labels, order, statics, theta = bench.workload_arrays(HEADLINE, seed=7, bond_dim=64)
    ref = O.EffMap(labels, order, statics, x_shape)(theta)
    return x_shape, labels, order, statics, theta, ref


# fp64: parity mode.  Mixed modes: the map error of the split products with FP32
# accumulation (1.6-1.7e-5 at D = 1024, K up to 10240; less at this K).
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp16x3", 2e-5), ("bf16x6", 2e-5),
                                           ("bf16x3", 2e-3), ("fp32", 2e-5)])
def test_headline_edge_class_matches_oracle(ctx, headline_small, precision, tol):
    x_shape, labels, order, statics, theta, ref = headline_small
    assert tuple(x_shape) == (8, 8, 2, 64, 2, 64)
    hm = EffectiveMap(ctx, x_shape, labels, order, [ctx.upload(s) for s in statics], precision)
    y = ctx.download(hm(ctx.upload(theta)))
    assert rel(y, ref) < tol, (precision, rel(y, ref))
    # the chain's algorithmic flop count is the oracle's env-first count
    assert abs(hm.flops - 8 * O.plan_macs([x_shape] + [s.shape for s in statics], labels, order)) <= 1e-9 * hm.flops
    hm.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp16x3", 2e-5)])
def test_map_apply_host_matches_device_and_oracle(ctx, headline_small, precision, tol):
    x_shape, labels, order, statics, theta, ref = headline_small
    hm = EffectiveMap(ctx, x_shape, labels, order, [ctx.upload(s) for s in statics], precision)
    y_dev = ctx.download(hm(ctx.upload(theta)))
    for _ in range(2):  # the first call allocates the staging buffers, the second reuses them
        y_host = hm.apply_host(theta)
        assert y_host.shape == tuple(hm.y_shape)
        assert rel(y_host, ref) < tol
        assert np.array_equal(y_host, y_dev)  # same kernels, same inputs: bitwise equal
    hm.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp16x3", 2e-5)])
def test_map_apply_host_page_locked(ctx, headline_small, precision, tol):
    # page-locked host buffers (the binding's fast path): the result equals the device
    # apply bit for bit, twice in a row
    import ctypes as C
    import torch
    x_shape, labels, order, statics, theta, ref = headline_small
    hm = EffectiveMap(ctx, x_shape, labels, order, [ctx.upload(s) for s in statics], precision)
    y_dev = ctx.download(hm(ctx.upload(theta)))
    xh = torch.from_numpy(theta.copy()).pin_memory()
    yh = torch.empty(tuple(hm.y_shape), dtype=torch.complex128).pin_memory()
    for _ in range(2):
        yh.zero_()
        assert ctx.lib.gtn_map_apply_host(hm.h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr())) == 0
        y = yh.numpy()
        assert rel(y, ref) < tol
        assert np.array_equal(y, y_dev)
    hm.close()


def test_map_apply_host_rejects_null_buffers(ctx, headline_small):
    from grafttn import _lib
    x_shape, labels, order, statics, theta, _ = headline_small
    hm = EffectiveMap(ctx, x_shape, labels, order, [ctx.upload(s) for s in statics], "fp64")
    assert ctx.lib.gtn_map_apply_host(hm.h, None, None) == _lib.GTN_ERR_INVALID
    hm.close()
