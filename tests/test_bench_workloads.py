"""The benchmark's workload table builds consistent maps (host check, no GPU): every eff_h2
workload, root edges included, instantiated at a small bond dimension, contracts through
the oracle to the shape of its two-site block and is Hermitian (environments Hermitian in
ket/bra, Heisenberg TTNO)."""
import numpy as np
import pytest

import bench
from oracle import ttn_oracle as O


@pytest.mark.parametrize("name", sorted(bench.WORKLOADS))
def test_workload_map_is_consistent_and_hermitian(name):
    x_shape, labels, order, statics, theta = bench.workload_arrays(name, bond_dim=4)
    assert theta.shape == x_shape and abs(np.linalg.norm(theta) - 1) < 1e-12
    h = O.EffMap(labels, order, statics, x_shape)
    rng = np.random.default_rng(80)
    a, b = O.randn_c(rng, x_shape), O.randn_c(rng, x_shape)
    ha, hb = h(a), h(b)
    assert ha.shape == x_shape
    assert abs(np.vdot(a, hb) - np.vdot(ha, b)) < 1e-10 * np.linalg.norm(a) * np.linalg.norm(b)


def test_root_edge_workload_closes_the_root():
    x_shape, labels, order, statics, _ = bench.workload_arrays("heisenberg_bin63_d1root_D256_eff_h2", bond_dim=4)
    assert x_shape[-1] == 1
    assert statics[-1].shape == (1, 1, 1)


def test_metric_labels():
    assert bench.metric_for(bench.WORKLOAD) == bench.METRIC
    other = bench.metric_for("heisenberg_bin63_d1root_D256_eff_h2")
    assert other != bench.METRIC and "d1root_D256" in other
