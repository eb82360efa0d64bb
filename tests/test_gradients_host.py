"""Host logic of the coupling gradients (no GPU): the nearest-neighbour TTNO builder puts
an edge's couplings into the parent's tensor only and affinely, which is what the adjoint
route's chain rule dE/dtheta_e = Re <G_p, dW_p/dtheta_e> relies on."""
import numpy as np

import grafttn as G
from grafttn.gradients import ttno_coupling_derivatives


def test_coupling_derivative_is_the_exact_affine_slope():
    topo = G.binary_topology(3)
    rng = np.random.default_rng(3)
    theta = {e: float(rng.uniform(0.5, 1.5)) for e in topo.edges()}
    delta = 0.7
    H = G.xxz(topo, theta, delta)
    dco = {e: [1.0, 1.0, delta] for e in topo.edges()}
    der = ttno_coupling_derivatives(H, dco)
    W0 = G.ttno_tensors(H)
    for e in list(topo.edges())[:5]:
        s = 0.37
        th2 = dict(theta)
        th2[e] += s
        W2 = G.ttno_tensors(G.xxz(topo, th2, delta))
        p, dW = der[e]
        assert p == e[1]
        for n in range(topo.nnodes):
            expect = W0[n] + (s * dW if n == p else 0.0)
            assert np.allclose(W2[n], expect, rtol=0, atol=1e-15), (e, n)
