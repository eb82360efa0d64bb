"""Gradient of <psi|H(theta)|psi> (XXZ, Delta = 0.7, per-edge couplings) with respect to the
site tensors and the couplings, checked against central finite differences (h = 1e-6) and
the a16 identities; the reference has no AD, so parity with a reference gradient is
unpinned and these checks are the gate."""
import numpy as np
import pytest

import grafttn as G
from grafttn import gradients as GR

pytestmark = pytest.mark.gpu

DELTA = 0.7


def edge_terms(topo, delta=DELTA):
    S = G.spin_ops()
    return {e: [(1.0, S["X"], S["X"]), (1.0, S["Y"], S["Y"]), (delta, S["Z"], S["Z"])] for e in topo.edges()}


def make(topo, theta, ctx):
    return G.TTNO.from_hamiltonian(G.xxz(topo, theta, DELTA), ctx)


@pytest.mark.parametrize("depth,bond", [(3, 6), (4, 16)])
def test_gradients_vs_finite_differences(ctx, depth, bond):
    topo = G.binary_topology(depth)
    rng = np.random.default_rng(21)
    theta = {e: float(rng.uniform(0.5, 1.5)) for e in topo.edges()}
    H = make(topo, theta, ctx)
    psi = G.random_ttns(rng, topo, 2, bond, ctx=ctx)
    E0 = GR.energy(psi, H).real
    # couplings: dE/dtheta_e = <psi|h_e|psi> vs central differences of E
    g_theta = GR.coupling_gradients(psi, edge_terms(topo))
    h = 1e-6
    for e in list(topo.edges())[:5]:
        tp, tm = dict(theta), dict(theta)
        tp[e] += h
        tm[e] -= h
        fd = (GR.energy(psi, make(topo, tp, ctx)).real - GR.energy(psi, make(topo, tm, ctx)).real) / (2 * h)
        assert abs(fd - g_theta[e]) <= 1e-6 * max(1.0, abs(g_theta[e])), (e, fd, g_theta[e])
    # E is linear in theta: sum_e theta_e dE/dtheta_e = E
    assert abs(sum(theta[e] * g_theta[e] for e in theta) - E0) < 1e-10 * max(1.0, abs(E0))
    # site tensors: directional derivative 2 Re <D, g_n> vs central differences
    grads = GR.site_gradients(psi, H, max_env_bytes=1 << 20)
    for n in [0, 1, topo.nnodes - 1]:
        A = psi.tensors[n]
        D = ctx.upload((rng.standard_normal(tuple(A.shape)) + 1j * rng.standard_normal(tuple(A.shape))) / 2)
        pp, pm = psi.copy(), psi.copy()
        pp.tensors[n] = ctx.axpby(h, D, 1.0, A.clone())
        pm.tensors[n] = ctx.axpby(-h, D, 1.0, A.clone())
        fd = (GR.energy(pp, H).real - GR.energy(pm, H).real) / (2 * h)
        an = 2 * ctx.dot(D, grads[n]).real
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (n, fd, an)
    # <A_n, g_n> = E at every node (the quadratic form), independent of gauge
    for n in range(topo.nnodes):
        assert abs(ctx.dot(psi.tensors[n], grads[n]) - E0) < 1e-10 * max(1.0, abs(E0))
