"""Device-resident scalar contractions and TTNO application against dense vectors:
inner / local expect (lib/GraftContractions/src/Contractions/expectation.jl:13-80) and the
exact TTNO-TTNS product (lib/GraftNetworks/src/Networks/apply.jl)."""
import numpy as np
import pytest

import grafttn as G
from grafttn import observables as OB
from oracle import ttn_oracle as O

pytestmark = pytest.mark.gpu


def dense(psi):
    ot = O.TreeTopology(psi.topo.ids[0], [(psi.topo.ids[psi.topo.parent[i]], psi.topo.ids[i])
                                          for i in range(1, psi.topo.nnodes)])
    return O.to_dense(O.TTNS(ot, psi.host_tensors(), psi.center))


def test_inner_matches_dense(ctx):
    topo = G.binary_topology(3)
    phi = G.random_ttns(np.random.default_rng(31), topo, 2, 4, ctx=ctx)
    psi = G.random_ttns(np.random.default_rng(32), topo, 2, 4, ctx=ctx)
    ref = np.vdot(dense(phi), dense(psi))
    got = OB.inner(phi, psi)
    assert abs(got - ref) < 1e-12 * max(1.0, abs(ref))
    assert abs(OB.inner(psi, psi) - 1.0) < 1e-12


def test_expect_local_matches_dense(ctx):
    topo = G.star_topology(3, 2)
    psi = G.random_ttns(np.random.default_rng(33), topo, 2, 4, ctx=ctx)
    v = dense(psi)
    Z = G.spin_ops()["Z"]
    n = topo.nnodes
    for site in range(n):
        ops = [np.eye(2)] * n
        # dense order follows the oracle's node order (site 0 slowest)
        ops = list(ops)
        ops[site] = Z
        full = ops[0]
        for o in ops[1:]:
            full = np.kron(full, o)
        ref = np.vdot(v, full @ v) / np.vdot(v, v)
        assert abs(OB.expect_local(psi, Z, site) - ref) < 1e-12
    assert psi.center == topo.root or psi.center in range(n)


def test_apply_ttno_matches_dense(ctx):
    topo = G.star_topology(3, 2)
    H = G.tfi(topo, g=0.9)
    W = G.TTNO.from_hamiltonian(H, ctx)
    Hd = O.dense_hamiltonian(O.tfi(O.star_topology(3, 2), g=0.9))
    psi = G.random_ttns(np.random.default_rng(34), topo, 2, 3, ctx=ctx)
    Hpsi = OB.apply_ttno(W, psi)
    assert np.linalg.norm(dense(Hpsi) - Hd @ dense(psi)) < 1e-12 * np.linalg.norm(Hd @ dense(psi))
    # <psi|H psi> through inner equals the sandwich closed at the centre
    e1 = OB.inner(psi, Hpsi)
    e2 = G.expect(psi, W)
    assert abs(e1 - e2) < 1e-12 * max(1.0, abs(e2))
