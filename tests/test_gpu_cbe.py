"""TDVP1_CBE (PredictorCBE) on the GPU against exact propagation, the reference's gates
(test/runtests.jl:933-958): growth from bond dimension 1 with fidelity <= 1e-6, and the
disabled expansion reproducing TDVP1 exactly."""
import numpy as np
import pytest

import grafttn as G
from grafttn.cbe import TDVP1_CBE, PredictorCBE
from oracle import ttn_oracle as O

pytestmark = pytest.mark.gpu


def dense(psi):
    ot = O.TreeTopology(psi.topo.ids[0], [(psi.topo.ids[psi.topo.parent[i]], psi.topo.ids[i])
                                          for i in range(1, psi.topo.nnodes)])
    return O.to_dense(O.TTNS(ot, psi.host_tensors(), psi.center))


def setup(ctx, seed=5):
    topo = G.star_topology(3, 2)
    W = G.TTNO.from_hamiltonian(G.tfi(topo, g=0.9), ctx)
    Hd = O.dense_hamiltonian(O.tfi(O.star_topology(3, 2), g=0.9))
    psi = G.random_ttns(np.random.default_rng(seed), topo, 2, 1, ctx=ctx)
    return topo, W, Hd, psi


def test_cbe_grows_bonds_and_tracks_exact(ctx):
    topo, W, Hd, psi = setup(ctx)
    dt = 0.02
    vex = O.exact_evolve(Hd, dense(psi), -1j * dt * 10)
    ev = TDVP1_CBE(PredictorCBE(max_add=8, spawn_threshold=1e-10), maxdim=16)
    for _ in range(10):
        ev.step(psi, W, -1j * dt)
    assert max(psi.bond_dims()) > 1
    assert abs(1 - abs(np.vdot(dense(psi), vex))) < 1e-6


def test_cbe_disabled_is_tdvp1(ctx):
    topo, W, Hd, psi = setup(ctx, seed=6)
    a, b = psi.copy(), psi.copy()
    eva = G.TDVP1(order=2)
    evb = TDVP1_CBE(enabled=False)
    for _ in range(3):
        eva.step(a, W, -1j * 0.02)
        evb.step(b, W, -1j * 0.02)
    assert np.linalg.norm(dense(a) - dense(b)) < 1e-14


def test_cbe_matches_oracle_trajectory(ctx):
    topo, W, Hd, psi = setup(ctx, seed=7)
    o = O.TTNS(O.star_topology(3, 2), psi.host_tensors(), psi.center)
    Ws = O.ttno_nn(O.tfi(O.star_topology(3, 2), g=0.9))
    ev = TDVP1_CBE(PredictorCBE(max_add=8, spawn_threshold=1e-10), maxdim=16)
    cache = None
    for _ in range(4):
        ev.step(psi, W, -1j * 0.02)
        cache = O.tdvp1_cbe_step(o, Ws, -1j * 0.02, cache, maxdim=16, max_add=8)
    assert psi.bond_dims() == O.bond_dims(o)
    assert abs(1 - abs(np.vdot(dense(psi), O.to_dense(o)))) < 1e-10
