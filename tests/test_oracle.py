"""CPU gates: the oracle against the reference's known-answer tests (exact diagonalisation
and identities), and the host-side metadata of the package against the oracle."""
import numpy as np
import pytest

import grafttn as G
from grafttn import contractions as GC
from oracle import ttn_oracle as O


def test_ttno_equals_dense_hamiltonian():
    # test/runtests.jl:362-393: TTNO builder == dense H within 1e-12
    for topo in (O.star_topology(3, 2), O.binary_topology(2), O.mps_topology(5)):
        for H in (O.tfi(topo, g=0.7), O.heisenberg(topo)):
            assert np.abs(O.ttno_to_dense(topo, O.ttno_nn(H)) - O.dense_hamiltonian(H)).max() < 1e-12


def test_package_ttno_matches_oracle():
    for name in ("star", "binary", "mps", "kary"):
        gt = {"star": G.star_topology(3, 2), "binary": G.binary_topology(3), "mps": G.mps_topology(6),
              "kary": G.kary_topology(4, 2)}[name]
        ot = {"star": O.star_topology(3, 2), "binary": O.binary_topology(3), "mps": O.mps_topology(6),
              "kary": O.kary_topology(4, 2)}[name]
        assert gt.parent == ot.parent and gt.children == ot.children and gt.postorder() == ot.postorder()
        for gh, oh in ((G.tfi(gt, J=1.0, g=0.9), O.tfi(ot, J=1.0, g=0.9)), (G.heisenberg(gt), O.heisenberg(ot))):
            for a, b in zip(G.ttno_tensors(gh), O.ttno_nn(oh)):
                assert a.shape == b.shape and np.array_equal(a, b)


def test_dmrg_vs_ed():
    # test/runtests.jl:687-700: TFI g=0.9 on star_topology(3,1), maxdim 16, 8 sweeps, 1e-10
    topo = O.star_topology(3, 1)
    H = O.tfi(topo, g=0.9)
    E0, _ = O.exact_groundstate(O.dense_hamiltonian(H))
    psi = O.random_ttns(np.random.default_rng(1), topo, 2, 2)
    _, Es = O.dmrg2(psi, O.ttno_nn(H), maxdim=16, nsweeps=8)
    assert abs(Es[-1] - E0) < 1e-10


def test_dmrg_star32_matches_golden():
    # the CPU-runnable workload: star_topology(3,2), -1.0 ZZ, -0.9 X, bond 2, maxdim 32
    golden = np.load(__file__.replace("test_oracle.py", "golden/star32_tfi.npz"))
    topo = O.star_topology(3, 2)
    H = O.tfi(topo, J=1.0, g=0.9)
    psi = O.random_ttns(np.random.default_rng(1), topo, 2, 2)
    _, Es = O.dmrg2(psi, O.ttno_nn(H), maxdim=32, nsweeps=10)
    assert abs(Es[-1] - float(golden["E_ed"])) < 1e-10


def test_closure_roundtrip_hermitian():
    topo = O.star_topology(3, 2)
    H = O.tfi(topo)
    Ws = O.ttno_nn(H)
    psi = O.random_ttns(np.random.default_rng(3), topo, 2, 4)
    v = O.to_dense(psi)
    Hd = O.dense_hamiltonian(H)
    # eff_h1 closes to <psi|H|psi> (test/runtests.jl:654-672)
    assert abs(O.expect(psi, Ws) - np.vdot(v, Hd @ v)) < 1e-12
    # merge/split round trip (test/runtests.jl:674-685)
    n, m = topo.index["b2_2"], topo.index["b2_1"]
    O.move_center(psi, n)
    th = O.two_site_tensor(psi, n, m)
    O.split_two_site(psi, th, n, m, center_on="m")
    assert np.linalg.norm(O.to_dense(psi) - v) < 1e-12
    # planned (env-first) == unplanned single ncon, and Hermitian (contraction_planning.jl:111-160)
    cache = O.EnvCache(topo)
    h2 = O.eff_h2(cache, psi, Ws, n, m)
    rng = np.random.default_rng(0)
    a, b = O.randn_c(rng, h2.shape), O.randn_c(rng, h2.shape)
    y_plan = h2(a)
    y_ref = O.ncon([a] + h2.statics, h2.labels, None, list(range(len(h2.labels))))
    assert np.linalg.norm(y_plan - y_ref) < 1e-11 * np.linalg.norm(y_ref)
    assert abs(np.vdot(a, h2(b)) - np.vdot(h2(a), b)) < 1e-11 * np.linalg.norm(a) * np.linalg.norm(b)


def test_tdvp1_full_rank_vs_exact():
    # test/runtests.jl:895-930: full-rank TDVP1 == exact evolution (fidelity 1e-10)
    topo = O.star_topology(3, 2)
    H = O.tfi(topo, g=0.9)
    Ws = O.ttno_nn(H)
    psi = O.random_ttns(np.random.default_rng(2), topo, 2, 8)
    Hd = O.dense_hamiltonian(H)
    vex = O.exact_evolve(Hd, O.to_dense(psi), -1j * 0.02 * 5)
    cache = None
    for _ in range(5):
        cache = O.tdvp1_step(psi, Ws, -1j * 0.02, cache)
    v = O.to_dense(psi)
    assert abs(1 - abs(np.vdot(v, vex))) < 1e-10
    assert abs(O.expect(psi, Ws) - np.vdot(vex, Hd @ vex)) < 1e-8


def test_dmrg1_full_bonds_vs_ed():
    # GroundState.jl:51-84 with full bond spaces: the variational space is complete
    topo = O.star_topology(3, 2)
    H = O.tfi(topo, g=0.9)
    E0, _ = O.exact_groundstate(O.dense_hamiltonian(H))
    psi = O.random_ttns(np.random.default_rng(5), topo, 2, 8)
    _, Es = O.dmrg1(psi, O.ttno_nn(H), nsweeps=10)
    assert abs(Es[-1] - E0) < 1e-10


def test_dmrg1_3s_grows_bonds_to_ed():
    # GroundState.jl:166-248: from bond 1, expansion between one-site sweeps reaches the
    # exact ground state of the 7-site star once the bonds have grown
    topo = O.star_topology(3, 2)
    H = O.tfi(topo, g=0.9)
    E0, _ = O.exact_groundstate(O.dense_hamiltonian(H))
    psi = O.random_ttns(np.random.default_rng(6), topo, 2, 1)
    _, Es = O.dmrg1_3s(psi, O.ttno_nn(H), maxdim=8, nsweeps=12, max_add=4)
    assert max(O.bond_dims(psi)) > 1
    assert abs(Es[-1] - E0) < 1e-9


@pytest.mark.parametrize("scheme", ["directqr", "rsvd", "rangefinder"])
def test_dmrg1_3s_schemes_grow_bonds_to_ed(scheme):
    # expand!'s other predictor schemes (expansion.jl:240-370) reach the same exact ground
    # state of the 7-site star from bond 1
    topo = O.star_topology(3, 2)
    H = O.tfi(topo, g=0.9)
    E0, _ = O.exact_groundstate(O.dense_hamiltonian(H))
    psi = O.random_ttns(np.random.default_rng(6), topo, 2, 1)
    _, Es = O.dmrg1_3s(psi, O.ttno_nn(H), maxdim=8, nsweeps=12, max_add=4, expand_scheme=scheme,
                       rng=np.random.default_rng(40))
    assert max(O.bond_dims(psi)) > 1
    assert abs(Es[-1] - E0) < 1e-9


@pytest.mark.parametrize("scheme,kw", [("exact", {}), ("rsvd", dict(oversample=2)), ("directqr", {}),
                                       ("rangefinder", dict(oversample=2, poweriter=1))])
def test_expand_keeps_the_state_and_grows_the_bond(scheme, kw):
    # the reference's expand! gates (test/runtests.jl:702-748): on a leaf edge of a bond-1
    # state of the 4-site star, every scheme leaves the state unchanged and grows the bond
    # within maxdim 4; the randomised schemes refuse to run without an rng
    topo = O.star_topology(3, 1)
    Ws = O.ttno_nn(O.tfi(topo, g=0.9))
    psi = O.random_ttns(np.random.default_rng(1101), topo, 2, 1)
    v = O.to_dense(psi)
    leaf = [n for n in range(topo.nnodes) if not topo.children[n]][0]
    rng = np.random.default_rng(2202) if scheme in ("rsvd", "rangefinder") else None
    O.expand(psi, Ws, O.EnvCache(topo), leaf, topo.parent[leaf], 4, max_add=3, scheme=scheme, rng=rng, **kw)
    assert np.linalg.norm(O.to_dense(psi) - v) < 1e-10
    assert 1 < max(O.bond_dims(psi)) <= 4
    if rng is not None:
        with pytest.raises(ValueError):
            O.expand(psi, Ws, O.EnvCache(topo), leaf, topo.parent[leaf], 4, max_add=3, scheme=scheme)
    with pytest.raises(ValueError):
        O.expand(psi, Ws, O.EnvCache(topo), leaf, topo.parent[leaf], 4, max_add=3, scheme="unknown")


def test_predictor_schemes_span_the_exact_predictor():
    # a rank-12 predictor: rangefinder and rsvd sketches with 12 + oversample columns capture
    # its whole range, so the exact scheme's leading directions lie inside both; directqr
    # spans the full column space; the randomised schemes insist on an explicit rng
    rng = np.random.default_rng(41)
    P = O.randn_c(rng, (40, 12)) @ O.randn_c(rng, (12, 30))
    ex = O.predictor_basis(P, 6, "exact")
    for scheme in ("rsvd", "rangefinder"):
        B = O.predictor_basis(P, 12, scheme, np.random.default_rng(42), oversample=4)
        assert np.allclose(B.conj().T @ B, np.eye(B.shape[1]), atol=1e-12)
        assert np.linalg.norm(ex - B @ (B.conj().T @ ex)) < 1e-10
    Q = O.predictor_basis(P, 6, "directqr")
    assert Q.shape == (40, 30)
    assert np.linalg.norm(P - Q @ (Q.conj().T @ P)) < 1e-10 * np.linalg.norm(P)
    # power iterations sharpen an rsvd sketch smaller than the rank
    Pd = (O.randn_c(rng, (40, 40)) * 0.7 ** np.arange(40)) @ O.randn_c(rng, (40, 30))
    e0 = O.predictor_basis(Pd, 4, "exact")
    errs = []
    for q in (0, 2):
        B = O.predictor_basis(Pd, 4, "rsvd", np.random.default_rng(43), oversample=2, poweriter=q)
        errs.append(np.linalg.norm(e0 - B @ (B.conj().T @ e0)))
    assert errs[1] < errs[0]
    with pytest.raises(ValueError):
        O.predictor_basis(P, 6, "rsvd")
    with pytest.raises(ValueError):
        O.predictor_basis(P, 6, "lanczos")


def test_tdvp1_non_hermitian_full_rank_vs_exact():
    # TFI plus an imaginary field 0.3i Z: the Arnoldi exponential (ishermitian = false,
    # tdvp.jl:204-281); at full bond dimension the TDVP1 splitting reproduces exp(dz H) v
    # for this non-normal generator as it does for a Hermitian one
    topo = O.star_topology(3, 2)
    H = O.tfi(topo, g=0.9)
    S = O.spin_ops()
    for i in range(topo.nnodes):
        H.onsite[i] = H.onsite[i] + 0.3j * S["Z"]
    Hd = O.dense_hamiltonian(H)
    psi = O.random_ttns(np.random.default_rng(12), topo, 2, 8)
    v0 = O.to_dense(psi)
    vex = O.exact_evolve(Hd, v0, -1j * 0.02 * 5)
    cache = None
    for _ in range(5):
        cache = O.tdvp1_step(psi, O.ttno_nn(H), -1j * 0.02, cache, hermitian=False)
    v1 = O.to_dense(psi)
    assert abs(np.linalg.norm(vex) - 1) > 1e-6  # not norm-preserving
    assert np.linalg.norm(v1 - vex) < 1e-9 * np.linalg.norm(vex)
    # the Lanczos form on the same generator is measurably wrong
    psi2 = O.random_ttns(np.random.default_rng(12), topo, 2, 8)
    cache = None
    for _ in range(5):
        cache = O.tdvp1_step(psi2, O.ttno_nn(H), -1j * 0.02, cache)
    assert np.linalg.norm(O.to_dense(psi2) - vex) > 1e-6 * np.linalg.norm(vex)


def test_tdvp2_full_rank_vs_exact():
    # full bond dimension: every two-site and one-site projector is the identity, so the
    # order-2 TDVP2 step equals exact evolution (tdvp.jl:307-431)
    topo = O.star_topology(3, 2)
    H = O.tfi(topo, g=0.9)
    Ws = O.ttno_nn(H)
    psi = O.random_ttns(np.random.default_rng(3), topo, 2, 8)
    Hd = O.dense_hamiltonian(H)
    vex = O.exact_evolve(Hd, O.to_dense(psi), -1j * 0.05 * 4)
    cache = None
    for _ in range(4):
        cache = O.tdvp2_step(psi, Ws, -1j * 0.05, cache, maxdim=64)
    assert abs(1 - abs(np.vdot(O.to_dense(psi), vex))) < 1e-10


def test_tdvp2_grows_bonds_from_product_state():
    # from bond dimension 1 TDVP2 grows the bonds (bounded by maxdim) and stays close to
    # exact evolution for a short time
    topo = O.star_topology(3, 2)
    H = O.tfi(topo, g=0.9)
    Ws = O.ttno_nn(H)
    psi = O.random_ttns(np.random.default_rng(4), topo, 2, 1)
    Hd = O.dense_hamiltonian(H)
    vex = O.exact_evolve(Hd, O.to_dense(psi), -1j * 0.02 * 5)
    cache = None
    for _ in range(5):
        cache = O.tdvp2_step(psi, Ws, -1j * 0.02, cache, maxdim=4, atol=1e-12)
    assert max(O.bond_dims(psi)) > 1 and max(O.bond_dims(psi)) <= 4
    assert abs(1 - abs(np.vdot(O.to_dense(psi), vex))) < 1e-4


@pytest.mark.parametrize("which", ["h1", "h2", "env"])
def test_package_specs_match_oracle(which):
    gt, ot = G.binary_topology(3), O.binary_topology(3)
    for n in range(gt.nnodes):
        K = gt.nchildren(n)
        if which == "h1":
            gl, go, _ = GC.h1_spec(gt, n, K + 2, K + 3)
            ol, oo = O.h1_spec(ot, n, K + 2, K + 3)
            assert gl == ol and go == oo
        elif which == "env":
            for v in gt.neighbors(n):
                gl, gc, _, _ = GC.env_spec(gt, n, v, K + 2, K + 3)
                a = np.zeros((1,) * (K + 2))
                w = np.zeros((1,) * (K + 3))
                ol, oc, _, _ = O.env_spec(ot, n, v, a, w)
                assert gl == ol and gc == oc
        elif gt.parent[n] >= 0:
            m = gt.parent[n]
            pn = K + 1
            xr = pn + gt.nchildren(m) + 1
            gl, go, _ = GC.h2_spec(gt, n, m, xr, K + 3, gt.nchildren(m) + 3, pn)
            ol, oo, _ = O.h2_spec(ot, n, m, xr, K + 3, gt.nchildren(m) + 3, pn)
            assert gl == ol and go == oo


def test_tdvp1_cbe_oracle_vs_exact():
    # test/runtests.jl:933-958: TDVP1_CBE from bond dimension 1 tracks exact evolution (1e-6),
    # plain TDVP1 stays stuck, and disabled expansion reproduces TDVP1 exactly
    topo = O.star_topology(3, 2)
    H = O.tfi(topo, g=0.9)
    Ws = O.ttno_nn(H)
    Hd = O.dense_hamiltonian(H)
    psi = O.random_ttns(np.random.default_rng(5), topo, 2, 1)
    vex = O.exact_evolve(Hd, O.to_dense(psi), -1j * 0.02 * 10)
    p = psi.copy()
    cache = None
    for _ in range(10):
        cache = O.tdvp1_cbe_step(p, Ws, -1j * 0.02, cache, maxdim=16, max_add=8)
    assert max(O.bond_dims(p)) > 1
    assert abs(1 - abs(np.vdot(O.to_dense(p), vex))) < 1e-6
    a, b = psi.copy(), psi.copy()
    ca = cb = None
    for _ in range(3):
        ca = O.tdvp1_step(a, Ws, -1j * 0.02, ca)
        cb = O.tdvp1_cbe_step(b, Ws, -1j * 0.02, cb, enabled=False)
    assert np.linalg.norm(O.to_dense(a) - O.to_dense(b)) < 1e-14


def test_sparse_hamiltonian_matches_dense():
    topo = O.star_topology(2, 2)
    H = O.heisenberg(topo)
    Hs = O.sparse_hamiltonian(H)
    assert np.abs(Hs.toarray() - O.dense_hamiltonian(H)).max() < 1e-14
    assert abs(O.sparse_ground_energy(Hs) - O.exact_groundstate(O.dense_hamiltonian(H))[0]) < 1e-10
