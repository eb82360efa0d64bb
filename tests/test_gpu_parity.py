"""The reference's own known-answer gates, run on the GPU path through the C ABI:
DMRG vs exact diagonalisation (test/runtests.jl:687-700), eff_h1 Rayleigh closure
(:654-672), merge/split round trip (:674-685), planned map == unplanned ncon and Hermitian
(test/contraction_planning.jl:111-160), TDVP1 vs exact propagation (:895-959)."""
import numpy as np
import pytest

import grafttn as G
from oracle import ttn_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def oracle_state(psi_dev):
    o = O.TTNS(O.TreeTopology(psi_dev.topo.ids[0], [(psi_dev.topo.ids[psi_dev.topo.parent[i]], psi_dev.topo.ids[i])
                                                     for i in range(1, psi_dev.topo.nnodes)]),
               psi_dev.host_tensors(), psi_dev.center)
    return o


def test_dmrg_vs_ed_star31(ctx):
    topo = G.star_topology(3, 1)
    H = G.tfi(topo, g=0.9)
    Hd = O.dense_hamiltonian(O.tfi(O.star_topology(3, 1), g=0.9))
    E0, _ = O.exact_groundstate(Hd)
    psi = G.random_ttns(np.random.default_rng(11), topo, 2, 2, ctx=ctx)
    W = G.TTNO.from_hamiltonian(H, ctx)
    _, Es = G.dmrg2(psi, W, G.TruncationScheme(maxdim=16), nsweeps=8)
    assert abs(Es[-1] - E0) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "bf16x6", "fp16x3"])
def test_dmrg_star32_tfi(ctx, precision):
    # star_topology(3,2) TFI (-1.0 ZZ, -0.9 X), bond 2, maxdim 32, 10 sweeps (exactly ED-checkable)
    topo = G.star_topology(3, 2)
    H = G.tfi(topo, J=1.0, g=0.9)
    E0, _ = O.exact_groundstate(O.dense_hamiltonian(O.tfi(O.star_topology(3, 2), J=1.0, g=0.9)))
    psi = G.random_ttns(np.random.default_rng(1), topo, 2, 2, ctx=ctx)
    W = G.TTNO.from_hamiltonian(H, ctx)
    _, Es = G.dmrg2(psi, W, G.TruncationScheme(maxdim=32), nsweeps=10, precision=precision)
    assert abs(Es[-1] - E0) / abs(E0) < 1e-10


@pytest.mark.parametrize("precision,fp64e", [("fp64", False), ("bf16x6", False), ("fp16x3", False),
                                             ("fp16x3", True)])
def test_dmrg_mps16_heisenberg_d256(ctx, precision, fp64e):
    # 16-site Heisenberg chain at bond 256 (exact): the centre two-site splits are 512 x 512
    # and go through the Gram-matrix SVD; energy against sparse Lanczos of the full matrix.
    # The mixed modes refine every local eigenvector with FP64 residuals (gtn_lanczos_refine)
    # and meet the FP64 bound, 1e-10 relative; with fp64e the environments, residuals and
    # Rayleigh quotients run in the FP64-grade tensor-core precision.
    E0 = O.sparse_ground_energy(O.sparse_hamiltonian(O.heisenberg(O.mps_topology(16))))
    topo = G.mps_topology(16)
    psi = G.random_ttns(np.random.default_rng(3), topo, 2, 256, ctx=ctx)
    W = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    _, Es = G.dmrg2(psi, W, G.TruncationScheme(maxdim=256), nsweeps=3, precision=precision,
                    refine="off" if precision == "fp64" else "all", fp64e=fp64e)
    assert abs(Es[-1] - E0) / abs(E0) < 1e-10, (Es, E0)
    assert abs(psi.norm() - 1.0) < 1e-10


def test_h1_closure_and_hermitian(ctx):
    topo = G.star_topology(3, 2)
    H = G.tfi(topo)
    W = G.TTNO.from_hamiltonian(H, ctx)
    psi = G.random_ttns(np.random.default_rng(3), topo, 2, 4, ctx=ctx)
    o = oracle_state(psi)
    Ws = O.ttno_nn(O.tfi(o.topo))
    v = O.to_dense(o)
    Hd = O.dense_hamiltonian(O.tfi(o.topo))
    e_dense = np.vdot(v, Hd @ v)
    e_gpu = G.expect(psi, W)
    assert abs(e_gpu - e_dense) < 1e-12
    cache = G.EnvCache(topo)
    c = psi.center
    h1 = G.eff_h1(cache, psi, W, c)
    x = psi.tensors[c]
    assert abs(ctx.dot(x, h1(x)) - e_dense) < 1e-12
    rng = np.random.default_rng(4)
    a = ctx.upload(O.randn_c(rng, tuple(x.shape)))
    b = ctx.upload(O.randn_c(rng, tuple(x.shape)))
    assert abs(ctx.dot(a, h1(b)) - ctx.dot(h1(a), b)) < 1e-11 * ctx.norm(a) * ctx.norm(b)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 2e-5), ("bf16x6", 2e-6), ("bf16x3", 1e-3),
                                           ("fp16x3", 4e-6)])
def test_h2_matches_oracle_binary_heisenberg(ctx, precision, tol):
    # planned GPU map == oracle ncon on every bond of a binary tree (contraction_planning.jl:111-160)
    topo = G.binary_topology(3)
    H = G.heisenberg(topo)
    W = G.TTNO.from_hamiltonian(H, ctx)
    psi = G.random_ttns(np.random.default_rng(5), topo, 2, 6, ctx=ctx)
    ot = O.binary_topology(3)
    Ws = O.ttno_nn(O.heisenberg(ot))
    rng = np.random.default_rng(6)
    for n in [7, 3, 1]:
        m = topo.parent[n]
        G.move_center(psi, n)
        o = oracle_state(psi)
        cache, ocache = G.EnvCache(topo), O.EnvCache(ot)
        h2 = G.eff_h2(cache, psi, W, n, m, precision)
        oh2 = O.eff_h2(ocache, o, Ws, n, m)
        x = O.randn_c(rng, oh2.shape)
        y = ctx.download(h2(ctx.upload(x)))
        assert rel(y, oh2(x)) < tol, (n, precision)
        h2.close()


@pytest.mark.parametrize("which", ["fork", "kary"])
def test_maps_match_oracle_on_fork_and_kary_trees(ctx, which):
    # planned maps == oracle ncon and Hermitian on the fork and 3-ary trees
    # (test/contraction_planning.jl:111-160,219-228): eff_h1 at every node, eff_h2 on every edge
    topo = G.fork_topology(2, 2) if which == "fork" else G.kary_topology(3, 2)
    W = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    psi = G.random_ttns(np.random.default_rng(30), topo, 2, 3, ctx=ctx)
    rng = np.random.default_rng(31)
    for n in range(topo.nnodes):
        G.move_center(psi, n)
        o = oracle_state(psi)
        Ws = O.ttno_nn(O.heisenberg(o.topo))
        cache, ocache = G.EnvCache(topo), O.EnvCache(o.topo)
        h1, oh1 = G.eff_h1(cache, psi, W, n), O.eff_h1(ocache, o, Ws, n)
        a, b = O.randn_c(rng, oh1.shape), O.randn_c(rng, oh1.shape)
        ha, hb = ctx.download(h1(ctx.upload(a))), ctx.download(h1(ctx.upload(b)))
        assert rel(ha, oh1(a)) < 1e-12, (which, n)
        assert abs(np.vdot(a, hb) - np.vdot(ha, b)) < 1e-11 * np.linalg.norm(a) * np.linalg.norm(b)
        h1.close()
        if topo.parent[n] >= 0:
            m = topo.parent[n]
            h2, oh2 = G.eff_h2(cache, psi, W, n, m, "fp64"), O.eff_h2(ocache, o, Ws, n, m)
            x = O.randn_c(rng, oh2.shape)
            assert rel(ctx.download(h2(ctx.upload(x))), oh2(x)) < 1e-12, (which, n, m)
            h2.close()


def test_h0_and_env_match_oracle(ctx):
    topo = G.binary_topology(2)
    H = G.heisenberg(topo)
    W = G.TTNO.from_hamiltonian(H, ctx)
    psi = G.random_ttns(np.random.default_rng(8), topo, 2, 3, ctx=ctx)
    ot = O.binary_topology(2)
    Ws = O.ttno_nn(O.heisenberg(ot))
    n, m = 3, 1
    G.move_center(psi, n)
    o = oracle_state(psi)
    cache, ocache = G.EnvCache(topo), O.EnvCache(ot)
    for (u, v) in [(3, 1), (1, 3), (0, 1), (1, 0)]:
        e = ctx.download(cache.env(psi, W, u, v))
        assert rel(e, ocache.env(o, Ws, u, v)) < 1e-12
    k0 = G.eff_h0(cache, psi, W, n, m)
    ok0 = O.eff_h0(ocache, o, Ws, n, m)
    x = O.randn_c(np.random.default_rng(9), ok0.shape)
    assert rel(ctx.download(k0(ctx.upload(x))), ok0(x)) < 1e-12


def test_h0_non_square_link_matches_oracle(ctx):
    # test/contraction_planning.jl:1151-1193: the TDVP1 child -> parent QR seam with a wide
    # old bond (physical 2, bond 4) leaves a non-square link C (2 x 4); h0 on C and on an
    # independent probe of that shape matches the oracle
    topo = G.mps_topology(2)
    root, child = 0, 1
    rng = np.random.default_rng(1701)
    tensors = [O.randn_c(rng, (4, 2, 1)), O.randn_c(rng, (2, 4))]   # root, child
    psi = G.TTNS(topo, tensors, child, ctx)
    W = G.TTNO.from_hamiltonian(G.tfi(topo, g=0.37), ctx)
    Q, C = G.networks.left_orth(ctx, psi.tensors[child])
    assert tuple(C.shape) == (2, 4)
    psi.tensors[child] = Q
    cache = G.EnvCache(topo)
    k0 = G.eff_h0(cache, psi, W, child, root)
    o = oracle_state(psi)
    ok0 = O.eff_h0(O.EnvCache(o.topo), o, O.ttno_nn(O.tfi(O.mps_topology(2), g=0.37)), child, root)
    assert tuple(ok0.shape) == (2, 4)
    for x in (ctx.download(C), O.randn_c(np.random.default_rng(1702), (2, 4))):
        assert rel(ctx.download(k0(ctx.upload(x))), ok0(x)) < 1e-12
    k0.close()


@pytest.mark.parametrize("which", ["mps6", "star32", "bin2"])
def test_gauge_moves_keep_the_state(ctx, which):
    # test/runtests.jl:336-347: a random bond-3 state is normalised, and moving its centre
    # to a leaf leaves the state unchanged
    topo = {"mps6": G.mps_topology(6), "star32": G.star_topology(3, 2), "bin2": G.binary_topology(2)}[which]
    psi = G.random_ttns(np.random.default_rng(20), topo, 2, 3, ctx=ctx)
    assert abs(psi.norm() - 1) < 1e-12
    v = O.to_dense(oracle_state(psi))
    assert abs(np.linalg.norm(v) - 1) < 1e-12
    leaf = [n for n in range(topo.nnodes) if not topo.children[n]][-1]
    G.move_center(psi, leaf)
    assert psi.center == leaf
    assert np.linalg.norm(O.to_dense(oracle_state(psi)) - v) < 1e-12


def test_merge_split_roundtrip(ctx):
    topo = G.star_topology(3, 2)
    psi = G.random_ttns(np.random.default_rng(10), topo, 2, 3, ctx=ctx)
    v0 = O.to_dense(oracle_state(psi))
    n, m = topo.index["b2_2"], topo.index["b2_1"]
    G.move_center(psi, n)
    theta = G.two_site_tensor(psi, n, m)
    G.split_two_site(psi, theta, n, m, center_on="m")
    assert np.linalg.norm(O.to_dense(oracle_state(psi)) - v0) < 1e-12


def test_tdvp1_full_rank_vs_exact(ctx):
    topo = G.star_topology(3, 2)
    H = G.tfi(topo, g=0.9)
    W = G.TTNO.from_hamiltonian(H, ctx)
    psi = G.random_ttns(np.random.default_rng(12), topo, 2, 8, ctx=ctx)
    Hd = O.dense_hamiltonian(O.tfi(O.star_topology(3, 2), g=0.9))
    v0 = O.to_dense(oracle_state(psi))
    dt, nsteps = 0.02, 5
    vex = O.exact_evolve(Hd, v0, -1j * dt * nsteps)
    ev = G.TDVP1(order=2)
    for _ in range(nsteps):
        ev.step(psi, W, -1j * dt)
    v1 = O.to_dense(oracle_state(psi))
    assert abs(1 - abs(np.vdot(v1, vex))) < 1e-10
    assert abs(np.linalg.norm(v1) - 1) < 1e-10


def test_tdvp1_non_hermitian_full_rank_vs_exact(ctx):
    # a TTNO without the Hermitian trait (TFI plus an imaginary field 0.3i Z on every site)
    # takes the Arnoldi exponential, as the reference's TDVP passes ishermitian(H) = false
    # to exponentiate (tdvp.jl:204-281); at full bond dimension TDVP1 is exact, and the
    # evolution is not norm-preserving
    topo = G.star_topology(3, 2)
    H = G.tfi(topo, g=0.9)
    S = G.spin_ops()
    for i in range(topo.nnodes):
        H.onsite[i] = H.onsite[i] + 0.3j * S["Z"]
    H.hermitian = False
    W = G.TTNO.from_hamiltonian(H, ctx)
    assert not W.ishermitian
    Ho = O.tfi(O.star_topology(3, 2), g=0.9)
    So = O.spin_ops()
    for i in range(len(Ho.onsite)):
        Ho.onsite[i] = Ho.onsite[i] + 0.3j * So["Z"]
    Hd = O.dense_hamiltonian(Ho)
    assert np.linalg.norm(Hd - Hd.conj().T) > 1.0
    psi = G.random_ttns(np.random.default_rng(12), topo, 2, 8, ctx=ctx)
    v0 = O.to_dense(oracle_state(psi))
    dt, nsteps = 0.02, 5
    vex = O.exact_evolve(Hd, v0, -1j * dt * nsteps)
    ev = G.TDVP1(order=2)
    for _ in range(nsteps):
        ev.step(psi, W, -1j * dt)
    v1 = O.to_dense(oracle_state(psi))
    assert abs(np.linalg.norm(vex) - 1) > 1e-6  # not norm-preserving
    assert np.linalg.norm(v1 - vex) < 1e-9 * np.linalg.norm(vex)


def test_tdvp2_full_rank_vs_exact(ctx):
    topo = G.star_topology(3, 2)
    W = G.TTNO.from_hamiltonian(G.tfi(topo, g=0.9), ctx)
    psi = G.random_ttns(np.random.default_rng(13), topo, 2, 8, ctx=ctx)
    Hd = O.dense_hamiltonian(O.tfi(O.star_topology(3, 2), g=0.9))
    v0 = O.to_dense(oracle_state(psi))
    vex = O.exact_evolve(Hd, v0, -1j * 0.05 * 4)
    ev = G.TDVP2(order=2, trunc=G.TruncationScheme(maxdim=64))
    for _ in range(4):
        ev.step(psi, W, -1j * 0.05)
    assert abs(1 - abs(np.vdot(O.to_dense(oracle_state(psi)), vex))) < 1e-10


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("bf16x6", 1e-10)])
def test_tdvp2_truncated_matches_oracle_trajectory(ctx, precision, tol):
    # bond growth from a product state under truncation: the same bond dimensions and the
    # same state as the oracle's TDVP2 after every step
    topo = G.star_topology(3, 2)
    W = G.TTNO.from_hamiltonian(G.tfi(topo, g=0.9), ctx)
    Ws = O.ttno_nn(O.tfi(O.star_topology(3, 2), g=0.9))
    psi = G.random_ttns(np.random.default_rng(14), topo, 2, 1, ctx=ctx)
    o = oracle_state(psi)
    ev = G.TDVP2(order=2, trunc=G.TruncationScheme(maxdim=4, atol=1e-12), precision=precision)
    cache = None
    for _ in range(3):
        ev.step(psi, W, -1j * 0.02)
        cache = O.tdvp2_step(o, Ws, -1j * 0.02, cache, maxdim=4, atol=1e-12)
        assert psi.bond_dims() == O.bond_dims(o)
    assert abs(1 - abs(np.vdot(O.to_dense(oracle_state(psi)), O.to_dense(o)))) < tol


@pytest.mark.parametrize("precision", ["fp64", "bf16x6"])
def test_dmrg1_full_bonds_vs_ed(ctx, precision):
    topo = G.star_topology(3, 2)
    W = G.TTNO.from_hamiltonian(G.tfi(topo, g=0.9), ctx)
    E0, _ = O.exact_groundstate(O.dense_hamiltonian(O.tfi(O.star_topology(3, 2), g=0.9)))
    psi = G.random_ttns(np.random.default_rng(15), topo, 2, 8, ctx=ctx)
    dims = psi.bond_dims()
    _, Es = G.dmrg1(psi, W, nsweeps=10, precision=precision)
    assert psi.bond_dims() == dims
    assert abs(Es[-1] - E0) / abs(E0) < 1e-10


def test_dmrg1_3s_matches_oracle_and_ed(ctx):
    # one-site DMRG with exact subspace expansion from bond 1: the same bond growth as the
    # oracle after every sweep, and the exact ground-state energy at the end
    topo = G.star_topology(3, 2)
    W = G.TTNO.from_hamiltonian(G.tfi(topo, g=0.9), ctx)
    Hd = O.dense_hamiltonian(O.tfi(O.star_topology(3, 2), g=0.9))
    E0, _ = O.exact_groundstate(Hd)
    psi = G.random_ttns(np.random.default_rng(16), topo, 2, 1, ctx=ctx)
    o = oracle_state(psi)
    _, Es = G.dmrg1_3s(psi, W, G.TruncationScheme(maxdim=8), nsweeps=3, max_add=4)
    _, Eo = O.dmrg1_3s(o, O.ttno_nn(O.tfi(O.star_topology(3, 2), g=0.9)), maxdim=8, nsweeps=3, max_add=4)
    assert psi.bond_dims() == O.bond_dims(o), (psi.bond_dims(), O.bond_dims(o))
    # the first sweep precedes any expansion; later sweeps may differ by which of several
    # equally weighted predictor directions each side kept
    assert abs(Es[0] - Eo[0]) < 1e-9 * abs(Eo[0]), (Es, Eo)
    _, Es = G.dmrg1_3s(psi, W, G.TruncationScheme(maxdim=8), nsweeps=10, max_add=4)
    assert abs(Es[-1] - E0) / abs(E0) < 1e-10


@pytest.mark.parametrize("scheme,kw", [("exact", {}), ("rsvd", dict(rsvd_oversample=2)), ("directqr", {}),
                                       ("rangefinder", dict(rsvd_oversample=2, rsvd_poweriter=1))])
def test_expand_keeps_the_state_and_grows_the_bond(ctx, scheme, kw):
    # the reference's expand! gates (test/runtests.jl:702-748) on the device path: a leaf edge
    # of a bond-1 state of the 4-site star grows within maxdim 4 and the state is unchanged
    from grafttn.contractions import EnvCache
    from grafttn.solvers import expand
    topo = G.star_topology(3, 1)
    W = G.TTNO.from_hamiltonian(G.tfi(topo, g=0.9), ctx)
    psi = G.random_ttns(np.random.default_rng(1101), topo, 2, 1, ctx=ctx)
    v = O.to_dense(oracle_state(psi))
    leaf = [n for n in range(topo.nnodes) if not topo.children[n]][0]
    rng = np.random.default_rng(2202) if scheme in ("rsvd", "rangefinder") else None
    assert expand(EnvCache(topo), psi, W, leaf, topo.parent[leaf], 4, max_add=3, scheme=scheme, rng=rng, **kw)
    assert np.linalg.norm(O.to_dense(oracle_state(psi)) - v) < 1e-10
    assert 1 < max(psi.bond_dims()) <= 4
    with pytest.raises(ValueError):
        expand(EnvCache(topo), psi, W, leaf, topo.parent[leaf], 4, max_add=3, scheme="unknown")


@pytest.mark.parametrize("scheme", ["directqr", "rsvd", "rangefinder"])
def test_dmrg1_3s_schemes_match_oracle_and_ed(ctx, scheme):
    # expand!'s other predictor schemes (expansion.jl:240-370), probes drawn from the same
    # seeded Generator on both sides: the same bond growth as the oracle, the same energy
    # after the first sweep, and the exact ground state once the bonds have grown
    topo = G.star_topology(3, 2)
    W = G.TTNO.from_hamiltonian(G.tfi(topo, g=0.9), ctx)
    Hd = O.dense_hamiltonian(O.tfi(O.star_topology(3, 2), g=0.9))
    E0, _ = O.exact_groundstate(Hd)
    psi = G.random_ttns(np.random.default_rng(16), topo, 2, 1, ctx=ctx)
    o = oracle_state(psi)
    _, Es = G.dmrg1_3s(psi, W, G.TruncationScheme(maxdim=8), nsweeps=3, max_add=4, expand_scheme=scheme,
                       rng=np.random.default_rng(60))
    _, Eo = O.dmrg1_3s(o, O.ttno_nn(O.tfi(O.star_topology(3, 2), g=0.9)), maxdim=8, nsweeps=3, max_add=4,
                       expand_scheme=scheme, rng=np.random.default_rng(60))
    assert psi.bond_dims() == O.bond_dims(o), (psi.bond_dims(), O.bond_dims(o))
    assert abs(Es[0] - Eo[0]) < 1e-9 * abs(Eo[0]), (Es, Eo)
    _, Es = G.dmrg1_3s(psi, W, G.TruncationScheme(maxdim=8), nsweeps=10, max_add=4, expand_scheme=scheme,
                       rng=np.random.default_rng(61))
    assert abs(Es[-1] - E0) / abs(E0) < 1e-10
    with pytest.raises(ValueError):
        G.dmrg1_3s(psi, W, G.TruncationScheme(maxdim=8), nsweeps=1, expand_scheme=scheme if scheme != "directqr"
                   else "lanczos")
