"""The adjoint entry point (gtn_contract_vjp) through the C ABI: its defining identity
<G, d op> = <ybar, dy> on a random contraction with conjugated operands; the environment
update's adjoints against central finite differences; and the gradient of
E(theta) = <psi|H(theta)|psi> with respect to the couplings of XXZ (Delta = 0.7) on the
31-site binary tree, by the W adjoints, against central finite differences (h = 1e-6) and
against the two-site expectation values."""
import numpy as np
import pytest

import grafttn as G
from grafttn import _lib
from grafttn import gradients as GR
from grafttn.contractions import EnvCache, env_spec
from oracle import ttn_oracle as O

pytestmark = pytest.mark.gpu


def crandn(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def ip(a, b):
    return np.vdot(a.ravel(), b.ravel())


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp16x3", 3e-5)])
def test_contract_vjp_identity(ctx, prec, tol):
    rng = np.random.default_rng(1)
    shapes = [(4, 5, 6), (6, 3, 7), (5, 7, 2), (2, 9)]
    labels = [[-1, 1, 2], [2, -2, 3], [1, 3, 4], [4, -3]]
    conj = [False, True, False, True]
    ops = [crandn(rng, s) for s in shapes]
    y = O.ncon(ops, labels, conj)
    ybar = crandn(rng, y.shape)
    dev = [ctx.upload(o) for o in ops]
    for slot in range(len(ops)):
        Gs = ctx.download(ctx.contract_vjp(dev, labels, ctx.upload(ybar), slot, conj=conj,
                                           precision=_lib.PRECISIONS[prec]))
        assert Gs.shape == shapes[slot]
        d = crandn(rng, shapes[slot])
        ops2 = list(ops)
        # the perturbation of the operand as it enters the contraction (after its conj flag)
        ops2[slot] = ops[slot] + (d.conj() if conj[slot] else d)
        dy = O.ncon(ops2, labels, conj) - y
        lhs, rhs = ip(Gs, d), ip(ybar, dy)
        assert abs(lhs - rhs) <= tol * abs(rhs), (slot, lhs, rhs)


def test_env_update_vjp_vs_finite_differences(ctx):
    # L(A, W) = Re <C, E(u->v)> for one environment update of a random bin7 state at bond 4:
    # W enters once (L linear in W), A twice (ket, and bra with conj: L quadratic in A)
    topo = G.binary_topology(2)
    Hd = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    psi = G.random_ttns(np.random.default_rng(2), topo, 2, 4, ctx=ctx)
    cache = EnvCache(topo)
    u, v = 1, 0  # the env of node 1 towards its parent (the root)
    pre = {w: cache.env(psi, Hd, w, u) for w in topo.neighbors(u) if w != v}
    A, W = psi.tensors[u].contiguous(), Hd.tensors[u]
    labels, conj, envs, has_cap = env_spec(topo, u, v, A.dim(), W.dim())
    assert not has_cap
    ops = [A] + [pre[w] for w in envs] + [W, A]
    iW, iket, ibra = len(ops) - 2, 0, len(ops) - 1
    E0 = ctx.contract(ops, labels, conj)
    rng = np.random.default_rng(3)
    Cb = ctx.upload(crandn(rng, tuple(E0.shape)))

    def L(ops_):
        return ctx.dot(Cb, ctx.contract(ops_, labels, conj)).real

    h = 1e-6
    # W
    GW = ctx.contract_vjp(ops, labels, Cb, iW, conj=conj)
    Dw = ctx.upload(crandn(rng, tuple(W.shape)))
    opp, opm = list(ops), list(ops)
    opp[iW], opm[iW] = ctx.axpby(h, Dw, 1.0, W.clone()), ctx.axpby(-h, Dw, 1.0, W.clone())
    fd = (L(opp) - L(opm)) / (2 * h)
    an = ctx.dot(GW, Dw).real
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)
    # A through both of its slots
    Gk = ctx.download(ctx.contract_vjp(ops, labels, Cb, iket, conj=conj))
    Gb = ctx.download(ctx.contract_vjp(ops, labels, Cb, ibra, conj=conj))
    Da = crandn(rng, tuple(A.shape))
    dA = ctx.upload(Da)
    Ap, Am = ctx.axpby(h, dA, 1.0, A.clone()), ctx.axpby(-h, dA, 1.0, A.clone())
    opp, opm = list(ops), list(ops)
    opp[iket], opp[ibra], opm[iket], opm[ibra] = Ap, Ap, Am, Am
    fd = (L(opp) - L(opm)) / (2 * h)
    an = (ip(Gk, Da) + ip(Gb, Da.conj())).real
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)


@pytest.fixture(scope="module")
def xxz_bin31(ctx):
    topo = G.binary_topology(4)
    rng = np.random.default_rng(11)
    theta = {e: float(rng.uniform(0.5, 1.5)) for e in topo.edges()}
    bond = {}
    for c in range(topo.nnodes):
        if topo.parent[c] >= 0:
            below = len(topo.subtree_nodes(c, topo.parent[c]))
            bond[c] = int(min(32, 2 ** below, 2 ** (topo.nnodes - below)))
    psi = G.random_ttns(rng, topo, 2, bond, ctx=ctx)
    return topo, theta, psi


def test_coupling_gradients_adjoint_vs_fd_and_expectations(ctx, xxz_bin31):
    topo, theta, psi = xxz_bin31
    delta = 0.7
    Hnn = G.xxz(topo, theta, delta)
    H = G.TTNO.from_hamiltonian(Hnn, ctx)
    dco = {e: [1.0, 1.0, delta] for e in topo.edges()}
    g_adj = GR.coupling_gradients_adjoint(psi, H, Hnn, dco)
    S = G.spin_ops()
    terms = {e: [(1.0, S["X"], S["X"]), (1.0, S["Y"], S["Y"]), (delta, S["Z"], S["Z"])] for e in topo.edges()}
    g_exp = GR.coupling_gradients(psi, terms)
    E = GR.energy(psi, H).real
    for e in topo.edges():
        assert abs(g_adj[e] - g_exp[e]) <= 1e-10 * max(1.0, abs(g_exp[e])), (e, g_adj[e], g_exp[e])
    # linearity in the couplings: sum_e theta_e dE/dtheta_e = E minus the on-site part (none here)
    assert abs(sum(theta[e] * g_adj[e] for e in theta) - E) <= 1e-10 * abs(E)
    h = 1e-6
    for e in list(topo.edges())[:6]:
        tp, tm = dict(theta), dict(theta)
        tp[e] += h
        tm[e] -= h
        Ep = GR.energy(psi, G.TTNO.from_hamiltonian(G.xxz(topo, tp, delta), ctx)).real
        Em = GR.energy(psi, G.TTNO.from_hamiltonian(G.xxz(topo, tm, delta), ctx)).real
        fd = (Ep - Em) / (2 * h)
        assert abs(fd - g_adj[e]) <= 1e-6 * max(1.0, abs(g_adj[e])), (e, fd, g_adj[e])


def test_ttno_gradients_under_env_budget(ctx, xxz_bin31):
    # environment recomputation: a byte budget that holds a few environments gives the same
    # W adjoints as the unbounded cache
    topo, theta, psi = xxz_bin31
    H = G.TTNO.from_hamiltonian(G.xxz(topo, theta, 0.7), ctx)
    g_full = GR.ttno_gradients(psi, H)
    g_small = GR.ttno_gradients(psi, H, max_env_bytes=3 * 32 * 5 * 32 * 16)
    for a, b in zip(g_full, g_small):
        assert ctx.norm(ctx.axpby(1.0, a, -1.0, b.clone())) <= 1e-13 * max(1.0, ctx.norm(a))
