"""U(1)-symmetric (abelian, charge-conserving) tree tensor networks on the device and the
two-site DMRG that runs on them (dmrg2!, lib/GraftGroundState/src/GroundState/
GroundState.jl:102-143, on TensorKit's abelian TensorMaps).

A tensor is a block structure (blocksparse.BlockTensor: U(1) legs with arrows, one dense
row-major block per allowed charge combination, Σ sign·q = 0) plus one flat c128 device
buffer holding every block.  The charge of a spin-1/2 basis state is its index (0 or 1),
so the total charge of a basis product state is its number of 1 entries.

Leg arrows (the planner matches contracted legs by opposite arrows):
  state A_n    children +1, phys +1, parent -1 (the root's parent leg: {Q: 1}, -1)
  TTNO W_n     children +1, P_out +1, P_in -1, parent -1 (the root's: {0: 1}, -1)
  env(w -> u)  from a child subtree: (ket -1, op -1, bra +1); from above: (+1, +1, -1)
  root cap     (bra {Q:1} -1, op {0:1} +1, ket {Q:1} +1)

Every contraction runs on the GPU through the block engine (gtn_blockmap: per coupled charge
one GEMM, all charges of a step in one grouped launch): environment updates, the two-site
merge and the effective map.  The Krylov solve is gtn_blockmap_lanczos_min on the map's flat
block buffer (mixed maps refined with FP64 residuals by gtn_blockmap_lanczos_refine).  The
gauge moves and the two-site split are per-sector factorisations: every coupled charge q of
the cut is one dense matrix (assembled from its blocks on the device), factorised by gtn_qr
or gtn_svd_trunc; the truncation rule (maxdim & atol & rtol & discarded weight,
Backend.jl:466-483) is applied to all sectors' singular values together, as TensorKit
truncates a block-diagonal spectrum.  Host work is bookkeeping: charges, offsets and the
static operands' B_q assembly of the block planner.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .blocksparse import BlockEffectiveMap, BlockPlan, BlockTensor, U1Leg, op_leg, u1_heisenberg_terms
from .contractions import env_spec, h2_spec
from .networks import TruncationScheme

PHYS = {0: 1, 1: 1}


class U1Tensor:
    """Block structure + flat device data."""

    def __init__(self, T: BlockTensor, data):
        self.T = T
        self.data = data
        self._where = {qs: (shape, off) for qs, shape, off in T.blocks}

    def block(self, qs):
        shape, off = self._where[qs]
        n = int(np.prod(shape))
        return self.data[off: off + n].view(*shape) if shape else self.data[off: off + n]

    def has(self, qs):
        return qs in self._where

    def host(self, ctx):
        return ctx.download(self.data)

    def copy(self, ctx):
        return U1Tensor(self.T, ctx.copy(self.data))


def _flip(T: BlockTensor):
    return BlockTensor([l.flipped() for l in T.legs], -T.qtot)


def _static(ctx, t: U1Tensor, conj=False):
    """(BlockTensor, host data) of a planner static; conj flips every arrow and conjugates."""
    d = t.host(ctx)
    if conj:
        T = _flip(t.T)
        return T, np.conj(d) if T.size == d.size else None
    return t.T, d


def _leg_from_sectors(sectors, sign):
    return U1Leg({q: int(d) for q, d in sectors.items() if d > 0}, sign)


def _copy2d(ctx, dst, dst_ld, src, src_ld, rows, cols):
    from ._lib import check
    check(ctx.lib.gtn_copy2d(ctx.h, rows, cols, C.c_void_p(src.data_ptr()), src_ld, C.c_void_p(dst.data_ptr()),
                             dst_ld), ctx.h, "copy2d")


class U1TTNO:
    """Charge-conserving TTNO tensors (the nearest-neighbour builder's tensors, operator bonds
    sorted by their charge)."""

    def __init__(self, ctx, topo, Hnn):
        from .operators import ttno_tensors
        self.ctx, self.topo = ctx, topo
        Wd = ttno_tensors(Hnn)
        oleg_out, operm = op_leg(+1)
        oleg_in, _ = op_leg(-1)
        self.tensors = []
        for u in range(topo.nnodes):
            W = Wd[u]
            K = topo.nchildren(u)
            root = topo.parent[u] < 0
            for ax in list(range(K)) + ([] if root else [K + 2]):
                W = np.take(W, operm, axis=ax)
            legs = [oleg_out] * K + [U1Leg(PHYS, 1), U1Leg(PHYS, -1)]
            legs.append(oleg_in if not root else U1Leg({0: 1}, -1))
            T = BlockTensor(legs)
            self.tensors.append(U1Tensor(T, ctx.upload(T.from_dense(W))))
        self.ishermitian = Hnn.hermitian


def u1_heisenberg(topo, J=1.0):
    """J (XX + YY + ZZ) (Pauli) as charge-conserving terms (2 S+S- + 2 S-S+ + ZZ)."""
    from .operators import NNHamiltonian
    H = NNHamiltonian(topo)
    for e in topo.edges():
        H.bonds[e] = [(J * c, a, b) for c, a, b in u1_heisenberg_terms()]
    return H


def bond_sectors(topo, Q, D):
    """Sectors of every bond c -> parent(c) for total charge Q: every subtree charge q that
    the rest of the tree can complete to Q, with dimension min(C(ns, q), C(N - ns, Q - q))
    (the exact rank), scaled down to at most D in total in proportion when larger."""
    N = topo.nnodes
    out = {}
    for c in range(N):
        if topo.parent[c] < 0:
            continue
        ns = len(topo.subtree_nodes(c, topo.parent[c]))
        exact = {}
        for q in range(max(0, Q - (N - ns)), min(ns, Q) + 1):
            exact[q] = min(math.comb(ns, q), math.comb(N - ns, Q - q))
        tot = sum(exact.values())
        if tot > D:
            dims = {q: max(1, min(d, int(D * d / tot))) for q, d in exact.items()}
            while sum(dims.values()) > D:
                q = max(dims, key=lambda k: (dims[k], -k))
                dims[q] -= 1
            exact = {q: d for q, d in dims.items() if d > 0}
        out[c] = exact
    return out


class U1TTNS:
    """Charge-conserving TTNS on the device with one orthogonality centre."""

    def __init__(self, ctx, topo, tensors, center, Q):
        self.ctx, self.topo, self.tensors, self.center, self.Q = ctx, topo, list(tensors), center, Q

    def structure(self, n, sectors):
        t = self.topo
        legs = [U1Leg(sectors[c], 1) for c in t.children[n]] + [U1Leg(PHYS, 1)]
        legs.append(U1Leg(sectors[n], -1) if t.parent[n] >= 0 else U1Leg({self.Q: 1}, -1))
        return BlockTensor(legs)

    @classmethod
    def random(cls, ctx, rng, topo, Q, D):
        sec = bond_sectors(topo, Q, D)
        psi = cls(ctx, topo, [None] * topo.nnodes, 0, Q)
        for n in range(topo.nnodes):
            T = psi.structure(n, sec)
            psi.tensors[n] = U1Tensor(T, ctx.upload(T.random(rng)))
        # canonical form: QR towards the root in postorder, then normalise the root
        for n in topo.postorder():
            if topo.parent[n] >= 0:
                psi.center = n
                move_center(psi, topo.parent[n])
        r = psi.tensors[psi.center]
        psi.tensors[psi.center] = U1Tensor(r.T, ctx.scale(r.data, 1.0 / ctx.norm(r.data)))
        return psi

    def copy(self):
        return U1TTNS(self.ctx, self.topo, [t.copy(self.ctx) for t in self.tensors], self.center, self.Q)

    def bond_dims(self):
        t = self.topo
        return [self.tensors[c].T.legs[-1].total for c in range(t.nnodes) if t.parent[c] >= 0]

    def norm(self):
        return self.ctx.norm(self.tensors[self.center].data)


# ---------------------------------------------------------------------------------------
# per-sector factorisations
# ---------------------------------------------------------------------------------------

def _matrices_by_charge(ctx, t: U1Tensor, nrow):
    """The tensor as block-diagonal matrices: rows = legs[:nrow], columns = the rest; the
    coupled charge of the cut is q = Σ_{rows} sign·charge.  Returns {q: (M_q device,
    row offsets {row charges: (off, n)}, col offsets {col charges: (off, n)})}."""
    rows, cols = {}, {}
    for qs, shape, _ in t.T.blocks:
        q = sum(l.sign * c for l, c in zip(t.T.legs[:nrow], qs[:nrow]))
        rk, ck = qs[:nrow], qs[nrow:]
        rows.setdefault(q, {}).setdefault(rk, int(np.prod(shape[:nrow])))
        cols.setdefault(q, {}).setdefault(ck, int(np.prod(shape[nrow:])))
    out = {}
    for q in sorted(rows):
        roff, o = {}, 0
        for rk in sorted(rows[q]):
            roff[rk] = (o, rows[q][rk])
            o += rows[q][rk]
        R = o
        coff, o = {}, 0
        for ck in sorted(cols[q]):
            coff[ck] = (o, cols[q][ck])
            o += cols[q][ck]
        Cn = o
        M = ctx.zeros((R, Cn))
        for rk, (ro, rn) in roff.items():
            for ck, (co, cn) in coff.items():
                qs = rk + ck
                if not t.has(qs):
                    continue
                blk = t.block(qs).reshape(rn, cn)
                _copy2d(ctx, M[ro:, co:], Cn, blk, cn, rn, cn)
        out[q] = (M, roff, coff)
    return out


def _assemble(ctx, T: BlockTensor, nrow, mats):
    """Inverse of _matrices_by_charge: a U1Tensor of structure T from {q: (M, roff, coff)}."""
    data = ctx.zeros((max(T.size, 1),))
    out = U1Tensor(T, data[: T.size])
    for qs, shape, _ in T.blocks:
        q = sum(l.sign * c for l, c in zip(T.legs[:nrow], qs[:nrow]))
        if q not in mats:
            continue
        M, roff, coff = mats[q]
        rk, ck = qs[:nrow], qs[nrow:]
        if rk not in roff or ck not in coff:
            continue
        ro, rn = roff[rk]
        co, cn = coff[ck]
        _copy2d(ctx, out.block(qs).reshape(rn, cn), cn, M[ro:, co:], M.shape[1], rn, cn)
    return out


def _permute(ctx, t: U1Tensor, perm):
    """Leg permutation of every block (gtn_permute per block)."""
    T2 = BlockTensor([t.T.legs[p] for p in perm], t.T.qtot)
    data = ctx.zeros((max(T2.size, 1),))
    out = U1Tensor(T2, data[: T2.size])
    for qs, shape, _ in t.T.blocks:
        q2 = tuple(qs[p] for p in perm)
        b = t.block(qs)
        ctx.copy_into(out.block(q2), ctx.permute(b.contiguous(), list(perm)) if len(shape) > 1 else b)
    return out


def left_orth_leg(ctx, t: U1Tensor, k):
    """QR of the tensor against its leg k (Backend.jl:602-609, per sector): returns
    (Q with leg k's sector dims shrunk to the kept ranks, {q: R_q}) with
    t[..., e@k, ...] = Σ_y Q[..., y@k, ...] R_q[y, e]."""
    r = len(t.T.legs)
    perm = [j for j in range(r) if j != k] + [k]
    tp = _permute(ctx, t, perm) if k != r - 1 else t
    mats = _matrices_by_charge(ctx, tp, r - 1)
    leg = tp.T.legs[-1]
    Qm, Rs, newdims = {}, {}, {}
    for q, (M, roff, coff) in mats.items():
        Q, R = ctx.qr(M)
        # charge q of the cut is Σ sign·charges of the other legs = -sign_k * charge_k
        ck = list(coff)[0]
        Qm[q] = (Q, roff, {ck: (0, Q.shape[1])})
        Rs[ck[0]] = R
        newdims[ck[0]] = Q.shape[1]
    legs = list(tp.T.legs[:-1]) + [U1Leg({c: d for c, d in newdims.items()}, leg.sign)]
    Tq = BlockTensor(legs, tp.T.qtot)
    Qt = _assemble(ctx, Tq, r - 1, Qm)
    if k != r - 1:
        inv = [0] * r
        for i, p in enumerate(perm):
            inv[p] = i
        Qt = _permute(ctx, Qt, inv)
    return Qt, Rs


def absorb_leg(ctx, t: U1Tensor, k, Rs, transpose=False):
    """t'[.., y@k, ..] = Σ_e R_q[y, e] t[.., e@k, ..] per charge q of leg k (transpose: R_q^T)."""
    legs = list(t.T.legs)
    newd = {}
    for c in legs[k].charges:
        if c in Rs:
            newd[c] = Rs[c].shape[1] if transpose else Rs[c].shape[0]
    legs[k] = U1Leg(newd, legs[k].sign)
    T2 = BlockTensor(legs, t.T.qtot)
    data = ctx.zeros((max(T2.size, 1),))
    out = U1Tensor(T2, data[: T2.size])
    r = len(legs)
    lab = [-(j + 1) for j in range(r)]
    lab[k] = 1
    for qs, shape, _ in T2.blocks:
        if not t.has(qs):
            continue
        R = Rs[qs[k]]
        Rl = [1, -(k + 1)] if transpose else [-(k + 1), 1]
        ctx.copy_into(out.block(qs), ctx.contract([t.block(qs).contiguous(), R.contiguous()], [lab, Rl]))
    return out


def move_center(psi: U1TTNS, target, cache=None):
    """(ttns.jl:126-203) QR steps along the path to target; cached environments whose side
    changed are dropped."""
    t = psi.topo
    ctx = psi.ctx
    path = t.path_between(psi.center, target)
    for m in path[1:]:
        n = psi.center
        if t.parent[n] == m:       # up: A_n = Q R on its parent leg, R into m's child slot
            k = t.childslot(m, n)
            Q, Rs = left_orth_leg(ctx, psi.tensors[n], len(psi.tensors[n].T.legs) - 1)
            psi.tensors[n] = Q
            psi.tensors[m] = absorb_leg(ctx, psi.tensors[m], k, Rs)
        else:                      # down: A_n = Q R on its child slot k, R into m's parent leg
            k = t.childslot(n, m)
            Q, Rs = left_orth_leg(ctx, psi.tensors[n], k)
            psi.tensors[n] = Q
            psi.tensors[m] = absorb_leg(ctx, psi.tensors[m], len(psi.tensors[m].T.legs) - 1, Rs)
        if cache is not None:
            cache.invalidate_node(n)
        psi.center = m


# ---------------------------------------------------------------------------------------
# environments, merge, effective map, split
# ---------------------------------------------------------------------------------------

def _cap(ctx, Q, kind="env"):
    """The all-ones root cap (Backend.jl:144-150) with the arrows of its place in the graph:
    an environment update closes (bra, op, ket) parent legs, a map (x, op) and opens the
    output's parent leg."""
    if kind == "env":
        legs = [U1Leg({Q: 1}, -1), U1Leg({0: 1}, 1), U1Leg({Q: 1}, 1)]
    else:
        legs = [U1Leg({Q: 1}, 1), U1Leg({0: 1}, 1), U1Leg({Q: 1}, -1)]
    T = BlockTensor(legs)
    return U1Tensor(T, ctx.upload(np.ones(T.size, dtype=np.complex128)))


def _block_contract(ctx, x: U1Tensor, x_labels, statics, order=None):
    """One-shot contraction on the block engine: x on the device, statics [(BlockTensor,
    labels, host data)]; returns the output U1Tensor (legs -1, -2, ...)."""
    order = order or list(range(len(statics) + 1))
    plan = BlockPlan(x.T, x_labels, statics, order)
    bm = BlockEffectiveMap(ctx, plan, "fp64")
    y = bm(x.data)
    bm.close()
    return U1Tensor(plan.y, y)


class U1EnvCache:
    """Directed-edge environments (envcache.jl:61-109) with the reference's invalidation."""

    def __init__(self, topo):
        self.topo = topo
        self.envs = {}
        self.builds = 0

    def invalidate_node(self, n):
        t = self.topo
        for key in [k for k in self.envs if t.in_subtree(n, k[0], k[1])]:
            del self.envs[key]

    def invalidate_edge(self, n, m):
        self.invalidate_node(n)
        self.invalidate_node(m)

    def env(self, psi: U1TTNS, H: U1TTNO, u, v):
        key = (u, v)
        if key in self.envs:
            return self.envs[key]
        t, ctx = self.topo, psi.ctx
        pre = {w: self.env(psi, H, w, u) for w in t.neighbors(u) if w != v}
        A, W = psi.tensors[u], H.tensors[u]
        labels, conj, envs, has_cap = env_spec(t, u, v, len(A.T.legs), len(W.T.legs))
        ops = [pre[w] for w in envs] + ([_cap(ctx, psi.Q)] if has_cap else []) + [W]
        statics = [(o.T, lab, o.host(ctx)) for o, lab in zip(ops, labels[1:-1])]
        Tb, db = _static(ctx, A, conj=True)
        statics.append((Tb, labels[-1], db))
        E = _block_contract(ctx, A, labels[0], statics)
        self.envs[key] = E
        self.builds += 1
        return E


def two_site_tensor(psi: U1TTNS, n, m):
    """Θ = A_n A_m over their bond (effective.jl:827-843): legs (n children..., phys_n,
    m children except n..., phys_m, m parent)."""
    t, ctx = psi.topo, psi.ctx
    Kn, Km, k = t.nchildren(n), t.nchildren(m), t.childslot(m, n)
    pn = Kn + 1
    la = [-(j + 1) for j in range(Kn + 1)] + [1]
    lb = []
    for j in range(Km):
        lb.append(1 if j == k else -(pn + 1 + (j if j < k else j - 1)))
    lb += [-(pn + Km), -(pn + Km + 1)]
    Am = psi.tensors[m]
    return _block_contract(ctx, psi.tensors[n], la, [(Am.T, lb, Am.host(ctx))])


def trunc_rank(s, maxdim, atol, rtol, dw):
    """The truncation rule of the dense split (maxdim & atol & rtol & relative discarded
    weight, Backend.jl:466-483) on a descending spectrum; at least one value is kept."""
    k = len(s)
    r = k if not maxdim else min(k, maxdim)
    if atol > 0 or rtol > 0:
        thr = max(atol, rtol * s[0])
        r = min(r, int(np.sum(s > thr)))
    if dw > 0:
        tot = float(np.sum(s ** 2))
        tail, rr = 0.0, k
        for i in range(k - 1, -1, -1):
            tail += s[i] ** 2
            if math.sqrt(tail) <= dw * math.sqrt(tot):
                rr = i
            else:
                break
        r = min(r, rr)
    return max(r, 1)


def split_two_site(psi: U1TTNS, theta: U1Tensor, n, m, trunc: TruncationScheme | None = None, center_on="n"):
    """Per-sector truncated SVD of Θ back into A_n, A_m (effective.jl:852-876): one SVD per
    coupled charge of the bond, the truncation rule on all sectors' values together; returns
    the discarded 2-norm."""
    t, ctx = psi.topo, psi.ctx
    trunc = trunc or TruncationScheme()
    Kn, Km, k = t.nchildren(n), t.nchildren(m), t.childslot(m, n)
    pn = Kn + 1
    mats = _matrices_by_charge(ctx, theta, pn)
    svds = {}
    allv = []
    for q, (M, roff, coff) in mats.items():
        U, S, Vh, _ = ctx.svd_trunc(M, maxdim=min(M.shape))
        svds[q] = (U, S, Vh, roff, coff)
        allv += [(float(s), q, i) for i, s in enumerate(S)]
    allv.sort(key=lambda v: (-v[0], v[1], v[2]))
    s = np.array([v[0] for v in allv])
    r = trunc_rank(s, trunc.maxdim, trunc.atol, trunc.rtol, trunc.discarded_weight)
    keep = {}
    for _, q, _ in allv[:r]:
        keep[q] = keep.get(q, 0) + 1
    disc = float(np.sqrt(np.sum(s[r:] ** 2)))
    # new bond: charge q of the cut (n-side charges, all arrows +1) with keep[q] states
    bond = U1Leg(keep, -1)
    Tn = BlockTensor(list(theta.T.legs[:pn]) + [bond])
    Un, Vm = {}, {}
    for q, (U, S, Vh, roff, coff) in svds.items():
        kq = keep.get(q, 0)
        if kq == 0:
            continue
        Uq = ctx.empty((U.shape[0], kq))
        _copy2d(ctx, Uq, kq, U, U.shape[1], U.shape[0], kq)
        Vq = Vh[:kq, :]
        if center_on == "n":
            ctx.diag_scale(Uq, S[:kq], side=0)
        else:
            ctx.diag_scale(Vq, S[:kq], side=1)
        Un[q] = (Uq, roff, {(q,): (0, kq)})
        Vm[q] = (Vq, {(q,): (0, kq)}, coff)
    psi.tensors[n] = _assemble(ctx, Tn, pn, Un)
    # A_m from S Vh: legs (bond, m's other children..., phys_m, parent), then bond to slot k
    Tv = BlockTensor([bond.flipped()] + list(theta.T.legs[pn:]))
    Av = _assemble(ctx, Tv, 1, Vm)
    perm = list(range(1, len(Tv.legs)))
    perm.insert(k, 0)
    psi.tensors[m] = _permute(ctx, Av, perm) if k != 0 else Av
    psi.center = n if center_on == "n" else m
    return disc


class U1EffH2:
    """Two-site map of edge n -> m on the block engine in `precision`, with its FP64 twin
    for Rayleigh quotients and refinement (effective.jl:986-1034)."""

    def __init__(self, cache: U1EnvCache, psi: U1TTNS, H: U1TTNO, n, m, precision="fp64", theta_T=None):
        t, ctx = psi.topo, psi.ctx
        self.ctx = ctx
        pn = t.nchildren(n) + 1
        xT = theta_T
        labels, order, envs = h2_spec(t, n, m, len(xT.legs), len(H.tensors[n].T.legs), len(H.tensors[m].T.legs), pn)
        ops = [H.tensors[n], H.tensors[m]] + [cache.env(psi, H, w, u) for (w, u) in envs]
        if t.parent[m] < 0:
            ops.append(_cap(ctx, psi.Q, "map"))
        statics = [(o.T, lab, o.host(ctx)) for o, lab in zip(ops, labels[1:])]
        self.plan = BlockPlan(xT, labels[0], statics, order)
        self.precision = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
        self.bm = BlockEffectiveMap(ctx, self.plan, self.precision)
        self.bm64 = self.bm if self.precision == _lib.PREC_FP64 else BlockEffectiveMap(ctx, self.plan, "fp64")

    def __call__(self, x):
        return self.bm(x)

    def lanczos_min(self, x0, krylovdim=20, tol=1e-12, maxiter=100, rq_fp64=False):
        x = self.ctx.copy(x0)
        E, info, res = C.c_double(), (C.c_int * 3)(), C.c_double()
        st = self.ctx.lib.gtn_blockmap_lanczos_min(self.bm.h, self.bm64.h if self.bm64 is not self.bm else None,
                                                   C.c_void_p(x.data_ptr()), krylovdim, tol, maxiter,
                                                   1 if rq_fp64 else 0, C.byref(E), info, C.byref(res))
        if st not in (_lib.GTN_OK, _lib.GTN_ERR_NOT_CONVERGED):
            _lib.check(st, self.ctx.h, "blockmap_lanczos_min")
        return E.value, x, dict(restarts=info[0], matvecs=info[1], converged=bool(info[2]), resid=res.value)

    def refine(self, x0, tol=1e-8, max_outer=8, inner_dim=20):
        x = self.ctx.copy(x0)
        E, info, res = C.c_double(), (C.c_int * 4)(), C.c_double()
        st = self.ctx.lib.gtn_blockmap_lanczos_refine(self.bm.h, self.bm64.h, C.c_void_p(x.data_ptr()), inner_dim,
                                                      tol, max_outer, C.byref(E), info, C.byref(res))
        if st not in (_lib.GTN_OK, _lib.GTN_ERR_NOT_CONVERGED):
            _lib.check(st, self.ctx.h, "blockmap_lanczos_refine")
        return E.value, x, dict(corrections=info[0], mixed_matvecs=info[1], fp64_matvecs=info[2],
                                converged=bool(info[3]), resid=res.value)

    def close(self):
        if self.bm64 is not self.bm:
            self.bm64.close()
        self.bm.close()


def dmrg2(psi: U1TTNS, H: U1TTNO, trunc: TruncationScheme | None = None, nsweeps=10, tol=1e-10, krylovdim=20,
          precision="fp64", lanczos_tol=1e-12, maxiter=100, refine="off", refine_tol=1e-8, stats=None):
    """Two-site DMRG on the U(1) network (GroundState.jl:102-143): the sweep schedule of the
    dense dmrg2 (postorder bonds, then reverse), block-sparse maps, Lanczos on the block
    buffer, per-sector split.  Mixed precisions close each sweep with the FP64 Rayleigh
    quotient, or refine the local vectors ("last" / "all") as the dense dmrg2 does."""
    t = psi.topo
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
    trunc = trunc or TruncationScheme()
    cache = U1EnvCache(t)
    bonds = [n for n in t.postorder() if t.parent[n] >= 0]
    sched = [(n, "m") for n in bonds] + [(n, "n") for n in reversed(bonds)]
    energies = []
    for _ in range(nsweeps):
        E = float("nan")
        for step, (n, center_on) in enumerate(sched):
            m = t.parent[n]
            last = step == len(sched) - 1
            move_center(psi, n, cache)
            theta = two_site_tensor(psi, n, m)
            h2 = U1EffH2(cache, psi, H, n, m, prec, theta.T)
            do_refine = prec != _lib.PREC_FP64 and (refine == "all" or (refine == "last" and last))
            E, v, info = h2.lanczos_min(theta.data, krylovdim, lanczos_tol, maxiter,
                                        rq_fp64=prec != _lib.PREC_FP64 and last and not do_refine)
            if do_refine:
                E, v, rinfo = h2.refine(v, tol=refine_tol * max(1.0, abs(E)), inner_dim=krylovdim)
            if stats is not None:
                stats["matvecs"] = stats.get("matvecs", 0) + info["matvecs"]
            h2.close()
            cache.invalidate_edge(n, m)
            split_two_site(psi, U1Tensor(theta.T, v), n, m, trunc, center_on)
        energies.append(float(E))
        if len(energies) >= 2 and abs(energies[-1] - energies[-2]) < tol:
            break
    return psi, energies


def to_dense_state(psi: U1TTNS):
    """Dense host tensors of the network (test helper: the oracle's contraction)."""
    ctx = psi.ctx
    return [t.T.to_dense(t.host(ctx)) for t in psi.tensors]
