"""Abelian U(1) block-sparse tensors and the planner of block-sparse effective maps.

A leg carries U(1) charge sectors (charge -> degeneracy) and an arrow sign (+1 codomain,
-1 domain; TensorKit's ``TensorMap`` codomain <- domain).  A tensor stores one dense
row-major block for every charge combination with ``sum_i sign_i q_i == qtot``, all blocks
contiguous in one buffer in lexicographic charge order.  This is TensorKit's abelian
unique-fusion block structure (``blocks(t)``) written out per sector combination.

The planner lowers an ncon label graph (the same h1/h2/h0/env graphs as the dense path,
lib/GraftContractions/src/Contractions/effective.jl:627-1034) over block tensors into
libgrafttn block-map descriptors: per pair step one GEMM problem per coupled charge q of
the contracted legs (C_q = A_q B_q^T, TensorKit's per-sector block mul!,
lib/GraftFoundation/src/Backend/Backend.jl:243-261,309-368) plus one gather per block of the
running tensor.  Static operands are assembled into B_q once, on the host.
"""
from __future__ import annotations

import ctypes as C
import itertools
import math

import numpy as np

from . import _lib
from ._lib import check, i64_array, int_array, ptr_array

BUF_X, BUF_Y, BUF_T0, BUF_T1 = 0, 1, 2, 3


class U1Leg:
    def __init__(self, sectors, sign=1):
        self.charges = sorted(int(q) for q in sectors)
        self.dims = [int(sectors[q]) for q in self.charges]
        self.sign = int(sign)
        self.offset = {}
        o = 0
        for q, d in zip(self.charges, self.dims):
            self.offset[q] = o
            o += d
        self.total = o

    def sectors(self):
        return dict(zip(self.charges, self.dims))

    def dim(self, q):
        return self.dims[self.charges.index(q)]

    def flipped(self):
        return U1Leg(self.sectors(), -self.sign)

    def __repr__(self):
        return f"U1Leg({self.sectors()}, sign={self.sign})"


class BlockTensor:
    """Block structure (no data): every allowed charge combination, row-major blocks."""

    def __init__(self, legs, qtot=0):
        self.legs = list(legs)
        self.qtot = int(qtot)
        self.blocks = []          # (charges, shape, offset)
        self.index = {}
        off = 0
        for qs in itertools.product(*[l.charges for l in self.legs]):
            if sum(l.sign * q for l, q in zip(self.legs, qs)) != self.qtot:
                continue
            shape = tuple(l.dim(q) for l, q in zip(self.legs, qs))
            self.index[qs] = len(self.blocks)
            self.blocks.append((qs, shape, off))
            off += int(np.prod(shape))
        self.size = off

    @property
    def dense_shape(self):
        return tuple(l.total for l in self.legs)

    def random(self, rng):
        return (rng.standard_normal(self.size) + 1j * rng.standard_normal(self.size)) / np.sqrt(2)

    def to_dense(self, data):
        out = np.zeros(self.dense_shape, dtype=np.complex128)
        for qs, shape, off in self.blocks:
            sl = tuple(slice(l.offset[q], l.offset[q] + d) for l, q, d in zip(self.legs, qs, shape))
            out[sl] = np.asarray(data[off: off + int(np.prod(shape))]).reshape(shape)
        return out

    def from_dense(self, dense, check_zero=True):
        data = np.zeros(self.size, dtype=np.complex128)
        mask = np.zeros(self.dense_shape, dtype=bool)
        for qs, shape, off in self.blocks:
            sl = tuple(slice(l.offset[q], l.offset[q] + d) for l, q, d in zip(self.legs, qs, shape))
            data[off: off + int(np.prod(shape))] = dense[sl].reshape(-1)
            mask[sl] = True
        if check_zero and np.abs(dense[~mask]).max(initial=0.0) > 1e-12:
            raise ValueError("dense tensor has weight outside the allowed charge blocks")
        return data


def _groups(dims, strides):
    """Index groups (outer..inner) over legs, merging contiguous neighbours, skipping dim 1."""
    gd, gs = [], []
    for d, s in zip(dims, strides):
        if d == 1:
            continue
        if gd and gs[-1] == s * d:
            gd[-1] *= d
            gs[-1] = s
        else:
            gd.append(d)
            gs.append(s)
    if len(gd) > 8:
        raise NotImplementedError("more than 8 non-contiguous leg groups")
    return gd, gs


def _fill_gather(g, dims_m, str_m, dims_k, str_k):
    md, ms = _groups(dims_m, str_m)
    kd, ks = _groups(dims_k, str_k)
    g.ng_m, g.ng_k = len(md), len(kd)
    for i, (d, s) in enumerate(zip(md, ms)):
        g.m_dim[i], g.m_str[i] = d, s
    for i, (d, s) in enumerate(zip(kd, ks)):
        g.k_dim[i], g.k_str[i] = d, s


def _row_major(dims):
    st = [1] * len(dims)
    for i in range(len(dims) - 2, -1, -1):
        st[i] = st[i + 1] * dims[i + 1]
    return st


def contract_statics(a, b):
    """Host contraction of two block-sparse statics (BlockTensor, labels, data) over their
    shared labels; the result keeps the unshared legs (a's, then b's) and every block
    allowed by the charge rule (zero where no block pair contributes)."""
    Ta, la, da = a
    Tb, lb, db = b
    shared = [l for l in la if l > 0 and l in lb]
    ia = [la.index(l) for l in shared]
    ib = [lb.index(l) for l in shared]
    fa = [i for i in range(len(la)) if i not in ia]
    fb = [i for i in range(len(lb)) if i not in ib]
    legs = [Ta.legs[i] for i in fa] + [Tb.legs[i] for i in fb]
    out = BlockTensor(legs, Ta.qtot + Tb.qtot)
    byk = {}
    for qs, shape, off in Tb.blocks:
        byk.setdefault(tuple(qs[i] for i in ib), []).append((qs, np.asarray(db[off: off + int(np.prod(shape))]).reshape(shape)))
    acc = {}
    for qs, shape, off in Ta.blocks:
        blk = np.asarray(da[off: off + int(np.prod(shape))]).reshape(shape)
        for qb, bb in byk.get(tuple(qs[i] for i in ia), []):
            qc = tuple(qs[i] for i in fa) + tuple(qb[i] for i in fb)
            c = np.tensordot(blk, bb, axes=(ia, ib))
            acc[qc] = acc[qc] + c if qc in acc else c
    data = np.zeros(out.size, dtype=np.complex128)
    for qs, shape, off in out.blocks:
        if qs in acc:
            data[off: off + int(np.prod(shape))] = acc[qs].reshape(-1)
    return out, [la[i] for i in fa] + [lb[i] for i in fb], data


def _dense_step_time(M, K, N):
    """Time model of one pair step on the mixed path (the plan compiler's model)."""
    flops = 8.0 * M * K * N
    if K <= 64:
        return 5e-6 + (M * K + M * N) * 8 / 5e12 + flops / 15e12
    Kp = math.ceil(K / 32) * 32
    return 5e-6 + flops / 200e12 + (M * K * 8 + M * 2 * Kp * 6 + M * N * 8) / 5e12


def choose_groups(x_labels, x_dims, statics, order, max_combined=1 << 20):
    """Partition the absorbed statics into consecutive groups (pre-contracted on the host)
    minimising the modelled chain time on the dense shapes; returns lists of static
    indices (1-based operand numbers)."""
    seq = list(order[1:])
    dims = {}
    for l, d in zip(x_labels, x_dims):
        dims[l] = d
    for T, lab, _ in statics:
        for l, leg in zip(lab, T.legs):
            dims[l] = leg.total

    def ext(group):
        cnt = {}
        for j in group:
            for l in statics[j - 1][1]:
                cnt[l] = cnt.get(l, 0) + 1
        return [l for j in group for l in statics[j - 1][1] if not (l > 0 and cnt[l] == 2)]

    def chain_time(groups):
        LT = list(x_labels)
        t = 0.0
        for g in groups:
            LS = ext(g) if len(g) > 1 else list(statics[g[0] - 1][1])
            sh = [l for l in LT if l > 0 and l in LS]
            M = math.prod(dims[l] for l in LT if l not in sh)
            K = math.prod(dims[l] for l in sh)
            N = math.prod(dims[l] for l in LS if l not in sh)
            t += _dense_step_time(M, K, N)
            LT = [l for l in LS if l not in sh] + [l for l in LT if l not in sh]
        return t
    best = [[j] for j in seq]
    best_t = chain_time(best)
    ns = len(seq)
    for mask in range(1 << max(ns - 1, 0)):
        groups, cur = [], []
        for i, j in enumerate(seq):
            cur.append(j)
            if i == ns - 1 or (mask >> i) & 1:
                groups.append(cur)
                cur = []
        if any(len(g) > 1 and math.prod(dims[l] for l in ext(g)) > max_combined for g in groups):
            continue
        t = chain_time(groups)
        if t < 0.9 * best_t:
            best, best_t = groups, t
    return best


class BlockPlan:
    """Descriptors of a block-sparse map application (host side, precision independent)."""

    def __init__(self, x: BlockTensor, x_labels, statics, order, group=True):
        """statics: list (operand order 1..) of (BlockTensor, labels, host data 1-D).  With
        ``group`` small consecutive statics are pre-contracted on the host first."""
        if group and len(order) > 2:
            groups = choose_groups(x_labels, [l.total for l in x.legs], statics, order)
            merged = []
            for g in groups:
                acc = statics[g[0] - 1]
                for j in g[1:]:
                    acc = contract_statics(acc, statics[j - 1])
                merged.append(acc)
            statics = merged
            order = [0] + list(range(1, len(merged) + 1))
            self.groups = groups
        else:
            self.groups = [[j] for j in order[1:]]
        self.x = x
        self.steps = []           # list of (gathers, gemms)
        self.B = []               # host B_q matrices
        self.flops = 0.0
        legs = {l: leg for l, leg in zip(x_labels, x.legs)}
        # running blocks: charges per label -> (buf, offset, dims, strides)
        LT = list(x_labels)
        blocks = {qs: (BUF_X, off, shape, tuple(_row_major(shape))) for qs, shape, off in x.blocks}
        buf_elems = {BUF_T0: 1, BUF_T1: 1}
        for si, j in enumerate(order[1:]):
            S, LS, Sdata = statics[j - 1]
            slegs = dict(zip(LS, S.legs))
            shared = [l for l in LT if l > 0 and l in LS]
            freeT = [l for l in LT if l not in shared]
            freeS = [l for l in LS if l not in shared]
            for l in shared:
                if slegs[l].sign != -legs[l].sign or slegs[l].charges != legs[l].charges or slegs[l].dims != legs[l].dims:
                    raise ValueError(f"label {l}: legs do not match (sectors or arrows)")
            tpos = {l: i for i, l in enumerate(LT)}
            spos = {l: i for i, l in enumerate(LS)}

            def coupled(charges_by_label):
                return sum(legs[l].sign * charges_by_label[l] for l in shared)
            # T blocks by coupled charge
            tb = {}
            for qs, info in blocks.items():
                by = dict(zip(LT, qs))
                f = tuple(by[l] for l in freeT)
                k = tuple(by[l] for l in shared)
                tb.setdefault(coupled(by), {})[(f, k)] = info
            sb = {}
            for qs, shape, off in S.blocks:
                by = dict(zip(LS, qs))
                g = tuple(by[l] for l in freeS)
                k = tuple(by[l] for l in shared)
                sb.setdefault(coupled(by), {})[(g, k)] = (shape, off)
            outbuf = BUF_T0 if si % 2 == 0 else BUF_T1
            gathers, gemms = [], []
            new_blocks = {}
            c_off = 0

            def size_of(labels, charges):
                return int(np.prod([legs_all[l].dim(q) for l, q in zip(labels, charges)] or [1]))
            legs_all = dict(legs)
            legs_all.update(slegs)
            for q in sorted(set(tb) | set(sb)):
                T_q, S_q = tb.get(q, {}), sb.get(q, {})
                F = sorted({f for f, _ in T_q})
                G = sorted({g for g, _ in S_q})
                Kset = sorted({k for _, k in T_q} & {k for _, k in S_q})
                if not F or not G or not Kset:
                    continue
                foff, o = {}, 0
                for f in F:
                    foff[f] = o
                    o += size_of(freeT, f)
                Mq = o
                koff, o = {}, 0
                for k in Kset:
                    koff[k] = o
                    o += size_of(shared, k)
                Kq = o
                goff, o = {}, 0
                for g in G:
                    goff[g] = o
                    o += size_of(freeS, g)
                Nq = o
                pidx = len(gemms)
                # B_q: static blocks permuted to (freeS legs, shared legs in T order)
                Bq = np.zeros((Nq, Kq), dtype=np.complex128)
                perm = [spos[l] for l in freeS] + [spos[l] for l in shared]
                for (g, k), (shape, off) in S_q.items():
                    if k not in koff:
                        continue
                    blk = np.asarray(Sdata[off: off + int(np.prod(shape))]).reshape(shape).transpose(perm)
                    blk = blk.reshape(size_of(freeS, g), size_of(shared, k))
                    Bq[goff[g]: goff[g] + blk.shape[0], koff[k]: koff[k] + blk.shape[1]] = blk
                bidx = len(self.B)
                self.B.append(Bq)
                gm = _lib.BlockGemm()
                gm.b_index, gm.c_buf, gm.c_off, gm.M, gm.N, gm.K = bidx, outbuf, c_off, Mq, Nq, Kq
                gemms.append(gm)
                self.flops += 8.0 * Mq * Nq * Kq
                # gathers: every (f, k) sub-rectangle of A_q
                for f in F:
                    for k in Kset:
                        ga = _lib.BlockGather()
                        ga.dst_index = pidx
                        ga.row_off, ga.col_off = foff[f], koff[k]
                        ga.M, ga.K, ga.Kw = size_of(freeT, f), size_of(shared, k), size_of(shared, k)
                        info = T_q.get((f, k))
                        if info is None:         # an absent (zero) block: write zeros
                            ga.src_buf, ga.src_off, ga.K = BUF_X, 0, 0
                            ga.ng_m = ga.ng_k = 0
                        else:
                            buf, off, dims, strides = info
                            ga.src_buf, ga.src_off = buf, off
                            _fill_gather(ga, [dims[tpos[l]] for l in freeT], [strides[tpos[l]] for l in freeT],
                                         [dims[tpos[l]] for l in shared], [strides[tpos[l]] for l in shared])
                        gathers.append(ga)
                # output blocks of C_q [N_q][M_q]: (g, f) with legs freeS + freeT
                for g in G:
                    gd = [legs_all[l].dim(c) for l, c in zip(freeS, g)]
                    gs = [s * Mq for s in _row_major(gd)]
                    for f in F:
                        fd = [legs_all[l].dim(c) for l, c in zip(freeT, f)]
                        fs = _row_major(fd)
                        new_blocks[g + f] = (outbuf, c_off + goff[g] * Mq + foff[f], tuple(gd + fd), tuple(gs + fs))
                c_off += Nq * Mq
            buf_elems[outbuf] = max(buf_elems[outbuf], c_off)
            self.steps.append((gathers, gemms))
            LT = freeS + freeT
            legs = {l: legs_all[l] for l in LT}
            blocks = new_blocks
        if any(l > 0 for l in LT):
            raise ValueError("unresolved labels after the last step")
        # output: y has legs -1, -2, ... with x's block structure
        R = len(LT)
        ylegs = [legs[-(k + 1)] for k in range(R)]
        self.y = BlockTensor(ylegs, x.qtot)
        ypos = [LT.index(-(k + 1)) for k in range(R)]
        self.final = []
        for qs, shape, off in self.y.blocks:
            tq = [None] * R
            for k in range(R):
                tq[ypos[k]] = qs[k]
            info = blocks.get(tuple(tq))
            ga = _lib.BlockGather()
            ga.row_off = off
            ga.M = int(np.prod(shape[:-1])) if R > 1 else 1
            ga.K = shape[-1] if R else 1
            ga.Kw = ga.K
            ga.ld = ga.K
            if info is None:
                ga.src_buf, ga.src_off, ga.K = BUF_X, 0, 0
            else:
                buf, boff, dims, strides = info
                ga.src_buf, ga.src_off = buf, boff
                _fill_gather(ga, [dims[ypos[k]] for k in range(R - 1)], [strides[ypos[k]] for k in range(R - 1)],
                             [dims[ypos[R - 1]]], [strides[ypos[R - 1]]])
            self.final.append(ga)
        self.buffer_elems = [x.size, self.y.size, buf_elems[BUF_T0], buf_elems[BUF_T1]]


def execute_numpy(plan: BlockPlan, x):
    """Run the descriptors on the host (the planner's own check, independent of the GPU)."""
    bufs = {BUF_X: np.asarray(x, dtype=np.complex128), BUF_T0: np.zeros(plan.buffer_elems[2], np.complex128),
            BUF_T1: np.zeros(plan.buffer_elems[3], np.complex128)}

    def gather_block(g):
        rows = []
        m_idx = [np.arange(int(g.m_dim[i])) * int(g.m_str[i]) for i in range(g.ng_m)]
        k_idx = [np.arange(int(g.k_dim[i])) * int(g.k_str[i]) for i in range(g.ng_k)]
        mo = np.zeros(1, dtype=np.int64)
        for a in m_idx:
            mo = (mo[:, None] + a[None, :]).reshape(-1)
        ko = np.zeros(1, dtype=np.int64)
        for a in k_idx:
            ko = (ko[:, None] + a[None, :]).reshape(-1)
        del rows
        if g.K == 0:
            return np.zeros((int(g.M), int(g.Kw)), np.complex128)
        return bufs[g.src_buf][int(g.src_off) + mo[:, None] + ko[None, :]]
    for gathers, gemms in plan.steps:
        A = [np.zeros((int(gm.M), int(gm.K)), np.complex128) for gm in gemms]
        for g in gathers:
            blk = gather_block(g)
            A[g.dst_index][int(g.row_off): int(g.row_off) + int(g.M), int(g.col_off): int(g.col_off) + int(g.Kw)] = blk
        for gm, a in zip(gemms, A):
            Cq = plan.B[gm.b_index] @ a.T           # [N][M]
            bufs[gm.c_buf][int(gm.c_off): int(gm.c_off) + Cq.size] = Cq.reshape(-1)
    y = np.zeros(plan.buffer_elems[1], np.complex128)
    for g in plan.final:
        blk = gather_block(g)
        y[int(g.row_off): int(g.row_off) + blk.size] = blk.reshape(-1)
    return y


class BlockEffectiveMap:
    """A block-sparse map compiled into libgrafttn (grouped launches per step, optional
    CUDA-graph replay)."""

    def __init__(self, ctx, plan: BlockPlan, precision="bf16x6", graph=False):
        self.ctx = ctx
        self.plan = plan
        self.precision = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
        dB = [ctx.upload(b) for b in plan.B]
        steps = plan.steps
        g_all = [g for gs, _ in steps for g in gs]
        m_all = [m for _, ms in steps for m in ms]
        GA = (_lib.BlockGather * max(len(g_all), 1))(*g_all)
        MA = (_lib.BlockGemm * max(len(m_all), 1))(*m_all)
        FA = (_lib.BlockGather * max(len(plan.final), 1))(*plan.final)
        nk = [v for b in plan.B for v in b.shape]
        h = C.c_void_p()
        check(ctx.lib.gtn_blockmap_create(ctx.h, len(steps), int_array([len(gs) for gs, _ in steps]),
                                          int_array([len(ms) for _, ms in steps]), C.cast(GA, C.c_void_p),
                                          C.cast(MA, C.c_void_p), len(plan.final), C.cast(FA, C.c_void_p), len(dB),
                                          ptr_array([b.data_ptr() for b in dB]), i64_array(nk),
                                          i64_array(plan.buffer_elems), self.precision, float(plan.flops), C.byref(h)),
              ctx.h, "blockmap_create")
        self.h = h
        self.flops = plan.flops
        self.n_problems = len(m_all)
        ctx.sync()  # statics copied: the uploads may go
        if graph:
            check(ctx.lib.gtn_blockmap_set_graph(self.h, 1), ctx.h, "blockmap_set_graph")

    def apply_into(self, x, y):
        check(self.ctx.lib.gtn_blockmap_apply(self.h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr())), self.ctx.h,
              "blockmap_apply")
        return y

    def __call__(self, x):
        return self.apply_into(x, self.ctx.empty((self.plan.y.size,)))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gtn_blockmap_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------------------
# U(1) Heisenberg structures (spin-1/2, charge = number of up spins)
# ---------------------------------------------------------------------------------------

def u1_heisenberg_terms():
    """XX + YY + ZZ = 2 (S+ S- + S- S+) + ZZ with S+ = [[0,1],[0,0]] (charge -1 at its site),
    S- = [[0,0],[1,0]] (charge +1); basis index = charge."""
    from .operators import spin_ops
    S = spin_ops()
    return [(2.0, S["Sp"], S["Sm"]), (2.0, S["Sm"], S["Sp"]), (1.0, S["Z"], S["Z"])]


# charges of the operator bond states of ttno_tensors for u1_heisenberg_terms:
# 0 vacuum, 1 finished, 2 S+ opened (-1), 3 S- opened (+1), 4 Z opened (0)
OP_BOND_CHARGES = [0, 0, -1, 1, 0]


def op_leg(sign):
    """Operator bond leg sorted by charge, and the permutation dense index -> sorted position."""
    order = sorted(range(len(OP_BOND_CHARGES)), key=lambda i: (OP_BOND_CHARGES[i], i))
    sectors = {}
    for i in order:
        sectors[OP_BOND_CHARGES[i]] = sectors.get(OP_BOND_CHARGES[i], 0) + 1
    return U1Leg(sectors, sign), order


def binomial_sectors(nsites, total, lo=4, hi=256):
    """Charge sectors 0..nsites of a subtree bond with dims following binomial(nsites, q),
    scaled to `total`, each clipped to [lo, hi] (exact when the full space fits)."""
    full = {q: math.comb(nsites, q) for q in range(nsites + 1)}
    if sum(full.values()) <= total:
        return full
    raw = np.array([math.comb(nsites, q) for q in range(nsites + 1)], dtype=float)
    dims = np.clip(np.round(raw / raw.sum() * total), lo, hi).astype(int)
    for _ in range(200):
        diff = total - int(dims.sum())
        if diff == 0:
            break
        order = np.argsort(-raw)
        for i in order:
            if diff > 0 and dims[i] < hi:
                dims[i] += 1
                diff -= 1
            elif diff < 0 and dims[i] > lo:
                dims[i] -= 1
                diff += 1
            if diff == 0:
                break
    return {q: int(d) for q, d in enumerate(dims) if d > 0}
