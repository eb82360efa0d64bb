"""Device-resident scalar contractions and TTNO application: ``inner`` and the local
``expect`` of lib/GraftContractions/src/Contractions/expectation.jl:13-80, and the exact
(untruncated) TTNO-TTNS product of lib/GraftNetworks/src/Networks/apply.jl.

Every contraction is a libgrafttn call (FP64); the host only walks the tree.
"""
from __future__ import annotations

from .device import Context
from .networks import TTNO, TTNS, move_center


def inner(phi: TTNS, psi: TTNS):
    """<phi|psi> (phi conjugated): overlap environments from the leaves to the root
    (expectation.jl:13-25; the operator-free environment of envcache.jl)."""
    if phi.topo is not psi.topo and phi.topo != psi.topo:
        raise ValueError("inner: mismatched topologies")
    t, ctx = psi.topo, psi.ctx
    env = {}
    for u in t.postorder():
        A, B = psi.tensors[u].contiguous(), phi.tensors[u].contiguous()
        N = A.dim()
        K = t.nchildren(u)
        aidx, bidx = [0] * N, [0] * N
        ops, labels, conj = [A], [aidx], [False]
        nxt = 1
        for j, c in enumerate(t.children[u]):
            ka, kb = nxt, nxt + 1
            nxt += 2
            aidx[j], bidx[j] = ka, kb
            ops.append(env.pop(c))
            labels.append([ka, kb])
            conj.append(False)
        aidx[K] = bidx[K] = nxt
        aidx[K + 1], bidx[K + 1] = -1, -2
        ops.append(B)
        labels.append(bidx)
        conj.append(True)
        env[u] = ctx.contract(ops, labels, conj)
    root = env[t.root]
    return complex(Context.download(root).reshape(-1)[0])


def expect_local(psi: TTNS, op, site) -> complex:
    """<psi|op_site|psi> / <psi|psi> for a one-site operator ``op`` (P_out x P_in) on node
    ``site`` (an index or a topology id), on a gauge-moved copy (expectation.jl:64-80)."""
    t = psi.topo
    n = t.index[site] if not isinstance(site, int) else site
    work = psi if psi.center == n else psi.copy()
    if work.center != n:
        move_center(work, n)
    ctx = work.ctx
    A = work.tensors[n].contiguous()
    N = A.dim()
    p = t.nchildren(n)
    lab = [-(j + 1) for j in range(N)]
    lab[p] = 1
    opd = ctx.upload(op)
    Ap = ctx.contract([A, opd], [lab, [-(p + 1), 1]])
    return ctx.dot(A, Ap) / ctx.dot(A, A)


def apply_ttno(H: TTNO, psi: TTNS) -> TTNS:
    """H|psi> exactly: at every node the site tensor absorbs the TTNO tensor over the
    physical leg, and each bond becomes the fused (state, operator) pair, state index
    major (bond dimension D * w, no truncation; apply.jl's exact path)."""
    t, ctx = psi.topo, psi.ctx
    out = []
    for u in range(t.nnodes):
        A, W = psi.tensors[u].contiguous(), H.tensors[u].contiguous()
        K = t.nchildren(u)
        aidx = [0] * A.dim()
        widx = [0] * W.dim()
        for j in range(K):
            aidx[j], widx[j] = -(2 * j + 1), -(2 * j + 2)
        widx[K] = -(2 * K + 1)          # P_out
        aidx[K] = widx[K + 1] = 1       # phys = P_in
        aidx[K + 1], widx[K + 2] = -(2 * K + 2), -(2 * K + 3)
        T = ctx.contract([A, W], [aidx, widx])
        shape = [A.shape[j] * W.shape[j] for j in range(K)] + [W.shape[K], A.shape[K + 1] * W.shape[K + 2]]
        out.append(T.reshape(shape).contiguous())
    res = psi.copy()
    res.tensors = out
    return res
