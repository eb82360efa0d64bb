"""Device-resident TTNS / TTNO and the gauge operations of the sweep.

Mirrors lib/GraftNetworks/src/Networks/ttns.jl (TTNS, move_center!, _move_center_edge!,
update_tensor!), ttno.jl (TTNO), lib/GraftFoundation/src/Backend/Backend.jl:533-630
(absorb_on_leg, orth_factor_leg) and lib/GraftContractions/src/Contractions/effective.jl:808-876
(two_site_tensor, split_two_site!).  For dense ComplexSpace legs the pivotal twists of the
reference are identities, so the link factors are absorbed as they come out of the QR.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .device import Context, default_context
from .operators import NNHamiltonian, ttno_tensors
from .topology import TreeTopology


@dataclass
class TruncationScheme:
    """(Backend.jl:466-483) maxdim & atol & rtol & discarded-weight truncation."""
    maxdim: int | None = None
    atol: float = 0.0
    rtol: float = 0.0
    discarded_weight: float = 0.0


class TTNO:
    """Operator tensors on the device, legs (children..., P_out, P_in, parent)."""

    def __init__(self, topo: TreeTopology, tensors, ishermitian=True, ctx: Context | None = None):
        self.topo = topo
        self.ctx = ctx or default_context()
        if len(tensors) != topo.nnodes:
            raise ValueError("need one tensor per node")
        self.tensors = [t if hasattr(t, "data_ptr") else self.ctx.upload(t) for t in tensors]
        self.ishermitian = ishermitian

    @classmethod
    def from_hamiltonian(cls, H: NNHamiltonian, ctx=None):
        return cls(H.topo, ttno_tensors(H), ishermitian=H.hermitian, ctx=ctx)


class TTNS:
    """State tensors on the device, legs (children..., phys, parent); one orthogonality centre."""

    def __init__(self, topo: TreeTopology, tensors, center, ctx: Context | None = None):
        self.topo = topo
        self.ctx = ctx or default_context()
        if len(tensors) != topo.nnodes:
            raise ValueError("need one tensor per node")
        self.tensors = [t if hasattr(t, "data_ptr") else self.ctx.upload(t) for t in tensors]
        self.center = center

    def copy(self):
        return TTNS(self.topo, [self.ctx.copy(t) for t in self.tensors], self.center, self.ctx)

    def host_tensors(self):
        return [self.ctx.download(t) for t in self.tensors]

    def bond_dims(self):
        return [int(self.tensors[c].shape[-1]) for c in range(self.topo.nnodes) if self.topo.parent[c] >= 0]

    def norm(self):
        return self.ctx.norm(self.tensors[self.center])


def _labels_except(rank, k, klabel):
    """Output labels -1..-rank with leg k contracted under `klabel`."""
    lab = [-(j + 1) for j in range(rank)]
    lab[k] = klabel
    return lab


def absorb_on_leg(ctx, A, Cm, k):
    """A'[.., y@k, ..] = sum_e C[y, e] A[.., e@k, ..] (Backend.jl:533-543)."""
    labA = _labels_except(A.dim(), k, 1)
    return ctx.contract([A, Cm], [labA, [-(k + 1), 1]])


def left_orth(ctx, A):
    """A[..., e] = sum_y Q[..., y] C[y, e] (QR across all legs but the last)."""
    sh = tuple(A.shape)
    Q, R = ctx.qr(A.reshape(-1, sh[-1]))
    return Q.reshape(sh[:-1] + (Q.shape[1],)), R


def orth_factor_leg(ctx, A, k):
    """(Backend.jl:602-609): QR of A permuted to (others, k); the new bond replaces leg k."""
    N = A.dim()
    perm = [j for j in range(N) if j != k] + [k]
    t = ctx.permute(A, perm)
    Q, C = left_orth(ctx, t)
    inv = list(range(N - 1))
    inv.insert(k, N - 1)
    return ctx.permute(Q, inv), C


def move_center_edge(psi: TTNS, m, on_edge=None):
    """One gauge step of the centre to its neighbour m (ttns.jl:181-203)."""
    ctx, t = psi.ctx, psi.topo
    n = psi.center
    A = psi.tensors[n]
    if t.parent[n] == m:
        Q, C = left_orth(ctx, A)
        psi.tensors[n] = Q
        psi.tensors[m] = absorb_on_leg(ctx, psi.tensors[m], C, t.childslot(m, n))
    else:
        k = t.childslot(n, m)
        Q, C = orth_factor_leg(ctx, A, k)
        psi.tensors[n] = Q
        Am = psi.tensors[m]
        r = Am.dim()
        psi.tensors[m] = ctx.contract([Am, C], [_labels_except(r, r - 1, 1), [-r, 1]])
    psi.center = m
    if on_edge is not None:
        on_edge(n, m)


def move_center(psi: TTNS, target, cache=None):
    """(ttns.jl:126-132) QR sweeps along the path; ``cache`` envs are invalidated."""
    target = psi.topo.nodeindex(target)
    path = psi.topo.path_between(psi.center, target)
    cb = cache.invalidate_edge if cache is not None else None
    for i in range(1, len(path)):
        move_center_edge(psi, path[i], cb)
    return psi


def canonicalize(psi: TTNS, center=None):
    """Leaf->root QR sweep, then a centre move (GraftTestUtils.jl:48-63)."""
    ctx, t = psi.ctx, psi.topo
    for n in t.postorder():
        if n == t.root:
            continue
        Q, C = left_orth(ctx, psi.tensors[n])
        psi.tensors[n] = Q
        p = t.parent[n]
        psi.tensors[p] = absorb_on_leg(ctx, psi.tensors[p], C, t.childslot(p, n))
    psi.center = t.root
    return move_center(psi, t.root if center is None else center)


def normalize(psi: TTNS):
    c = psi.center
    nrm = psi.ctx.norm(psi.tensors[c])
    psi.tensors[c] = psi.ctx.scale(psi.tensors[c], 1.0 / nrm)
    return psi


def random_ttns(rng, topo: TreeTopology, d, bond, center=None, ctx=None):
    """Random canonical TTNS (GraftTestUtils.jl:71-92): complex normal entries with unit
    total variance from a numpy Generator, canonicalised and normalised on the device.
    ``bond`` is an int or a dict child-node -> dim."""
    ctx = ctx or default_context()

    def edim(c):
        return bond if isinstance(bond, int) else bond[c]
    host = []
    for n in range(topo.nnodes):
        shape = [edim(c) for c in topo.children[n]] + [d, 1 if topo.parent[n] < 0 else edim(n)]
        host.append((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0))
    psi = TTNS(topo, host, topo.root, ctx)
    canonicalize(psi, center)
    return normalize(psi)


def two_site_tensor(psi: TTNS, n, m, precision=None):
    """Θ: A_n's codomain legs, then A_m's legs except slot k (effective.jl:827-843).
    ``precision``: GTN_PREC_FP64 (default) or GTN_PREC_FP64E for the contraction."""
    t = psi.topo
    if t.parent[n] != m:
        raise ValueError("two_site_tensor: m must be the parent of n")
    k = t.childslot(m, n)
    A, B = psi.tensors[n], psi.tensors[m]
    pn = A.dim() - 1
    labA = [-(j + 1) for j in range(pn)] + [1]
    labB = []
    pos = pn
    for j in range(B.dim()):
        if j == k:
            labB.append(1)
        else:
            pos += 1
            labB.append(-pos)
    if precision is None:
        return psi.ctx.contract([A, B], [labA, labB])
    return psi.ctx.contract([A, B], [labA, labB], precision=precision)


def split_two_site(psi: TTNS, theta, n, m, trunc: TruncationScheme | None = None, center_on="n"):
    """Truncated SVD of Θ back into A_n, A_m (effective.jl:852-876); returns the
    discarded 2-norm."""
    ctx, t = psi.ctx, psi.topo
    trunc = trunc or TruncationScheme()
    k = t.childslot(m, n)
    pn = psi.tensors[n].dim() - 1
    sh = tuple(theta.shape)
    rows = int(np.prod(sh[:pn]))
    U, S, Vh, disc = ctx.svd_trunc(theta.reshape(rows, -1), trunc.maxdim, trunc.atol, trunc.rtol,
                                   trunc.discarded_weight)
    r = len(S)
    if center_on == "n":
        ctx.diag_scale(U, S, side=0)
    else:
        ctx.diag_scale(Vh, S, side=1)
    psi.tensors[n] = U.reshape(sh[:pn] + (r,))
    Rm = Vh.reshape((r,) + sh[pn:])
    nm = Rm.dim()
    perm = list(range(1, nm))
    perm.insert(k, 0)
    psi.tensors[m] = ctx.permute(Rm.contiguous(), perm) if k != 0 else Rm.contiguous()
    psi.center = n if center_on == "n" else m
    return disc
