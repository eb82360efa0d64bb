"""Controlled bond expansion for one-site TDVP: TDVP1_CBE with the PredictorCBE selector
(lib/GraftEvolution/src/Evolution/cbe.jl:132-148 PredictorCBE, :240-259 TDVP1_CBE,
:308-352 projected factors, :530-589 direction selection and state-preserving splice,
:741-806 the split overrides) on the device.

At the link split of the active endpoint u towards v, active = Q link (QR).  The reference
selects new directions as the leading left singular vectors of the biprojected core
M = Na^H * S link T^T * conj(Np) (Na, Np the complements of Q and of the partner site;
S, T the two halves of the two-site Hamiltonian sandwich, two_site_factor_frame.jl:308-426).
Here the complements are never materialised: with G = S link (ext_u x (edge*w)) and the
partner half T (ext_v x (edge*w)), the core is the product of two tall-skinny factors
G' = (1 - Q Q^H) G and T' = (1 - P P^H) T.  With G' = Q1 R1 and T' = Q2 R2 (thin QR) it is
Q1 (R1 R2^T) Q2^T, so its left singular pairs are Q1 times those of the small R1 R2^T.
Directions with singular value >= spawn_threshold * ||active|| / |dz| are spliced as
U = [Q E], R = U^H active (exact: U R = active).  Every step is a libgrafttn call (FP64).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .contractions import EnvCache, choose_order, eff_h0
from .networks import TTNO, TTNS, absorb_on_leg


@dataclass
class PredictorCBE:
    max_add: int = 32
    spawn_threshold: float = 1e-10
    neigs: int = 2
    krylovdim: int = 4

    def __post_init__(self):
        if self.max_add < 0:
            raise ValueError("PredictorCBE max_add must be nonnegative")
        if self.spawn_threshold < 0:
            raise ValueError("PredictorCBE spawn_threshold must be nonnegative")
        if self.neigs < 1:
            raise ValueError("PredictorCBE neigs must be positive")
        if self.krylovdim < self.neigs:
            raise ValueError("PredictorCBE krylovdim must be at least neigs")


def _opleg(t, u, w):
    return t.nchildren(u) + 2 if t.parent[u] == w else t.childslot(u, w)


def _stateleg(t, u, w):
    return t.nchildren(u) + 1 if t.parent[u] == w else t.childslot(u, w)


def site_half(cache: EnvCache, psi: TTNS, H: TTNO, site, peer, X, k_site):
    """Half of the two-site sandwich at `site` (two_site_factor_frame.jl:308-403).  X is a
    site tensor in the original leg order whose leg k_site faces `peer`.  Result legs:
    (external legs in original order..., edge ket, edge operator)."""
    t, ctx = psi.topo, psi.ctx
    W = H.tensors[site]
    N = X.dim()
    order = [j for j in range(N) if j != k_site] + [k_site]
    out_pos = {raw: j for j, raw in enumerate(order)}
    K = t.nchildren(site)
    xidx, widx = [0] * N, [0] * W.dim()
    labels = [xidx, widx]
    nxt = [0]

    def fresh():
        nxt[0] += 1
        return nxt[0]
    xidx[k_site] = -N
    widx[_opleg(t, site, peer)] = -(N + 1)
    pin = fresh()
    xidx[K] = pin
    widx[K + 1] = pin
    widx[K] = -(out_pos[K] + 1)
    ops = [X.contiguous(), W]
    for w in t.neighbors(site):
        if w == peer:
            continue
        raw = _stateleg(t, site, w)
        kk, oo = fresh(), fresh()
        xidx[raw] = kk
        widx[_opleg(t, site, w)] = oo
        labels.append([kk, oo, -(out_pos[raw] + 1)])
        ops.append(cache.env(psi, H, w, site))
    if t.parent[site] < 0:
        raw = N - 1
        ka, ko = fresh(), fresh()
        xidx[raw] = ka
        widx[-1] = ko
        labels.append([ka, ko, -(out_pos[raw] + 1)])
        ops.append(ctx.upload(np.ones((1, 1, 1))))
    order = choose_order([tuple(o.shape) for o in ops], labels, list(range(len(ops))))
    return ctx.contract(ops, labels, None, order)


def _mat(ctx, A, k):
    """A with leg k moved last, as a (prod others) x dim_k matrix, and the moved shape."""
    perm = [j for j in range(A.dim()) if j != k] + [k]
    t = ctx.permute(A.contiguous(), perm) if k != A.dim() - 1 else A.contiguous()
    return t.reshape(-1, t.shape[-1]), tuple(t.shape)


def _unmat(ctx, M, shape, k):
    """Inverse of _mat: (rows x new_dim) back to the original leg order with leg k new."""
    t = M.reshape(tuple(shape[:-1]) + (M.shape[1],))
    N = t.dim()
    if k == N - 1:
        return t.contiguous()
    inv = list(range(N - 1))
    inv.insert(k, N - 1)
    return ctx.permute(t.contiguous(), inv)


def _matmul(ctx, A, B, conjA=False, transA=False):
    return ctx.matmul(A, B, conjA, transA)


def cbe_split(cache: EnvCache, psi: TTNS, H: TTNO, u, v, dz, maxdim, strategy: PredictorCBE, info=None):
    """PredictorCBE split of the centre u towards its neighbour v.  Returns (U as u's new
    tensor in its original leg order, R with legs (new, edge))."""
    ctx, t = psi.ctx, psi.topo
    if t.parent[u] == v:
        ku, kv = psi.tensors[u].dim() - 1, t.childslot(v, u)
    else:
        ku, kv = t.childslot(u, v), psi.tensors[v].dim() - 1
    act, ashape = _mat(ctx, psi.tensors[u], ku)
    Q, link = ctx.qr(act)
    r = Q.shape[1]
    m = Q.shape[0]
    budget = min(max(0, (maxdim or 1 << 30) - r), strategy.max_add, strategy.neigs)
    E = None
    selected = 0
    if budget > 0 and dz != 0 and r < m:
        par, _ = _mat(ctx, psi.tensors[v], kv)
        n_ext = par.shape[0]
        if par.shape[1] < n_ext:
            Xq = _unmat(ctx, Q, ashape, ku)
            S = site_half(cache, psi, H, u, v, Xq, ku)                  # ext_u..., a, o
            T = site_half(cache, psi, H, v, u, psi.tensors[v], kv)      # ext_v..., b, o
            S = S.reshape(m, S.shape[-2], S.shape[-1])
            T = T.reshape(n_ext, -1)                                     # (ext_v) x (b o)
            G = ctx.contract([S, link], [[-1, 1, -3], [1, -2]]).reshape(m, -1)   # S link: ext_u x (b o)
            # complements: G' = G - Q (Q^H G), T' = T - P (P^H T)
            G = ctx.axpby(-1.0, _matmul(ctx, Q, _matmul(ctx, Q, G, conjA=True, transA=True)), 1.0, G)
            T = ctx.axpby(-1.0, _matmul(ctx, par, _matmul(ctx, par, T, conjA=True, transA=True)), 1.0, T)
            # M = G' T'^T = Q1 (R1 R2^T) Q2^T with G' = Q1 R1 and T' = Q2 R2: the singular
            # pairs come from the small factor directly (accurate to eps * sigma_max; the
            # Gram matrix of M would square the noise floor up to sqrt(eps) * sigma_max)
            Q1, R1 = ctx.qr(G)
            _, R2 = ctx.qr(T)
            Z = ctx.contract([R1.contiguous(), R2.contiguous()], [[-1, 1], [-2, 1]])
            Uz, sig, _, _ = ctx.svd_trunc(Z, maxdim=budget)
            cutoff = strategy.spawn_threshold * max(ctx.norm(act), 1e-300) / abs(dz)
            keep = int(np.sum(sig >= cutoff))
            if keep > 0:
                E = _matmul(ctx, Q1, Uz[:, :keep].contiguous())
                # re-orthogonalise against Q; directions left with no weight outside span(Q)
                # (null columns of a rank-deficient G') are dropped before the QR
                E = ctx.axpby(-1.0, _matmul(ctx, Q, _matmul(ctx, Q, E, conjA=True, transA=True)), 1.0, E)
                norms = np.linalg.norm(ctx.download(E), axis=0)
                good = [j for j in range(keep) if norms[j] > 1e-6]
                if len(good) < keep:
                    E = E[:, good].contiguous() if good else None
                if E is not None:
                    E, _ = ctx.qr(E)
                    E = ctx.axpby(-1.0, _matmul(ctx, Q, _matmul(ctx, Q, E, conjA=True, transA=True)), 1.0, E)
                    E, _ = ctx.qr(E)
                    selected = E.shape[1]
            if info is not None:
                info.update(sigmas=sig.tolist(), cutoff=cutoff)
    Unew = ctx.concat_cols(Q, E) if E is not None else Q
    R = _matmul(ctx, Unew, act, conjA=True, transA=True)                 # (r + k) x edge
    if info is not None:
        info.update(selected=selected, old_rank=r)
    return _unmat(ctx, Unew, ashape, ku), R


class TDVP1_CBE:
    """One-site TDVP whose link splits expand the bond with PredictorCBE (order-2 splitting).
    ``enabled=False`` reproduces TDVP1 exactly (the reference's behavioural contract)."""

    def __init__(self, cbe: PredictorCBE | None = None, maxdim=100, order=2, enabled=True, krylovdim=30,
                 tol=1e-12, precision="fp64"):
        from .solvers import TDVP1
        self.cbe = cbe or PredictorCBE()
        self.maxdim = maxdim
        self.enabled = enabled
        self._base = TDVP1(order=order, krylovdim=krylovdim, tol=tol, precision=precision)
        self._base._evolve_link_and_move = self._evolve_link_and_move
        self.last_info = {}

    @property
    def cache(self):
        return self._base.cache

    def step(self, psi: TTNS, H: TTNO, dz):
        return self._base.step(psi, H, dz)

    def _evolve_link_and_move(self, psi, H, u, v, dz):
        from .solvers import TDVP1
        if not self.enabled:
            return TDVP1._evolve_link_and_move(self._base, psi, H, u, v, dz)
        ctx, t, cache = psi.ctx, psi.topo, self._base.cache
        info = {}
        U, R = cbe_split(cache, psi, H, u, v, dz, self.maxdim, self.cbe, info)
        self.last_info = info
        psi.tensors[u] = U
        cache.invalidate_node(u)
        b = self._base
        if t.parent[u] == v:
            k0 = eff_h0(cache, psi, H, u, v, b.precision)
            C, _ = k0.exponentiate(-dz, R, b.krylovdim, b.tol, hermitian=H.ishermitian)
            k0.close()
            psi.tensors[v] = absorb_on_leg(ctx, psi.tensors[v], C, t.childslot(v, u))
        else:
            Ct = ctx.permute(R.contiguous(), [1, 0])
            k0 = eff_h0(cache, psi, H, v, u, b.precision)
            C, _ = k0.exponentiate(-dz, Ct, b.krylovdim, b.tol, hermitian=H.ishermitian)
            k0.close()
            Av = psi.tensors[v]
            rk = Av.dim()
            lab = [-(j + 1) for j in range(rk - 1)] + [1]
            psi.tensors[v] = ctx.contract([Av, C], [lab, [1, -rk]])
        psi.center = v
        cache.invalidate_node(v)
