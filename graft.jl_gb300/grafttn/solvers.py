"""Sweep drivers: dmrg2! (lib/GraftGroundState/src/GroundState/GroundState.jl:102-143) and
TDVP1 (lib/GraftEvolution/src/Evolution/tdvp.jl:171-301) on the device-resident network.

The host keeps only the sweep order and the gauge bookkeeping; every tensor operation
(QR, SVD, environment builds, the effective maps and their Krylov solves) runs through
libgrafttn on the GPU.
"""
from __future__ import annotations

import time

from . import _lib
from .expansion import check_scheme, factorized_rangefinder_enrichment, predictor_basis
from .contractions import EnvCache, eff_h0, eff_h1, eff_h2
from .networks import (TTNO, TTNS, TruncationScheme, absorb_on_leg, left_orth, move_center,
                       orth_factor_leg, split_two_site, two_site_tensor)


def refine_local(h2, E, v, refine_tol, max_outer=8, inner_dim=20, stats=None):
    """FP64 iterative refinement of a local eigenvector of a mixed-precision map
    (gtn_lanczos_refine): FP64 residuals, mixed-precision corrections.  The tolerance is
    relative to the energy: |H v - E v| <= refine_tol * max(1, |E|).  Returns (E, v)."""
    E2, v2, info = h2.refine(v, tol=refine_tol * max(1.0, abs(E)), max_outer=max_outer, inner_dim=inner_dim)
    if stats is not None:
        stats["refine_fp64_matvecs"] = stats.get("refine_fp64_matvecs", 0) + info["fp64_matvecs"]
        stats["refine_mixed_matvecs"] = stats.get("refine_mixed_matvecs", 0) + info["mixed_matvecs"]
    return E2, v2


def dmrg2(psi: TTNS, H: TTNO, trunc: TruncationScheme | None = None, nsweeps=10, tol=1e-10,
          krylovdim=20, precision="fp64", rq_fp64=None, lanczos_tol=1e-12, maxiter=100,
          verbose=False, stats=None, refine="off", refine_tol=1e-8, fp64e=False):
    """Two-site DMRG; returns (psi, energies per sweep).  ``precision`` selects the map
    arithmetic.  With a mixed mode the energy that closes each sweep (the one returned and
    used for the convergence test) is the FP64 Rayleigh quotient of the last local
    eigenvector (``rq_fp64`` defaults to True for mixed modes); the other local solves keep
    their mixed-precision Ritz values, which nothing downstream reads.

    ``refine`` ("off", "last" or "all"; mixed modes only) refines the local eigenvectors of
    the sweep-closing solve or of every solve to FP64 accuracy (refine_local): the FP64
    residual |H v - E v| is brought below refine_tol * max(1, |E|), and the energy is the
    FP64 Rayleigh quotient of the refined vector.

    ``fp64e`` runs the FP64-accurate work of a mixed sweep on the tensor cores: environment
    updates and two-site merges in GTN_PREC_FP64E, the Gram-matrix products of the truncated
    SVD (gtn_ctx_set_linalg_precision), and the Rayleigh quotients and refinement residuals
    through an FP64E twin of each local map (gtn_map_set_fp64)."""
    if not H.ishermitian:
        raise ValueError("dmrg2: DMRG requires ishermitian(H) == true")
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
    if rq_fp64 is None:
        rq_fp64 = prec != _lib.PREC_FP64
    trunc = trunc or TruncationScheme()
    t = psi.topo
    use_e = fp64e and prec != _lib.PREC_FP64
    cache = EnvCache(t, precision="fp64e" if use_e else "fp64")
    merge_prec = _lib.PREC_FP64E if use_e else _lib.PREC_FP64
    old_linalg = psi.ctx.linalg_precision(_lib.PREC_FP64E if use_e else None)
    try:
        return _dmrg2_sweeps(psi, H, trunc, nsweeps, tol, krylovdim, prec, rq_fp64, lanczos_tol, maxiter,
                             verbose, stats, refine, refine_tol, use_e, cache, merge_prec)
    finally:
        psi.ctx.linalg_precision(old_linalg)


def _dmrg2_sweeps(psi, H, trunc, nsweeps, tol, krylovdim, prec, rq_fp64, lanczos_tol, maxiter, verbose, stats,
                  refine, refine_tol, use_e, cache, merge_prec):
    t = psi.topo
    energies = []
    bonds = [n for n in t.postorder() if t.parent[n] >= 0]
    sched = [(n, "m") for n in bonds] + [(n, "n") for n in reversed(bonds)]
    timing = stats is not None and stats.get("timing", False)

    def mark(key, t_start):
        if timing:
            psi.ctx.sync()
            stats[key] = stats.get(key, 0.0) + time.perf_counter() - t_start
        return time.perf_counter()
    for sweep in range(nsweeps):
        E = float("nan")
        t0 = time.perf_counter()
        for step, (n, center_on) in enumerate(sched):
            if stats is not None and stats.get("max_steps") is not None and step >= stats["max_steps"]:
                break
            m = t.parent[n]
            tt = time.perf_counter()
            move_center(psi, n, cache)
            tt = mark("t_gauge", tt)
            theta = two_site_tensor(psi, n, m, precision=merge_prec)
            tt = mark("t_merge", tt)
            h2 = eff_h2(cache, psi, H, n, m, prec)
            h2e = None
            last = step == len(sched) - 1 or (stats is not None and stats.get("max_steps") is not None
                                               and step == stats["max_steps"] - 1)
            do_refine = prec != _lib.PREC_FP64 and (refine == "all" or (refine == "last" and last))
            if use_e and (do_refine or (rq_fp64 and last)):
                h2e = eff_h2(cache, psi, H, n, m, _lib.PREC_FP64E)
                h2.set_fp64_map(h2e)
            tt = mark("t_env_and_map", tt)
            E, v, info = h2.lanczos_min(theta, krylovdim=krylovdim, tol=lanczos_tol, maxiter=maxiter,
                                        rq_fp64=rq_fp64 and last and not do_refine)
            tt = mark("t_lanczos", tt)
            if do_refine:
                E, v = refine_local(h2, E, v, refine_tol, inner_dim=krylovdim, stats=stats)
                tt = mark("t_refine", tt)
            if stats is not None:
                stats["matvecs"] = stats.get("matvecs", 0) + info["matvecs"]
                stats["steps"] = stats.get("steps", 0) + 1
                stats.setdefault("energies", []).append(E)
            h2.close()
            if h2e is not None:
                h2e.close()
            cache.invalidate_edge(n, m)
            split_two_site(psi, v, n, m, trunc, center_on)
            tt = mark("t_split", tt)
        energies.append(float(E))
        if verbose:
            print(f"dmrg2 sweep {sweep + 1}: E = {E:.15f}  ({time.perf_counter() - t0:.3f} s)")
        if len(energies) >= 2 and abs(energies[-1] - energies[-2]) < tol:
            break
    return psi, energies


def dmrg1(psi: TTNS, H: TTNO, nsweeps=10, tol=1e-10, krylovdim=20, precision="fp64", rq_fp64=None,
          lanczos_tol=1e-12, maxiter=100, stats=None):
    """Single-site DMRG (GroundState.jl:51-84): bond dimensions stay those of psi; postorder
    then reverse postorder, the local ground state of eff_h1 at every node; returns
    (psi, energies per sweep), stopping early when the energy change drops below tol."""
    if not H.ishermitian:
        raise ValueError("dmrg1: DMRG requires ishermitian(H) == true")
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
    if rq_fp64 is None:
        rq_fp64 = prec != _lib.PREC_FP64
    t = psi.topo
    cache = EnvCache(t)
    order = t.postorder()
    energies = []
    for sweep in range(nsweeps):
        E = float("nan")
        seq = list(order) + list(reversed(order))
        for i, n in enumerate(seq):
            move_center(psi, n, cache)
            h1 = eff_h1(cache, psi, H, n, prec)
            E, v, info = h1.lanczos_min(psi.tensors[n], krylovdim=krylovdim, tol=lanczos_tol, maxiter=maxiter,
                                        rq_fp64=rq_fp64 and i == len(seq) - 1)
            h1.close()
            if stats is not None:
                stats["matvecs"] = stats.get("matvecs", 0) + info["matvecs"]
            psi.tensors[n] = v
            cache.invalidate_node(n)
        energies.append(float(E))
        if len(energies) >= 2 and abs(energies[-1] - energies[-2]) < tol:
            break
    return psi, energies


def expand_exact(cache: EnvCache, psi: TTNS, H: TTNO, n, m, maxdim, max_add=8, mixing=1.0, enr_rtol=1e-10,
                 enr_atol=1e-12, precision="fp64"):
    """expand with the exact predictor scheme."""
    return expand(cache, psi, H, n, m, maxdim, max_add, mixing, enr_rtol, enr_atol, precision, scheme="exact")


def expand(cache: EnvCache, psi: TTNS, H: TTNO, n, m, maxdim, max_add=8, mixing=1.0, enr_rtol=1e-10,
           enr_atol=1e-12, precision="fp64", scheme="exact", rng=None, rsvd_oversample=8, rsvd_poweriter=0,
           factorized=False):
    """3S subspace expansion of the bond n -> m (expand!, unfactorised branch,
    lib/GraftContractions/src/Contractions/expansion.jl:40-131, 240-370, 488-512): P = the
    predictor basis of mixing * H2 Theta (n-side legs x rest; expansion.predictor_basis with
    cap = min(maxdim, D + max_add) and the scheme exact / directqr / rsvd / rangefinder); its
    directions outside range(A_n) (left singular vectors of P - Q Q^H P with Q spanning A_n,
    at most cap - D, enrichment tolerances atol / rtol) are appended to A_n; the factor U of
    [A_n E] (at most cap columns) replaces A_n and R = U^H A_n is absorbed into A_m (the
    state is unchanged: U U^H A_n = A_n).  The randomised schemes draw their probe block
    from rng, a numpy Generator.  factorized with scheme rangefinder takes the factorised
    range finder's enrichment (expansion.factorized_rangefinder_enrichment, expansion.jl:
    134-216) and U = [Q E] with no final SVD.  Returns True when the bond grew."""
    check_scheme(scheme, rng)
    ctx, t = psi.ctx, psi.topo
    olddim = psi.tensors[n].shape[-1]
    cap = min(maxdim, olddim + max_add)
    if cap <= olddim or mixing == 0:
        return False
    move_center(psi, n, cache)
    A = psi.tensors[n].contiguous()
    sh = tuple(A.shape)
    Am = A.reshape(-1, sh[-1])
    theta = two_site_tensor(psi, n, m)
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
    h2 = eff_h2(cache, psi, H, n, m, prec)
    Pt = h2(theta)
    h2.close()
    if mixing != 1:
        Pt = ctx.scale(Pt, mixing)
    if factorized and scheme == "rangefinder":
        Q, E = factorized_rangefinder_enrichment(ctx, Am, Pt.reshape(Am.shape[0], -1), cap - olddim, rng,
                                                 rsvd_oversample, rsvd_poweriter, enr_atol, enr_rtol)
        if E is None:
            return False
        U = ctx.concat_cols(Q, E)
        R = ctx.matmul(U, Am, conjA=True, transA=True)
        psi.tensors[n] = U.reshape(sh[:-1] + (U.shape[1],))
        psi.tensors[m] = absorb_on_leg(ctx, psi.tensors[m], R, t.childslot(m, n))
        psi.center = m
        cache.invalidate_edge(n, m)
        return True
    P = predictor_basis(ctx, Pt.reshape(Am.shape[0], -1), cap, scheme, rng, rsvd_oversample, rsvd_poweriter)
    room = min(max_add, cap - olddim)
    expanded = Am
    if room > 0 and Am.shape[0] > Am.shape[1]:
        Q, _ = ctx.qr(Am)
        Pc = ctx.axpby(-1.0, ctx.matmul(Q, ctx.matmul(Q, P, conjA=True, transA=True)), 1.0, P.contiguous())
        E, sig, _, _ = ctx.svd_trunc(Pc, maxdim=room, atol=enr_atol, rtol=enr_rtol)
        if E.shape[1] > 0:
            E = ctx.axpby(-1.0, ctx.matmul(Q, ctx.matmul(Q, E, conjA=True, transA=True)), 1.0, E.contiguous())
            expanded = ctx.concat_cols(Am, E)
    U, _, _, _ = ctx.svd_trunc(expanded.contiguous(), maxdim=cap)
    if U.shape[1] == olddim:
        return False
    R = ctx.matmul(U, Am, conjA=True, transA=True)
    psi.tensors[n] = U.contiguous().reshape(sh[:-1] + (U.shape[1],))
    psi.tensors[m] = absorb_on_leg(ctx, psi.tensors[m], R, t.childslot(m, n))
    psi.center = m
    cache.invalidate_edge(n, m)
    return True


def dmrg1_3s(psi: TTNS, H: TTNO, trunc: TruncationScheme | None = None, nsweeps=10, tol=1e-10, krylovdim=20,
             mixing=1.0, max_add=8, enr_rtol=1e-10, enr_atol=1e-12, precision="fp64", rq_fp64=None,
             lanczos_tol=1e-12, maxiter=100, expand_scheme="exact", rng=None, rsvd_oversample=8,
             rsvd_poweriter=0):
    """Single-site DMRG with subspace expansion between sweeps (GroundState.jl:166-248):
    dmrg1's local ground states, then expand with expand_scheme on every bond in postorder
    with mixing(sweep) (a number or a function of the sweep) and factorized=true, as the
    reference passes it (rangefinder is then the factorised range finder); bonds grow by at
    most max_add per sweep up to trunc.maxdim.  The randomised schemes (rsvd, rangefinder)
    draw their probes from rng, a numpy Generator, bond by bond.  Returns (psi, energies per
    sweep)."""
    if not H.ishermitian:
        raise ValueError("dmrg1_3s: DMRG requires ishermitian(H) == true")
    check_scheme(expand_scheme, rng, "dmrg1_3s")
    if rsvd_oversample < 0 or rsvd_poweriter < 0:
        raise ValueError("dmrg1_3s: rsvd_oversample and rsvd_poweriter must be nonnegative")
    trunc = trunc or TruncationScheme(maxdim=100)
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
    if rq_fp64 is None:
        rq_fp64 = prec != _lib.PREC_FP64
    t = psi.topo
    cache = EnvCache(t)
    order = t.postorder()
    bonds = [n for n in order if t.parent[n] >= 0]
    energies = []
    for sweep in range(nsweeps):
        E = float("nan")
        seq = list(order) + list(reversed(order))
        for i, n in enumerate(seq):
            move_center(psi, n, cache)
            h1 = eff_h1(cache, psi, H, n, prec)
            E, v, _ = h1.lanczos_min(psi.tensors[n], krylovdim=krylovdim, tol=lanczos_tol, maxiter=maxiter,
                                     rq_fp64=rq_fp64 and i == len(seq) - 1)
            h1.close()
            psi.tensors[n] = v
            cache.invalidate_node(n)
        alpha = mixing(sweep + 1) if callable(mixing) else mixing
        if alpha != 0:
            for n in bonds:
                expand(cache, psi, H, n, t.parent[n], trunc.maxdim or (1 << 30), max_add, alpha, enr_rtol,
                       enr_atol, prec, expand_scheme, rng, rsvd_oversample, rsvd_poweriter, factorized=True)
        energies.append(float(E))
        if len(energies) >= 2 and abs(energies[-1] - energies[-2]) < tol:
            break
    return psi, energies


class TDVP1:
    """One-site TDVP with order-2 splitting (tdvp.jl:31-44, 171-301)."""

    def __init__(self, order=2, krylovdim=30, tol=1e-12, precision="fp64"):
        if order not in (1, 2):
            raise ValueError("order must be 1 or 2")
        self.order = order
        self.krylovdim = krylovdim
        self.tol = tol
        self.precision = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
        self.cache = None

    def step(self, psi: TTNS, H: TTNO, dz):
        if self.cache is None or self.cache.topo != psi.topo:
            self.cache = EnvCache(psi.topo)
        if self.order == 1:
            self._sweep(psi, H, dz, rev=False)
        else:
            self._sweep(psi, H, dz / 2, rev=False, terminal_dz=dz)
            self._sweep(psi, H, dz / 2, rev=True, skip_initial=True)
        return psi

    def _sweep(self, psi, H, dz, rev, terminal_dz=None, skip_initial=False):
        t = psi.topo
        cache = self.cache
        order = t.postorder()
        if rev:
            order = order[::-1]
        move_center(psi, order[0], cache)
        for i, n in enumerate(order):
            assert psi.center == n
            if not (skip_initial and i == 0):
                sdz = terminal_dz if (terminal_dz is not None and i == len(order) - 1) else dz
                h1 = eff_h1(cache, psi, H, n, self.precision)
                A, _ = h1.exponentiate(sdz, psi.tensors[n], self.krylovdim, self.tol, hermitian=H.ishermitian)
                h1.close()
                psi.tensors[n] = A
                cache.invalidate_node(n)
            if i == len(order) - 1:
                break
            seg = t.path_between(n, order[i + 1])
            for j in range(1, len(seg)):
                u, v = seg[j - 1], seg[j]
                if (t.parent[u] == v) != rev:
                    self._evolve_link_and_move(psi, H, u, v, dz)
                else:
                    move_center(psi, v, cache)

    def _evolve_link_and_move(self, psi, H, u, v, dz):
        """(tdvp.jl:257-288)"""
        ctx, t, cache = psi.ctx, psi.topo, self.cache
        if t.parent[u] == v:
            Q, Cl = left_orth(ctx, psi.tensors[u])
            psi.tensors[u] = Q
            cache.invalidate_node(u)
            k0 = eff_h0(cache, psi, H, u, v, self.precision)
            Cl, _ = k0.exponentiate(-dz, Cl, self.krylovdim, self.tol, hermitian=H.ishermitian)
            k0.close()
            psi.tensors[v] = absorb_on_leg(ctx, psi.tensors[v], Cl, t.childslot(v, u))
        else:
            k = t.childslot(u, v)
            Q, Cd = orth_factor_leg(ctx, psi.tensors[u], k)
            psi.tensors[u] = Q
            Cl = ctx.permute(Cd, [1, 0])
            cache.invalidate_node(u)
            k0 = eff_h0(cache, psi, H, v, u, self.precision)
            Cl, _ = k0.exponentiate(-dz, Cl, self.krylovdim, self.tol, hermitian=H.ishermitian)
            k0.close()
            Av = psi.tensors[v]
            r = Av.dim()
            lab = [-(j + 1) for j in range(r - 1)] + [1]
            psi.tensors[v] = ctx.contract([Av, Cl], [lab, [1, -r]])
        psi.center = v
        cache.invalidate_node(v)


class TDVP2:
    """Two-site TDVP (tdvp.jl:67-84, 307-431): every bond is evolved forward as a two-site
    block and split by truncated SVD (bond dimensions adapt up to ``trunc.maxdim``), with a
    backward one-site evolution of the connecting parent between consecutive bonds.  Order
    2 fuses the turning bond's two half steps into one full step and one split."""

    def __init__(self, order=2, trunc: TruncationScheme | None = None, krylovdim=30, tol=1e-12,
                 precision="fp64", fuse_turning=True):
        if order not in (1, 2):
            raise ValueError("order must be 1 or 2")
        self.order = order
        self.trunc = trunc or TruncationScheme()
        self.krylovdim = krylovdim
        self.tol = tol
        self.fuse_turning = fuse_turning
        self.precision = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
        self.cache = None

    def step(self, psi: TTNS, H: TTNO, dz):
        if self.cache is None or self.cache.topo != psi.topo:
            self.cache = EnvCache(psi.topo)
        if self.order == 1:
            self._sweep(psi, H, dz, rev=False)
        elif self.fuse_turning:
            self._sweep(psi, H, dz / 2, rev=False, terminal_dz=dz)
            self._sweep(psi, H, dz / 2, rev=True, skip_initial=True)
        else:
            self._sweep(psi, H, dz / 2, rev=False)
            self._sweep(psi, H, dz / 2, rev=True)
        return psi

    def _sweep(self, psi, H, dz, rev, terminal_dz=None, skip_initial=False):
        t = psi.topo
        bonds = [n for n in t.postorder() if t.parent[n] >= 0]
        last = len(bonds) - 1
        for j in (range(last, -1, -1) if rev else range(last + 1)):
            if rev and skip_initial and j == last:
                continue
            n = bonds[j]
            m = t.parent[n]
            move_center(psi, m, self.cache)
            if rev:
                if j != last:
                    self._site_backward(psi, H, m, dz)
                self._bond_forward(psi, H, n, m, dz, "n")
            else:
                term = terminal_dz is not None and j == last
                self._bond_forward(psi, H, n, m, terminal_dz if term else dz, "n" if term else "m")
                if j != last:
                    self._site_backward(psi, H, m, dz)

    def _bond_forward(self, psi, H, n, m, dz, center_on):
        theta = two_site_tensor(psi, n, m)
        h2 = eff_h2(self.cache, psi, H, n, m, self.precision)
        theta, _ = h2.exponentiate(dz, theta, self.krylovdim, self.tol, hermitian=H.ishermitian)
        h2.close()
        self.cache.invalidate_edge(n, m)
        split_two_site(psi, theta, n, m, self.trunc, center_on)

    def _site_backward(self, psi, H, m, dz):
        assert psi.center == m
        h1 = eff_h1(self.cache, psi, H, m, self.precision)
        A, _ = h1.exponentiate(-dz, psi.tensors[m], self.krylovdim, self.tol, hermitian=H.ishermitian)
        h1.close()
        psi.tensors[m] = A
        self.cache.invalidate_node(m)


def evolve(ev, psi: TTNS, H: TTNO, dz, nsteps):
    """(Evolution.jl:86-93)"""
    for _ in range(nsteps):
        ev.step(psi, H, dz)
    return psi
