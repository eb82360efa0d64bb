"""Predictor bases of the 3S bond expansion (expand!, lib/GraftContractions/src/Contractions/
expansion.jl:240-370) over the device context.

The randomised schemes take their Gaussian probe block from a caller-owned numpy Generator,
in place of the reference's caller-owned Xoshiro stream (whose draws cannot be reproduced
outside Julia): real parts first, then imaginary parts, scaled to unit complex variance.
The probe is drawn on the host and uploaded; every product, QR and SVD runs on the device.
This module only needs a context object with upload / matmul / qr / svd_trunc / axpby / scale,
so its logic is importable without a GPU.
"""
from __future__ import annotations

import numpy as np

SCHEMES = ("exact", "directqr", "rsvd", "rangefinder")


def check_scheme(scheme, rng, who="expand"):
    """The reference's argument checks (expansion.jl:60-79, GroundState.jl:193-199)."""
    if scheme not in SCHEMES:
        raise ValueError(f"{who}: scheme must be one of {SCHEMES}")
    if scheme in ("rsvd", "rangefinder") and rng is None:
        raise ValueError(f"{who}: scheme={scheme} requires an explicit rng")


def probe_block(rng, rest, budget):
    """Complex Gaussian rest x budget block with unit variance (expansion.jl:372-446)."""
    re = rng.standard_normal((rest, budget))
    im = rng.standard_normal((rest, budget))
    return (re + 1j * im) / np.sqrt(2.0)


def predictor_basis(ctx, P, cap, scheme="exact", rng=None, oversample=8, poweriter=0):
    """Orthonormal predictor basis of the row-major (n-side legs) x (rest) device matrix P
    (_child_predictor_basis, expansion.jl:240-272):

    * exact: the leading cap left singular vectors (split_svd with maxdim = cap);
    * directqr: Q of the compact QR of P (_directqr_predictor_basis, :275-278);
    * rsvd: the leading cap left singular vectors of (P P^H)^q P Omega (:348-370);
    * rangefinder: Q of QR(P Omega), then q steps Z = Q(P^H Q), Q = Q(P Z) (rangefinder,
      :280-326).

    Omega has min(rest, cap + oversample) columns and q = poweriter."""
    check_scheme(scheme, rng)
    if oversample < 0 or poweriter < 0:
        raise ValueError("expand: rsvd_oversample and rsvd_poweriter must be nonnegative")
    P = P.contiguous()
    if scheme == "exact":
        U, _, _, _ = ctx.svd_trunc(P, maxdim=cap)
        return U
    if scheme == "directqr":
        Q, _ = ctx.qr(P)
        return Q
    rest = int(P.shape[1])
    budget = min(rest, cap + oversample)
    omega = ctx.upload(probe_block(rng, rest, budget))
    Y = ctx.matmul(P, omega)
    if scheme == "rsvd":
        for _ in range(poweriter):
            Y = ctx.matmul(P, ctx.matmul(P, Y, conjA=True, transA=True))
        U, _, _, _ = ctx.svd_trunc(Y.contiguous(), maxdim=cap)
        return U
    Q, _ = ctx.qr(Y.contiguous())
    for _ in range(poweriter):
        Z, _ = ctx.qr(ctx.matmul(P, Q, conjA=True, transA=True).contiguous())
        Q, _ = ctx.qr(ctx.matmul(P, Z).contiguous())
    return Q


def factorized_rangefinder_enrichment(ctx, Am, P, room, rng, oversample=8, poweriter=0, enr_atol=1e-12,
                                      enr_rtol=1e-10):
    """Enrichment of the factorised range finder (_factorized_rangefinder_enrich_split,
    expansion.jl:134-216) for the row-major n-side matrix A_n and the predictor
    P = mixing * H2 Theta (n-side legs x rest), both on the device.

    The reference range-finds N^H P, with N an orthonormal basis of the complement of
    range(A_n), and appends E = N S L, where S is the range-finder basis and L holds the
    kept left singular vectors of S^H N^H P (maxdim = room, atol, rtol). Here the complement
    is the projector 1 - Q Q^H, with Q from the QR of A_n, so that no basis of N is formed:
    P_c = P - Q (Q^H P) has the same range-finder sketches as N^H P, mapped by N. A QR of
    P_c Omega that is wider than the complement completes with columns of zero weight, and
    the rank cut on S^H P_c drops them. Returns (Q, E), with E None when nothing is added."""
    Q, _ = ctx.qr(Am.contiguous())
    if room <= 0 or Am.shape[0] <= Q.shape[1]:
        return Q, None
    # P_c is formed in place in a copy of P
    Pc = ctx.axpby(-1.0, ctx.matmul(Q, ctx.matmul(Q, P, conjA=True, transA=True)), 1.0,
                   ctx.scale(P.contiguous(), 1.0))
    rest = int(P.shape[1])
    sk = min(rest, room + oversample)
    omega = ctx.upload(probe_block(rng, rest, sk))
    S, _ = ctx.qr(ctx.matmul(Pc, omega).contiguous())
    for _ in range(poweriter):
        Z, _ = ctx.qr(ctx.matmul(Pc, S, conjA=True, transA=True).contiguous())
        S, _ = ctx.qr(ctx.matmul(Pc, Z).contiguous())
    L, _, _, _ = ctx.svd_trunc(ctx.matmul(S, Pc, conjA=True, transA=True).contiguous(), maxdim=room,
                               atol=enr_atol, rtol=enr_rtol)
    if L.shape[1] == 0:
        return Q, None
    E = ctx.matmul(S, L)
    # keep E orthogonal to range(A_n) to working precision
    E = ctx.axpby(-1.0, ctx.matmul(Q, ctx.matmul(Q, E, conjA=True, transA=True)), 1.0, E.contiguous())
    return Q, E
