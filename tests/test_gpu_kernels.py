"""Kernel-level parity of libgrafttn against numpy (called through the C ABI)."""
import numpy as np
import pytest

from oracle import ttn_oracle as O

pytestmark = pytest.mark.gpu

RTOL = {"fp64": 1e-12, "fp32": 2e-5, "bf16x6": 1e-5, "bf16x3": 1e-3, "fp16x3": 1e-5}  # FP32 TMEM accumulation error grows with K


def crandn(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("shape,perm", [((3, 4, 5), (2, 0, 1)), ((7, 1, 33, 2), (3, 2, 1, 0)),
                                        ((64, 65), (1, 0)), ((2, 3, 4, 5, 6), (4, 1, 3, 0, 2))])
def test_permute(ctx, shape, perm):
    rng = np.random.default_rng(0)
    a = crandn(rng, shape)
    out = ctx.download(ctx.permute(ctx.upload(a), list(perm)))
    assert np.array_equal(out, a.transpose(perm))


def _contract_case(ctx, rng, shapes, labels, order, prec):
    ts = [crandn(rng, s) for s in shapes]
    ref = O.ncon(ts, labels, None, order)
    from grafttn import _lib
    out = ctx.download(ctx.contract([ctx.upload(t) for t in ts], labels, None, order, _lib.PRECISIONS[prec]))
    return rel(out, ref)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "bf16x6", "bf16x3"])
def test_contract_small_k(ctx, prec):
    # W-like step: K = 10 (strided SIMT path), legs interleaved
    rng = np.random.default_rng(1)
    shapes = [(5, 6, 2, 7), (5, 2, 2, 3)]
    labels = [[1, -1, 2, -2], [1, -3, 2, -4]]
    assert _contract_case(ctx, rng, shapes, labels, [0, 1], prec) < RTOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "fp32", "bf16x6", "bf16x3", "fp16x3"])
@pytest.mark.parametrize("mkn", [(130, 200, 70), (257, 1000, 129), (64, 96, 300), (1, 128, 1)])
def test_contract_gemm(ctx, prec, mkn):
    # GEMM path (K > 64): tcgen05 for the bf16 modes, SIMT for fp64 / fp32
    M, K, N = mkn
    rng = np.random.default_rng(2)
    shapes = [(M, K), (K, N)]
    labels = [[-1, 1], [1, -2]]
    assert _contract_case(ctx, rng, shapes, labels, [0, 1], prec) < RTOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "bf16x6", "fp16x3"])
def test_contract_gemm_permuted(ctx, prec):
    # contracted legs not innermost in the running tensor, statics with conj
    rng = np.random.default_rng(3)
    a, b = crandn(rng, (9, 40, 3, 8)), crandn(rng, (8, 11, 40))
    labels = [[-1, 1, -2, 2], [2, -3, 1]]
    ref = O.ncon([a, b], labels, [False, True])
    from grafttn import _lib
    out = ctx.download(ctx.contract([ctx.upload(a), ctx.upload(b)], labels, [False, True], None,
                                    _lib.PRECISIONS[prec]))
    assert rel(out, ref) < RTOL[prec]


def test_tc_gemm_large(ctx):
    # multi-tile, multi-stage pipeline: M, 2N and 2K well above one tile / stage ring
    rng = np.random.default_rng(4)
    M, K, N = 700, 2000, 300
    from grafttn import _lib
    for prec in ("bf16x6", "bf16x3", "fp16x3"):
        assert _contract_case(ctx, rng, [(M, K), (K, N)], [[-1, 1], [1, -2]], [0, 1], prec) < RTOL[prec]
    ctx.sync()


def test_chain_map_all_precisions(ctx):
    # a chain of steps with mixed small-K / GEMM steps: an h2-like map on random statics
    rng = np.random.default_rng(5)
    D, w, d = 40, 5, 2
    theta = crandn(rng, (D, d, d, D))
    L, R = crandn(rng, (D, w, D)), crandn(rng, (D, w, D))
    W1, W2 = crandn(rng, (w, d, d, w)), crandn(rng, (w, d, d, w))
    # labels: theta [a, s1, s2, b]; L [a, wl, -1]; W1 [wl, -2, s1, wm]; W2 [wm, -3, s2, wr]; R [b, wr, -4]
    labels = [[1, 2, 3, 4], [1, 5, -1], [5, -2, 2, 6], [6, -3, 3, 7], [4, 7, -4]]
    ref = O.ncon([theta, L, W1, W2, R], labels)
    from grafttn.contractions import EffectiveMap
    for prec in ("fp64", "fp32", "bf16x6", "bf16x3", "fp16x3"):
        hm = EffectiveMap(ctx, theta.shape, labels, [0, 1, 2, 3, 4],
                          [ctx.upload(x) for x in (L, W1, W2, R)], prec)
        y = ctx.download(hm(ctx.upload(theta)))
        assert rel(y, ref) < RTOL[prec], prec
        hm.close()


@pytest.mark.parametrize("m,n,kind", [(4096, 16, "random"), (131072, 16, "random"), (20000, 64, "random"),
                                       (50000, 24, "cond1e10"), (30000, 16, "rank_deficient"), (8192, 8, "zero"),
                                       (40, 10, "rank_deficient"), (16, 16, "zero"), (3, 20, "random"),
                                       (64, 64, "cond1e10"), (1, 1, "random")])
def test_qr_tall_skinny(ctx, m, n, kind):
    """Thin QR on the device paths: one-CTA Householder for small matrices, shifted Cholesky
    QR with refinement for tall-skinny ones (the cuSOLVER Householder QR when the matrix is
    too ill-conditioned for it): Q orthonormal, A = Q R, R upper triangular."""
    rng = np.random.default_rng(m + n)
    a = crandn(rng, (m, n))
    k = min(m, n)
    if kind == "cond1e10":
        u, _ = np.linalg.qr(a)
        v, _ = np.linalg.qr(crandn(rng, (n, n)))
        a = (u[:, :k] * np.logspace(0, -10, k)) @ v[:k].conj()
    elif kind == "rank_deficient":
        a[:, n // 2:] = a[:, : n - n // 2] * (1 + 2j)
    elif kind == "zero":
        a[:] = 0
    Q, R = ctx.qr(ctx.upload(a))
    Q, R = ctx.download(Q), ctx.download(R)
    scale = max(np.linalg.norm(a), 1e-300)
    assert np.linalg.norm(Q @ R - a) <= 1e-13 * scale + (0 if kind != "zero" else 1e-300)
    assert np.abs(Q.conj().T @ Q - np.eye(k)).max() < 1e-12
    assert np.allclose(np.tril(R, -1), 0)


@pytest.mark.parametrize("m,n,rank", [(30, 20, 5), (20, 30, 20), (64, 64, 64), (7, 3, 0), (1, 9, 1)])
def test_svd_small_jacobi(ctx, m, n, rank):
    """The one-CTA Jacobi SVD of small matrices (min(m, n) <= 64, m n <= 4096): singular values
    against numpy, orthonormal factors also for rank-deficient and zero input, reconstruction."""
    rng = np.random.default_rng(m * 100 + n)
    k = min(m, n)
    a = crandn(rng, (m, rank)) @ crandn(rng, (rank, n)) if rank > 0 else np.zeros((m, n), complex)
    U, S, Vh, disc = ctx.svd_trunc(ctx.upload(a))
    U, Vh = ctx.download(U), ctx.download(Vh)
    assert len(S) == k
    assert np.allclose(S, np.linalg.svd(a, compute_uv=False), rtol=1e-12, atol=1e-12 * max(1.0, np.abs(S).max()))
    assert np.abs(U.conj().T @ U - np.eye(k)).max() < 1e-12
    assert np.abs(Vh @ Vh.conj().T - np.eye(k)).max() < 1e-12
    assert np.linalg.norm((U * S) @ Vh - a) <= 1e-13 * max(np.linalg.norm(a), 1e-300)


def test_qr_svd(ctx):
    rng = np.random.default_rng(6)
    for m, n in [(50, 20), (20, 50), (33, 33)]:
        a = crandn(rng, (m, n))
        Q, R = ctx.qr(ctx.upload(a))
        Q, R = ctx.download(Q), ctx.download(R)
        assert rel(Q @ R, a) < 1e-13
        assert np.allclose(Q.conj().T @ Q, np.eye(min(m, n)), atol=1e-13)
        assert np.allclose(np.tril(R, -1), 0)
        U, S, Vh, disc = ctx.svd_trunc(ctx.upload(a))
        U, Vh = ctx.download(U), ctx.download(Vh)
        assert rel((U * S) @ Vh, a) < 1e-13
        assert np.allclose(S, np.linalg.svd(a, compute_uv=False), rtol=1e-12)
        U, S, Vh, disc = ctx.svd_trunc(ctx.upload(a), maxdim=5)
        s_all = np.linalg.svd(a, compute_uv=False)
        assert len(S) == 5 and abs(disc - np.sqrt(np.sum(s_all[5:] ** 2))) < 1e-12


def test_lanczos_and_expm(ctx):
    rng = np.random.default_rng(7)
    n = 60
    A = crandn(rng, (n, n))
    Hm = (A + A.conj().T) / 2
    # a map y = H x as a one-step contraction of x[n] with the static H[n, n] -> y[n]
    from grafttn.contractions import EffectiveMap
    hm = EffectiveMap(ctx, (n,), [[1], [-1, 1]], [0, 1], [ctx.upload(Hm)], "fp64")
    x0 = crandn(rng, (n,))
    E, v, info = hm.lanczos_min(ctx.upload(x0), krylovdim=30, tol=1e-13, maxiter=50)
    w = np.linalg.eigvalsh(Hm)
    assert abs(E - w[0]) < 1e-10, (E, w[0], info)
    vv = ctx.download(v)
    assert np.linalg.norm(Hm @ vv - E * vv) < 1e-6
    y, info = hm.exponentiate(-0.3j, ctx.upload(x0), krylovdim=30, tol=1e-12)
    import scipy.linalg as sla
    ref = sla.expm(-0.3j * Hm) @ x0
    assert rel(ctx.download(y), ref) < 1e-10
    hm.close()


@pytest.mark.parametrize("linalg", ["fp64", "fp64e"])
@pytest.mark.parametrize("m,n", [(500, 700), (700, 500), (512, 512)])
def test_svd_gram_path_large(ctx, m, n, linalg):
    # above the Gram threshold: Gram matrix (FP64 SIMT or FP64-grade tensor-core GEMM, the
    # context's linear-algebra precision) + Zheevd; decaying spectrum down to 1e-7
    rng = np.random.default_rng(8)
    k = min(m, n)
    U0, _ = np.linalg.qr(crandn(rng, (m, k)))
    V0, _ = np.linalg.qr(crandn(rng, (n, k)))
    s0 = np.logspace(0, -7, k)
    a = (U0 * s0) @ V0.conj().T
    old = ctx.linalg_precision(linalg)
    try:
        U, S, Vh, disc = ctx.svd_trunc(ctx.upload(a), maxdim=300)
    finally:
        ctx.linalg_precision(old)
    U, Vh = ctx.download(U), ctx.download(Vh)
    assert len(S) == 300
    # the Gram path resolves sigma to ~eps * s_max^2 / sigma: ~1e-12 absolute here
    assert np.allclose(S, s0[:300], rtol=1e-6, atol=1e-12)
    ref = (U0[:, :300] * s0[:300]) @ V0[:, :300].conj().T
    assert np.linalg.norm((U * S) @ Vh - ref) < 1e-9 * np.linalg.norm(ref)
    assert np.allclose(U.conj().T @ U, np.eye(300), atol=1e-9)
    assert np.allclose(Vh @ Vh.conj().T, np.eye(300), atol=1e-9)
    # discarded 2-norm from Gram eigenvalues: absolute accuracy ~ sqrt(k) * eps / s_300
    assert abs(disc - np.sqrt(np.sum(s0[300:] ** 2))) < 1e-8


@pytest.mark.parametrize("m,n", [(1536, 2048), (2048, 1536)])
def test_svd_subspace_route(ctx, m, n, monkeypatch):
    # maxdim 64 of 1536: subspace iteration on 96 vectors instead of the Gram matrix; a
    # geometric spectrum (0.85^i: sigma_97 / sigma_64 = 5e-3) settles in three iterations
    rng = np.random.default_rng(21)
    k = min(m, n)
    U0, _ = np.linalg.qr(crandn(rng, (m, k)))
    V0, _ = np.linalg.qr(crandn(rng, (n, k)))
    s0 = 0.85 ** np.arange(k)
    a = (U0 * s0) @ V0.conj().T
    U, S, Vh, disc = ctx.svd_trunc(ctx.upload(a), maxdim=64)
    U, Vh = ctx.download(U), ctx.download(Vh)
    assert len(S) == 64
    assert np.allclose(S, s0[:64], rtol=1e-10, atol=1e-14)
    assert np.allclose(U.conj().T @ U, np.eye(64), atol=1e-12)
    assert np.allclose(Vh @ Vh.conj().T, np.eye(64), atol=1e-12)
    ref = (U0[:, :64] * s0[:64]) @ V0[:, :64].conj().T
    assert np.linalg.norm((U * S) @ Vh - ref) < 1e-8 * np.linalg.norm(ref)
    # discarded 2-norm from |A|_F^2 minus the kept weight: absolute accuracy ~ eps |A|_F^2 / disc
    assert abs(disc - np.sqrt(np.sum(s0[64:] ** 2))) < 1e-9
    # the Gram route (switched off subspace iteration) gives the same truncation
    monkeypatch.setenv("GTN_SVD_SUBSPACE", "0")
    U2, S2, Vh2, disc2 = ctx.svd_trunc(ctx.upload(a), maxdim=64)
    assert np.allclose(S2, S, rtol=1e-9)
    assert np.linalg.norm((ctx.download(U2) * S2) @ ctx.download(Vh2) - (U * S) @ Vh) < 1e-8 * np.linalg.norm(ref)
    assert abs(disc2 - disc) < 1e-9


def test_svd_subspace_flat_spectrum_falls_back(ctx):
    # a nearly flat spectrum does not settle within the iteration cap: the Gram route runs
    rng = np.random.default_rng(22)
    m, n = 1536, 1600
    U0, _ = np.linalg.qr(crandn(rng, (m, m)))
    V0, _ = np.linalg.qr(crandn(rng, (n, m)))
    s0 = np.linspace(1.0, 0.9, m)
    a = (U0 * s0) @ V0.conj().T
    U, S, Vh, disc = ctx.svd_trunc(ctx.upload(a), maxdim=64)
    U, Vh = ctx.download(U), ctx.download(Vh)
    assert np.allclose(S, s0[:64], rtol=1e-9)
    assert np.allclose(U.conj().T @ U, np.eye(64), atol=1e-10)
    assert np.allclose(Vh @ Vh.conj().T, np.eye(64), atol=1e-10)
    assert abs(disc - np.sqrt(np.sum(s0[64:] ** 2))) < 1e-8


@pytest.mark.parametrize("m,n", [(512, 768), (768, 512)])
def test_svd_gram_rank_deficient(ctx, m, n):
    # rank 200 < maxdim: the kept directions beyond the rank still form isometries, so a
    # two-site split of a low-rank tensor keeps a normalised state
    rng = np.random.default_rng(9)
    a = crandn(rng, (m, 200)) @ crandn(rng, (200, n))
    U, S, Vh, disc = ctx.svd_trunc(ctx.upload(a), maxdim=400)
    U, Vh = ctx.download(U), ctx.download(Vh)
    assert len(S) == 400
    assert np.allclose(U.conj().T @ U, np.eye(400), atol=1e-9)
    assert np.allclose(Vh @ Vh.conj().T, np.eye(400), atol=1e-9)
    assert np.linalg.norm((U * S) @ Vh - a) < 1e-9 * np.linalg.norm(a)
    assert np.allclose(S[:200], np.linalg.svd(a, compute_uv=False)[:200], rtol=1e-9)


def test_fp16x3_wide_dynamic_range(ctx):
    # rows whose magnitudes differ by 1e12 (power-of-two row scales keep each row's
    # relative accuracy), plus an all-zero row
    rng = np.random.default_rng(12)
    M, K, N = 300, 700, 90
    a = crandn(rng, (M, K)) * np.logspace(-6, 6, M)[:, None]
    a[7] = 0
    b = crandn(rng, (K, N)) * np.logspace(3, -3, N)[None, :]
    from grafttn import _lib
    out = ctx.download(ctx.contract([ctx.upload(a), ctx.upload(b)], [[-1, 1], [1, -2]], None, [0, 1],
                                    _lib.PRECISIONS["fp16x3"]))
    ref = a @ b
    rows = np.linalg.norm(out - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)
    assert np.all(rows[np.arange(M) != 7] < 1e-5)
    assert np.all(out[7] == 0)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("N", [5, 16, 40])
def test_contract_tall_skinny_splitk(ctx, prec, N):
    # few output tiles, long K: the SIMT GEMM splits K over CTAs and sums the slices
    # (64 x 16 tiles for N <= 16, 64 x 64 above)
    rng = np.random.default_rng(13)
    K, M = 70001, 48
    a, b = crandn(rng, (K, M)), crandn(rng, (K, N))
    from grafttn import _lib
    out = ctx.download(ctx.contract([ctx.upload(a), ctx.upload(b)], [[1, -1], [1, -2]], [False, True], None,
                                    _lib.PRECISIONS[prec]))
    ref = a.T @ b.conj()
    assert rel(out, ref) < (1e-12 if prec == "fp64" else 2e-5)
