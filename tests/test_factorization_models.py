"""Host models of the device factorisations (no GPU): numpy restatements of the formulas the
kernels in csrc/gtn_tsqr.cu apply, run on the same kinds of input as the GPU tests.

* Shifted Cholesky QR with two refinement passes (Fukaya, Kannan, Nakatsukasa, Zhang and
  Yamamoto 2020): the shift s = 11 (m n + n (n + 1)) u |A|_F^2, three Cholesky factors,
  row-wise triangular solves, and the acceptance rule (every pivot positive, |Q^H Q - I| <=
  1e-12 entrywise) under which the library keeps the result; otherwise it runs Householder.
* One-sided Jacobi SVD (Hestenes): the complex rotation of a column pair, the round-robin
  pair schedule of the eight warps, the 1e-15 relative orthogonality threshold, and the
  completion of exact null columns."""
import numpy as np
import pytest


def crandn(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


# ---- shifted Cholesky QR ------------------------------------------------------------------

def cholesky_upper(G):
    """Upper R with G = R^H R, or None when a pivot is not positive (host_cholesky)."""
    n = G.shape[0]
    R = np.zeros_like(G)
    for j in range(n):
        d = G[j, j].real - np.sum(np.abs(R[:j, j]) ** 2)
        if not (d > 0.0) or not np.isfinite(d):
            return None
        R[j, j] = np.sqrt(d)
        for c in range(j + 1, n):
            R[j, c] = (G[j, c] - np.sum(np.conj(R[:j, j]) * R[:j, c])) / R[j, j]
    return R


def forward_rows(A, R):
    """Q = A R^-1 row by row: q_j = (a_j - sum_{i<j} q_i R_ij) / R_jj (tsqr_trsm)."""
    Q = A.astype(complex).copy()
    for j in range(R.shape[0]):
        Q[:, j] = (Q[:, j] - Q[:, :j] @ R[:j, j]) / R[j, j].real
    return Q


def shifted_cholesky_qr3(A):
    m, n = A.shape
    X, Rtot = A, None
    for p in range(3):
        G = X.conj().T @ X
        if p == 0:
            G = G + 11.0 * (m * n + n * (n + 1)) * 2.0 ** -53 * np.trace(G).real * np.eye(n)
        R = cholesky_upper(G)
        if R is None:
            return None
        X = forward_rows(X, R)
        Rtot = R if Rtot is None else R @ Rtot
    if np.abs(X.conj().T @ X - np.eye(n)).max() > 1e-12:
        return None  # the library then runs the Householder QR
    return X, Rtot


@pytest.mark.parametrize("m,n,kind", [(4096, 16, "random"), (2000, 24, "cond1e10"), (3000, 8, "cond1e14"),
                                       (1000, 16, "rank_deficient"), (512, 8, "zero")])
def test_shifted_cholesky_qr_model(m, n, kind):
    rng = np.random.default_rng(m + n)
    A = crandn(rng, (m, n))
    if kind.startswith("cond"):
        u, _ = np.linalg.qr(A)
        v, _ = np.linalg.qr(crandn(rng, (n, n)))
        A = (u * np.logspace(0, -float(kind[6:]), n)) @ v.conj().T
    elif kind == "rank_deficient":
        A[:, n // 2:] = A[:, : n - n // 2] * (1 - 0.5j)
    elif kind == "zero":
        A[:] = 0
    out = shifted_cholesky_qr3(A)
    if kind in ("random", "cond1e10"):
        assert out is not None, kind  # well-conditioned input takes the fast path
    if kind == "zero":
        assert out is None  # no positive pivot even after the shift: Householder takes over
    if out is not None:
        # whenever the result is kept: orthonormal to 1e-12 (the acceptance rule), A = Q R to
        # rounding (the row-wise solves are backward stable), R upper with a positive diagonal
        Q, R = out
        assert np.abs(Q.conj().T @ Q - np.eye(n)).max() <= 1e-12
        assert np.linalg.norm(Q @ R - A) <= 1e-14 * np.linalg.norm(A) * np.sqrt(m)
        assert np.allclose(np.tril(R, -1), 0)
        assert np.all(np.diag(R).real > 0)


# ---- one-sided Jacobi SVD ------------------------------------------------------------------

def round_robin_pairs(bc):
    """The pairs of each round, as the kernel's warps take them (circle method)."""
    P = bc + (bc & 1)
    rounds = []
    for r in range(P - 1):
        pairs = []
        for i in range(P // 2):
            p = P - 1 if i == 0 else (r + i) % (P - 1)
            q = r % (P - 1) if i == 0 else (r + P - 1 - i) % (P - 1)
            p, q = min(p, q), max(p, q)
            if q < bc:
                pairs.append((p, q))
        rounds.append(pairs)
    return rounds


def jacobi_svd(A):
    m, n = A.shape
    tall = m >= n
    W = (A if tall else A.conj().T).astype(complex).copy()
    br, bc = W.shape
    V = np.eye(bc, dtype=complex)
    for _ in range(40):
        rotated = False
        for pairs in round_robin_pairs(bc):
            for p, q in pairs:
                a, b = W[:, p], W[:, q]
                al, be = np.vdot(a, a).real, np.vdot(b, b).real
                g = np.vdot(a, b)  # conj(a) . b
                ag = abs(g)
                if not (ag > 1e-15 * np.sqrt(al * be)) or ag == 0.0:
                    continue
                rotated = True
                ph = np.conj(g) / ag
                zeta = (be - al) / (2.0 * ag)
                t = (1.0 if zeta >= 0 else -1.0) / (abs(zeta) + np.sqrt(1.0 + zeta * zeta))
                c = 1.0 / np.sqrt(1.0 + t * t)
                s = c * t
                eb = ph * b
                W[:, p], W[:, q] = c * a - s * eb, s * a + c * eb
                vp, vq = V[:, p].copy(), V[:, q] * ph
                V[:, p], V[:, q] = c * vp - s * vq, s * vp + c * vq
        if not rotated:
            break
    nrm = np.linalg.norm(W, axis=0)
    order = np.argsort(-nrm, kind="stable")
    thr = nrm[order[0]] * 1e-200
    X = np.zeros_like(W)
    for j, c in enumerate(order):
        if nrm[c] > thr and nrm[c] > 0.0:
            X[:, j] = W[:, c] / nrm[c]
            continue
        for e in range(br):  # completion of a null column by Gram-Schmidt on unit vectors
            x = np.zeros(br, complex)
            x[e] = 1.0
            for _ in range(2):
                x = x - X[:, :j] @ (X[:, :j].conj().T @ x)
            if np.vdot(x, x).real > 0.25:
                X[:, j] = x / np.linalg.norm(x)
                break
    S = np.where(nrm[order] > thr, nrm[order], 0.0)
    Vo = V[:, order]
    if tall:
        return X, S, Vo.conj().T
    return Vo, S, X.conj().T


def test_round_robin_covers_every_pair_once():
    for bc in (1, 2, 3, 7, 16, 33, 64):
        seen = [pq for rnd in round_robin_pairs(bc) for pq in rnd]
        assert len(seen) == len(set(seen)) == bc * (bc - 1) // 2
        for rnd in round_robin_pairs(bc):
            cols = [c for pq in rnd for c in pq]
            assert len(cols) == len(set(cols))  # disjoint within a round: warps never collide


@pytest.mark.parametrize("m,n,rank", [(30, 20, 20), (20, 30, 20), (40, 12, 4), (9, 9, 0), (64, 64, 64)])
def test_one_sided_jacobi_model(m, n, rank):
    rng = np.random.default_rng(7 * m + n)
    k = min(m, n)
    A = crandn(rng, (m, rank)) @ crandn(rng, (rank, n)) if rank else np.zeros((m, n), complex)
    U, S, Vh = jacobi_svd(A)
    assert np.allclose(S, np.linalg.svd(A, compute_uv=False), rtol=1e-12, atol=1e-12 * max(1.0, S.max()))
    assert np.abs(U.conj().T @ U - np.eye(k)).max() < 1e-12
    assert np.abs(Vh @ Vh.conj().T - np.eye(k)).max() < 1e-12
    assert np.linalg.norm((U * S) @ Vh - A) <= 1e-13 * max(np.linalg.norm(A), 1e-300)
