"""The arithmetic of the FP64-grade tensor-core GEMM (GTN_PREC_FP64E), restated in numpy on
the CPU: 7 signed base-128 digits per row-scaled value, the digit products of level
i + j <= 6 summed per level in chunks of 256 (each level sum must stay an exact FP32
integer) and combined with the level weights 2^{-7(i+j+2)}.  Checks the digit bounds that
make every digit exact in bf16, the exactness bound of the chunk sums, and the accuracy of
the truncated product against the FP64 product (the kernel's own arithmetic is checked on
the GPU by tests/test_gpu_f64e.py)."""
import numpy as np

S, CHUNK = 7, 256


def row_exp(mx):
    if mx == 0:
        return 0
    e = int(np.frexp(np.float32(mx))[1])  # mx = f 2^e, f in [0.5, 1)
    return -e  # |x| 2^k < 1


def digits(x, k):
    """x 2^k = sum_i d_i 2^{-7(i+1)} with round-half-up peeling of N = round(x 2^{k + 7 S})."""
    N = np.rint(np.ldexp(x, k + 7 * S)).astype(np.int64)
    out = []
    for i in range(S):
        w = 7 * (S - 1 - i)
        if w > 0:
            d = (N + (1 << (w - 1))) >> w
            N = N - (d << w)
        else:
            d = N
        out.append(d)
    return out


def model_gemm(A, B):
    """A [M, K], B [N, K] real -> A B^T by the digit scheme."""
    ka = np.array([row_exp(np.abs(r).max()) for r in A])
    kb = np.array([row_exp(np.abs(r).max()) for r in B])
    DA = digits(A, ka[:, None])
    DB = digits(B, kb[:, None])
    M, K = A.shape
    N = B.shape[0]
    acc = np.zeros((M, N))
    for c0 in range(0, K, CHUNK):
        sl = slice(c0, c0 + CHUNK)
        for lev in range(S):
            L = np.zeros((M, N), dtype=np.int64)
            for i in range(S):
                j = lev - i
                if 0 <= j < S:
                    L += DA[i][:, sl] @ DB[j][:, sl].T
            assert np.abs(L).max() < 2 ** 24  # an exact FP32 sum
            acc += np.ldexp(L.astype(np.float64), -7 * (lev + 2))
    return acc * np.ldexp(1.0, -(ka[:, None] + kb[None, :]))


def test_digit_bounds_and_reconstruction():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((64, 300)) * np.exp(rng.uniform(-20, 20, (64, 1)))
    k = np.array([row_exp(np.abs(r).max()) for r in x])[:, None]
    d = digits(x, k)
    assert np.abs(d[0]).max() <= 128 and all(np.abs(di).max() <= 64 for di in d[1:])
    rec = sum(np.ldexp(di.astype(np.float64), -7 * (i + 1)) for i, di in enumerate(d))
    assert np.max(np.abs(rec - np.ldexp(x, k))) <= 2.0 ** -49


def test_truncated_digit_product_accuracy():
    rng = np.random.default_rng(2)
    for (M, K, N) in [(40, 1000, 30), (17, 2560, 9)]:
        A = rng.standard_normal((M, K))
        B = rng.standard_normal((N, K))
        A[3] *= 1e-9                       # rows far apart keep their own accuracy
        ref = A @ B.T
        got = model_gemm(A, B)
        scale = np.abs(A) @ np.abs(B).T
        assert np.max(np.abs(got - ref) / scale) < 1e-14
