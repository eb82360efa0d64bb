// Thin QR of small and of tall-skinny complex matrices, and the SVD of small ones.
//
// Small matrices (m n and m min(m, n) at most 4096 elements): one CTA holds the matrix in
// shared memory and runs the Householder QR (LAPACK's zgeqrf / zungqr conventions: reflectors
// H = I - tau v v^H with v_j = 1, beta real with the sign opposite to Re(alpha), Q formed
// by applying the reflectors to the identity in reverse order). No host synchronisation:
// sweeps whose bond dimensions change factor thousands of small matrices of ever new
// shapes, and cuSOLVER's first call for each new shape costs milliseconds.
//
// Tall-skinny matrices (m >= 2n, n <= 64): the gauge moves, the
// predictor and expansion bases and the basis re-orthonormalisations of the tree solvers
// factor matrices of a few to a few hundred thousand rows and at most a few dozen columns,
// where a Householder QR is a sequence of column steps bound by latency (lib/GraftFoundation/
// src/Backend/Backend.jl:602-630 is the reference's QR; it calls LAPACK's Householder QR).
//
// Method: shifted Cholesky QR with two refinement passes, "shifted CholeskyQR3" (Fukaya,
// Kannan, Nakatsukasa, Zhang and Yamamoto, SIAM J. Sci. Comput. 42 (2020) A477-A503):
//   pass 0: G = A^H A + s I with s = 11 (m n + n (n + 1)) u ||A||_F^2, R0 = chol(G), Q0 = A R0^-1
//   pass 1: R1 = chol(Q0^H Q0), Q1 = Q0 R1^-1;  pass 2: R2 = chol(Q1^H Q1), Q = Q1 R2^-1
//   R = R2 R1 R0.
// The Gram matrices are FP64 split-K reductions over the rows (per-CTA partial sums of the
// upper triangle, then a fixed-order sum: deterministic); the n x n Cholesky factors are
// formed on the host; the triangular solves Q = A R^-1 run on the device, row by row. The
// result is accepted only if every Cholesky pivot is positive and the final Q has
// |Q^H Q - I| <= 1e-12 entrywise; otherwise the caller runs the Householder QR. R has a real
// positive diagonal (the Householder QR's diagonal is real with either sign).
#include "gtn_internal.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace {

constexpr int kTsqrMaxN = 64;
constexpr int kTsqrCtas = 4 * 152;

__device__ __forceinline__ void conj_fma(double2& acc, double2 a, double2 b) {  // acc += conj(a) b
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}

// Partial Gram sums: CTA c adds conj(A[r][i]) A[r][j] over its rows for every i <= j
// (entry e of the upper triangle, row-major), staging 2048 / n rows at a time.
__global__ void __launch_bounds__(256) tsqr_gram_partial(const double2* __restrict__ A, int64_t m, int n,
                                                         int64_t rows_per_cta, double2* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char ts_smem[];
  double2* tile = reinterpret_cast<double2*>(ts_smem);
  const int TR = 2048 / n, ne = n * (n + 1) / 2, tid = threadIdx.x;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
  const int64_t r1 = min(m, r0 + rows_per_cta);
  constexpr int EPT = (kTsqrMaxN * (kTsqrMaxN + 1) / 2 + 255) / 256;  // entries per thread
  double2 acc[EPT];
  int ei[EPT], ej[EPT];
#pragma unroll
  for (int q = 0; q < EPT; ++q) {
    acc[q] = make_double2(0.0, 0.0);
    const int e = tid + 256 * q;
    int i = 0, rem = e;  // entry e -> (i, j), i <= j, row-major over the upper triangle
    while (i < n && rem >= n - i) {
      rem -= n - i;
      ++i;
    }
    ei[q] = e < ne ? i : -1;
    ej[q] = e < ne ? i + rem : 0;
  }
  for (int64_t rb = r0; rb < r1; rb += TR) {
    const int rows = (int)min((int64_t)TR, r1 - rb);
    __syncthreads();
    for (int x = tid; x < rows * n; x += 256) tile[x] = A[rb * n + x];
    __syncthreads();
    // The branch encloses a whole row loop, so it cannot be turned into predicated FP64
    // instructions: on this part the FP64 pipe is narrow, and predicated-off FMAs of idle
    // entries would still take its issue slots.  Two partial sums halve the FMA chains.
#pragma unroll
    for (int q = 0; q < EPT; ++q) {
      if (ei[q] >= 0) {
        const double2* ci = tile + ei[q];
        const double2* cj = tile + ej[q];
        double2 a0 = acc[q], a1 = make_double2(0.0, 0.0);
        int r = 0;
        for (; r + 1 < rows; r += 2) {
          conj_fma(a0, ci[r * n], cj[r * n]);
          conj_fma(a1, ci[(r + 1) * n], cj[(r + 1) * n]);
        }
        if (r < rows) conj_fma(a0, ci[r * n], cj[r * n]);
        acc[q] = make_double2(a0.x + a1.x, a0.y + a1.y);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < EPT; ++q)
    if (ei[q] >= 0) part[(int64_t)blockIdx.x * ne + tid + 256 * q] = acc[q];
}

// G (n x n, both halves) = the fixed-order sum of the partials.
__global__ void tsqr_gram_reduce(const double2* __restrict__ part, int nparts, int n, double2* __restrict__ G) {
  const int ne = n * (n + 1) / 2;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int p = 0; p < nparts; ++p) {
      const double2 v = part[(int64_t)p * ne + e];
      s.x += v.x;
      s.y += v.y;
    }
    int i = 0, rem = e;
    while (rem >= n - i) {
      rem -= n - i;
      ++i;
    }
    const int j = i + rem;
    G[i * n + j] = s;
    G[j * n + i] = make_double2(s.x, -s.y);
  }
}

// Q = A R^-1 row by row (R upper triangular): forward substitution
// q_j = (a_j - sum_{i<j} q_i R_ij) / R_jj, one thread per row, in place on the staged rows
// (2048 / n rows at a time); a row-wise triangular solve is backward stable, so A = Q R holds
// to rounding however ill-conditioned R is.
__global__ void __launch_bounds__(256) tsqr_trsm(const double2* __restrict__ A, const double2* __restrict__ Rg,
                                                 int64_t m, int n, int64_t rows_per_cta, double2* __restrict__ Q) {
  extern __shared__ __align__(16) unsigned char ts_smem[];
  const int TR = 2048 / n, tid = threadIdx.x;
  double2* Rs = reinterpret_cast<double2*>(ts_smem);  // [n][n]
  double2* tile = Rs + n * n;                          // [TR][n + 1]
  const int P = n + 1;
  for (int x = tid; x < n * n; x += 256) Rs[x] = Rg[x];
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
  const int64_t r1 = min(m, r0 + rows_per_cta);
  for (int64_t rb = r0; rb < r1; rb += TR) {
    const int rows = (int)min((int64_t)TR, r1 - rb);
    __syncthreads();
    for (int x = tid; x < rows * n; x += 256) {
      const int r = x / n;
      tile[r * P + (x - r * n)] = A[rb * n + x];
    }
    __syncthreads();
    if (tid < rows) {
      double2* q = tile + tid * P;
      for (int j = 0; j < n; ++j) {
        double2 s0 = q[j], s1 = make_double2(0.0, 0.0);
        int i = 0;
        for (; i + 1 < j; i += 2) {  // two partial sums for two independent FMA chains
          const double2 a0 = q[i], b0 = Rs[i * n + j], a1 = q[i + 1], b1 = Rs[(i + 1) * n + j];
          s0.x = fma(-a0.x, b0.x, s0.x);
          s0.x = fma(a0.y, b0.y, s0.x);
          s0.y = fma(-a0.x, b0.y, s0.y);
          s0.y = fma(-a0.y, b0.x, s0.y);
          s1.x = fma(-a1.x, b1.x, s1.x);
          s1.x = fma(a1.y, b1.y, s1.x);
          s1.y = fma(-a1.x, b1.y, s1.y);
          s1.y = fma(-a1.y, b1.x, s1.y);
        }
        if (i < j) {
          const double2 a0 = q[i], b0 = Rs[i * n + j];
          s0.x = fma(-a0.x, b0.x, s0.x);
          s0.x = fma(a0.y, b0.y, s0.x);
          s0.y = fma(-a0.x, b0.y, s0.y);
          s0.y = fma(-a0.y, b0.x, s0.y);
        }
        const double inv = 1.0 / Rs[j * n + j].x;  // R_jj is real and positive
        q[j] = make_double2((s0.x + s1.x) * inv, (s0.y + s1.y) * inv);
      }
    }
    __syncthreads();
    for (int x = tid; x < rows * n; x += 256) {
      const int r = x / n;
      Q[rb * n + x] = tile[r * P + (x - r * n)];
    }
  }
}

// ---- small QR in one CTA -----------------------------------------------------------------
constexpr int kSmallQrElems = 4096;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {  // conj(a) b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// Sum over the CTA (256 threads); every thread gets the result.
__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int w = 0; w < 8; ++w) s += red[w];
  return s;
}

// A (row-major m x n) -> Q (row-major m x k), R (row-major k x n), k = min(m, n).
__global__ void __launch_bounds__(256) small_qr_kernel(const double2* __restrict__ A, int m, int n,
                                                       double2* __restrict__ Q, double2* __restrict__ R) {
  extern __shared__ __align__(16) unsigned char sq_smem[];
  const int k = m < n ? m : n, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double2* a = reinterpret_cast<double2*>(sq_smem);  // column-major m x n: a[c * m + i]
  double2* q = a + (size_t)m * n;                     // column-major m x k
  double2* tau = q + (size_t)m * k;                   // [k]
  double* red = reinterpret_cast<double*>(tau + k);   // [8]
  for (int x = tid; x < m * n; x += 256) {
    const int i = x / n, c = x - i * n;
    a[c * m + i] = A[x];
  }
  __syncthreads();
  for (int j = 0; j < k; ++j) {
    double2* col = a + (size_t)j * m;
    double part = 0.0;
    for (int i = j + 1 + tid; i < m; i += 256) part += col[i].x * col[i].x + col[i].y * col[i].y;
    const double xnorm2 = block_sum(part, red);
    const double2 alpha = col[j];
    double2 t = make_double2(0.0, 0.0);
    if (xnorm2 > 0.0 || alpha.y != 0.0) {
      const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2), alpha.x);
      t = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
      const double2 d = make_double2(alpha.x - beta, alpha.y);  // v_i = x_i / (alpha - beta)
      const double dd = d.x * d.x + d.y * d.y;
      const double2 inv = make_double2(d.x / dd, -d.y / dd);
      __syncthreads();  // every thread has read alpha
      for (int i = j + 1 + tid; i < m; i += 256) col[i] = cmul(col[i], inv);
      if (tid == 0) col[j] = make_double2(beta, 0.0);
    }
    if (tid == 0) tau[j] = t;
    __syncthreads();
    if (t.x != 0.0 || t.y != 0.0) {
      // A(j:, j+1:) -= conj(tau) v (v^H A(j:, j+1:)), one warp per column
      for (int c = j + 1 + warp; c < n; c += 8) {
        double2* cc = a + (size_t)c * m;
        double2 w = lane == 0 ? cc[j] : make_double2(0.0, 0.0);  // v_j = 1
        for (int i = j + 1 + lane; i < m; i += 32) {
          const double2 p = cmulc(col[i], cc[i]);
          w.x += p.x;
          w.y += p.y;
        }
        for (int o = 16; o > 0; o >>= 1) {
          w.x += __shfl_xor_sync(0xffffffffu, w.x, o);
          w.y += __shfl_xor_sync(0xffffffffu, w.y, o);
        }
        const double2 f = cmul(make_double2(t.x, -t.y), w);  // conj(tau) w
        if (lane == 0) cc[j] = make_double2(cc[j].x - f.x, cc[j].y - f.y);
        for (int i = j + 1 + lane; i < m; i += 32) {
          const double2 p = cmul(col[i], f);
          cc[i] = make_double2(cc[i].x - p.x, cc[i].y - p.y);
        }
      }
    }
    __syncthreads();
  }
  // R: the upper triangle of the first k rows
  for (int x = tid; x < k * n; x += 256) {
    const int i = x / n, c = x - i * n;
    R[x] = i <= c ? a[(size_t)c * m + i] : make_double2(0.0, 0.0);
  }
  // Q = H(0) ... H(k-1) I[:, :k], reflectors applied in reverse order
  for (int x = tid; x < m * k; x += 256) {
    const int c = x / m, i = x - c * m;
    q[x] = make_double2(i == c ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  for (int j = k - 1; j >= 0; --j) {
    const double2 t = tau[j];
    if (t.x == 0.0 && t.y == 0.0) continue;
    const double2* col = a + (size_t)j * m;
    for (int c = j + warp; c < k; c += 8) {  // columns < j are untouched (their rows >= j are zero)
      double2* qc = q + (size_t)c * m;
      double2 w = lane == 0 ? qc[j] : make_double2(0.0, 0.0);
      for (int i = j + 1 + lane; i < m; i += 32) {
        const double2 p = cmulc(col[i], qc[i]);
        w.x += p.x;
        w.y += p.y;
      }
      for (int o = 16; o > 0; o >>= 1) {
        w.x += __shfl_xor_sync(0xffffffffu, w.x, o);
        w.y += __shfl_xor_sync(0xffffffffu, w.y, o);
      }
      const double2 f = cmul(t, w);  // H = I - tau v v^H
      if (lane == 0) qc[j] = make_double2(qc[j].x - f.x, qc[j].y - f.y);
      for (int i = j + 1 + lane; i < m; i += 32) {
        const double2 p = cmul(col[i], f);
        qc[i] = make_double2(qc[i].x - p.x, qc[i].y - p.y);
      }
    }
    __syncthreads();
  }
  for (int x = tid; x < m * k; x += 256) {
    const int i = x / k, c = x - i * k;
    Q[x] = q[(size_t)c * m + i];
  }
}

// ---- small SVD in one CTA ----------------------------------------------------------------
// One-sided Jacobi (Hestenes 1958; Demmel and Veselic 1992): the columns of W (br x bc,
// br >= bc; W = A when m >= n, W = A^H otherwise) are rotated pairwise by complex plane
// rotations until every pair is orthogonal to 1e-15 relative to the product of its norms,
// V accumulating the rotations; then sigma_j = |w_j|, and the normalised columns of W are
// the singular vectors of the long side.  Pairs of one round of the round-robin schedule are
// disjoint, so the eight warps rotate them concurrently.  Columns whose norm is exactly zero
// (or below 1e-200 of the largest) are completed by Gram-Schmidt on unit vectors, so that
// the returned factors stay orthonormal for rank-deficient input.
constexpr int kSmallSvdMaxCols = 64, kSmallSvdElems = 4096;

__global__ void __launch_bounds__(256) small_svd_kernel(const double2* __restrict__ A, int m, int n,
                                                        double* __restrict__ S, double2* __restrict__ U,
                                                        double2* __restrict__ Vh) {
  extern __shared__ __align__(16) unsigned char sv_smem[];
  const bool tall = m >= n;
  const int br = tall ? m : n, bc = tall ? n : m, P = (bc + 1) & ~1;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double2* w = reinterpret_cast<double2*>(sv_smem);  // column-major br x bc
  double2* v = w + (size_t)br * bc;                   // column-major bc x bc
  double* nrm = reinterpret_cast<double*>(v + (size_t)bc * bc);
  int* ord = reinterpret_cast<int*>(nrm + bc);
  __shared__ int rotated;
  for (int x = tid; x < m * n; x += 256) {
    const int i = x / n, c = x - i * n;  // A[i][c]
    const double2 a = A[x];
    if (tall) w[(size_t)c * m + i] = a;
    else w[(size_t)i * n + c] = make_double2(a.x, -a.y);  // W = A^H: W[c][i] = conj(A[i][c])
  }
  for (int x = tid; x < bc * bc; x += 256) v[x] = make_double2((x % bc) == (x / bc) ? 1.0 : 0.0, 0.0);
  __syncthreads();
  for (int sweep = 0; sweep < 40; ++sweep) {
    if (tid == 0) rotated = 0;
    __syncthreads();
    for (int r = 0; r < P - 1; ++r) {
      for (int i = warp; i < P / 2; i += 8) {
        int p = i == 0 ? P - 1 : (r + i) % (P - 1), q = (r + P - 1 - i) % (P - 1);
        if (i == 0) q = r % (P - 1);
        if (p > q) { const int t = p; p = q; q = t; }
        if (q >= bc) continue;  // the bye of an odd column count
        double2* wp = w + (size_t)p * br;
        double2* wq = w + (size_t)q * br;
        double al = 0.0, be = 0.0;
        double2 g = make_double2(0.0, 0.0);
        for (int x = lane; x < br; x += 32) {
          const double2 a = wp[x], b = wq[x];
          al += a.x * a.x + a.y * a.y;
          be += b.x * b.x + b.y * b.y;
          g.x += a.x * b.x + a.y * b.y;  // conj(a) b
          g.y += a.x * b.y - a.y * b.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
          al += __shfl_xor_sync(0xffffffffu, al, o);
          be += __shfl_xor_sync(0xffffffffu, be, o);
          g.x += __shfl_xor_sync(0xffffffffu, g.x, o);
          g.y += __shfl_xor_sync(0xffffffffu, g.y, o);
        }
        const double ag = sqrt(g.x * g.x + g.y * g.y);
        if (!(ag > 1e-15 * sqrt(al * be)) || ag == 0.0) continue;  // orthogonal enough (warp-uniform)
        if (lane == 0) rotated = 1;
        const double2 ph = make_double2(g.x / ag, -g.y / ag);  // e^{-i phi}, gamma = |gamma| e^{i phi}
        const double zeta = (be - al) / (2.0 * ag);
        const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
        // w_p' = c w_p - s e^{-i phi} w_q,  w_q' = s w_p + c e^{-i phi} w_q
        for (int x = lane; x < br; x += 32) {
          const double2 a = wp[x], b = wq[x];
          const double2 eb = make_double2(ph.x * b.x - ph.y * b.y, ph.x * b.y + ph.y * b.x);
          wp[x] = make_double2(c * a.x - sn * eb.x, c * a.y - sn * eb.y);
          wq[x] = make_double2(sn * a.x + c * eb.x, sn * a.y + c * eb.y);
        }
        double2* vp = v + (size_t)p * bc;
        double2* vq = v + (size_t)q * bc;
        for (int x = lane; x < bc; x += 32) {
          const double2 a = vp[x], b = vq[x];
          const double2 eb = make_double2(ph.x * b.x - ph.y * b.y, ph.x * b.y + ph.y * b.x);
          vp[x] = make_double2(c * a.x - sn * eb.x, c * a.y - sn * eb.y);
          vq[x] = make_double2(sn * a.x + c * eb.x, sn * a.y + c * eb.y);
        }
      }
      __syncthreads();
    }
    if (!rotated) break;
    __syncthreads();
  }
  for (int j = warp; j < bc; j += 8) {
    double s2 = 0.0;
    for (int x = lane; x < br; x += 32) s2 += w[(size_t)j * br + x].x * w[(size_t)j * br + x].x +
                                             w[(size_t)j * br + x].y * w[(size_t)j * br + x].y;
    for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    if (lane == 0) nrm[j] = sqrt(s2);
  }
  __syncthreads();
  if (tid == 0) {  // descending order (insertion sort, bc <= 64)
    for (int j = 0; j < bc; ++j) ord[j] = j;
    for (int j = 1; j < bc; ++j) {
      const int x = ord[j];
      int l = j - 1;
      while (l >= 0 && nrm[ord[l]] < nrm[x]) {
        ord[l + 1] = ord[l];
        --l;
      }
      ord[l + 1] = x;
    }
  }
  __syncthreads();
  const double thr = nrm[ord[0]] * 1e-200;
  for (int j = warp; j < bc; j += 8) {  // normalise the long-side vectors
    const int c = ord[j];
    const double sg = nrm[c];
    if (sg > thr && sg > 0.0)
      for (int x = lane; x < br; x += 32) {
        const double2 a = w[(size_t)c * br + x];
        w[(size_t)c * br + x] = make_double2(a.x / sg, a.y / sg);
      }
  }
  __syncthreads();
  if (warp == 0) {  // orthonormal completion of the null columns (in singular-value order)
    for (int j = 0; j < bc; ++j) {
      const int c = ord[j];
      if (nrm[c] > thr && nrm[c] > 0.0) continue;
      double2* x = w + (size_t)c * br;
      for (int e = 0; e < br; ++e) {
        for (int t = lane; t < br; t += 32) x[t] = make_double2(t == e ? 1.0 : 0.0, 0.0);
        __syncwarp();
        for (int pass = 0; pass < 2; ++pass)
          for (int l = 0; l < j; ++l) {
            const double2* y = w + (size_t)ord[l] * br;
            double2 d = make_double2(0.0, 0.0);  // y^H x
            for (int t = lane; t < br; t += 32) {
              d.x += y[t].x * x[t].x + y[t].y * x[t].y;
              d.y += y[t].x * x[t].y - y[t].y * x[t].x;
            }
            for (int o = 16; o > 0; o >>= 1) {
              d.x += __shfl_xor_sync(0xffffffffu, d.x, o);
              d.y += __shfl_xor_sync(0xffffffffu, d.y, o);
            }
            for (int t = lane; t < br; t += 32)
              x[t] = make_double2(x[t].x - (d.x * y[t].x - d.y * y[t].y), x[t].y - (d.x * y[t].y + d.y * y[t].x));
            __syncwarp();
          }
        double s2 = 0.0;
        for (int t = lane; t < br; t += 32) s2 += x[t].x * x[t].x + x[t].y * x[t].y;
        for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        if (s2 > 0.25) {
          const double inv = 1.0 / sqrt(s2);
          for (int t = lane; t < br; t += 32) x[t] = make_double2(x[t].x * inv, x[t].y * inv);
          __syncwarp();
          break;
        }
      }
    }
  }
  __syncthreads();
  const int k = bc;
  for (int j = tid; j < k; j += 256) S[j] = nrm[ord[j]] > thr ? nrm[ord[j]] : 0.0;
  if (tall) {  // A = W = U S V^H: U[i][j] = w_ord[j][i], Vh[j][c] = conj(v[c][ord[j]])
    for (int x = tid; x < m * k; x += 256) {
      const int i = x / k, j = x - i * k;
      U[x] = w[(size_t)ord[j] * br + i];
    }
    for (int x = tid; x < k * n; x += 256) {
      const int j = x / n, c = x - j * n;
      const double2 a = v[(size_t)ord[j] * bc + c];
      Vh[x] = make_double2(a.x, -a.y);
    }
  } else {  // A = W^H = V S U_W^H: U[i][j] = v[i][ord[j]], Vh[j][c] = conj(w_ord[j][c])
    for (int x = tid; x < m * k; x += 256) {
      const int i = x / k, j = x - i * k;
      U[x] = v[(size_t)ord[j] * bc + i];
    }
    for (int x = tid; x < k * n; x += 256) {
      const int j = x / n, c = x - j * n;
      const double2 a = w[(size_t)ord[j] * br + c];
      Vh[x] = make_double2(a.x, -a.y);
    }
  }
}

using cplx = std::complex<double>;

// Upper R with G = R^H R (G Hermitian positive definite, row-major n x n); false when a
// pivot is not positive and finite.
bool host_cholesky(const std::vector<cplx>& G, int n, std::vector<cplx>& R) {
  R.assign((size_t)n * n, cplx(0.0, 0.0));
  for (int j = 0; j < n; ++j) {
    double d = G[(size_t)j * n + j].real();
    for (int k = 0; k < j; ++k) d -= std::norm(R[(size_t)k * n + j]);
    if (!(d > 0.0) || !std::isfinite(d)) return false;
    const double rjj = std::sqrt(d);
    R[(size_t)j * n + j] = rjj;
    for (int c = j + 1; c < n; ++c) {
      cplx s = G[(size_t)j * n + c];
      for (int k = 0; k < j; ++k) s -= std::conj(R[(size_t)k * n + j]) * R[(size_t)k * n + c];
      R[(size_t)j * n + c] = s / rjj;
    }
  }
  return true;
}

std::vector<cplx> host_upper_mul(const std::vector<cplx>& X, const std::vector<cplx>& Y, int n) {
  std::vector<cplx> Z((size_t)n * n, cplx(0.0, 0.0));
  for (int i = 0; i < n; ++i)
    for (int k = i; k < n; ++k)
      for (int j = k; j < n; ++j) Z[(size_t)i * n + j] += X[(size_t)i * n + k] * Y[(size_t)k * n + j];
  return Z;
}

}  // namespace

bool tsqr_applies(int64_t m, int64_t n) { return n >= 1 && n <= kTsqrMaxN && m >= 2 * n && m * n >= 4096; }

bool small_svd_applies(int64_t m, int64_t n) {
  return m >= 1 && n >= 1 && std::min(m, n) <= kSmallSvdMaxCols && m * n <= kSmallSvdElems;
}

size_t small_svd_smem(int64_t m, int64_t n) {
  const int64_t k = std::min(m, n);
  return (size_t)(m * n + k * k) * sizeof(double2) + (size_t)k * (sizeof(double) + sizeof(int)) + 16;
}

int svd_small_launch(gtn_ctx ctx, int64_t m, int64_t n, const double2* A, double* S, double2* U, double2* Vh) {
  if (!small_svd_applies(m, n)) return GTN_ERR_UNSUPPORTED;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(small_svd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 140 * 1024) !=
        cudaSuccess)
      return set_err(ctx, GTN_ERR_CUDA, "svd: kernel attribute");
    attr = true;
  }
  small_svd_kernel<<<1, 256, small_svd_smem(m, n), ctx->stream>>>(A, (int)m, (int)n, S, U, Vh);
  ctx->launches++;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GTN_OK : set_err(ctx, GTN_ERR_CUDA, std::string("svd: ") + cudaGetErrorString(e));
}

bool small_qr_applies(int64_t m, int64_t n) {
  return m >= 1 && n >= 1 && m * n <= kSmallQrElems && m * std::min(m, n) <= kSmallQrElems;
}

int qr_small(gtn_ctx ctx, int64_t m, int64_t n, const double2* A, double2* Q, double2* R) {
  if (!small_qr_applies(m, n)) return GTN_ERR_UNSUPPORTED;
  const int64_t k = std::min(m, n);
  const size_t smem = (size_t)(m * n + m * k + k) * sizeof(double2) + 8 * sizeof(double);
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(small_qr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 140 * 1024) !=
        cudaSuccess)
      return set_err(ctx, GTN_ERR_CUDA, "qr: kernel attribute");
    attr = true;
  }
  small_qr_kernel<<<1, 256, smem, ctx->stream>>>(A, (int)m, (int)n, Q, R);
  ctx->launches++;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GTN_OK : set_err(ctx, GTN_ERR_CUDA, std::string("qr: ") + cudaGetErrorString(e));
}

// Returns GTN_OK with Q (m x n) and R (n x n, row-major, device) filled, or
// GTN_ERR_UNSUPPORTED when the matrix is too ill-conditioned for the method (nothing to clean
// up; the caller then runs the Householder QR), or another error code.
int qr_tall_cholesky(gtn_ctx ctx, int64_t m, int64_t n, const double2* A, double2* Q, double2* R) {
  if (!tsqr_applies(m, n)) return GTN_ERR_UNSUPPORTED;
  cudaStream_t s = ctx->stream;
  const int ni = (int)n, ne = ni * (ni + 1) / 2;
  const int TR = 2048 / ni;
  int64_t rpc = (m + kTsqrCtas - 1) / kTsqrCtas;
  rpc = (rpc + TR - 1) / TR * TR;
  const int nparts = (int)((m + rpc - 1) / rpc);
  const size_t bT = ((size_t)m * n * sizeof(double2) + 255) / 256 * 256;
  const size_t bP = ((size_t)nparts * ne * sizeof(double2) + 255) / 256 * 256;
  const size_t bG = ((size_t)n * n * sizeof(double2) + 255) / 256 * 256;
  void* ws = nullptr;
  cudaError_t e = ctx_workspace(ctx, bT + bP + 2 * bG, &ws);
  if (e != cudaSuccess) return set_err(ctx, GTN_ERR_MEMORY, "qr: workspace");
  char* p = static_cast<char*>(ws);
  double2* T = reinterpret_cast<double2*>(p);
  double2* part = reinterpret_cast<double2*>(p + bT);
  double2* dG = reinterpret_cast<double2*>(p + bT + bP);
  double2* dRi = reinterpret_cast<double2*>(p + bT + bP + bG);
  const size_t smem_g = (size_t)TR * n * sizeof(double2);
  const size_t smem_r = (size_t)TR * (n + 1) * sizeof(double2) + (size_t)n * n * sizeof(double2);
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(tsqr_trsm, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024) != cudaSuccess)
      return set_err(ctx, GTN_ERR_CUDA, "qr: kernel attribute");
    attr = true;
  }
  std::vector<double2> hG((size_t)n * n);
  auto gram = [&](const double2* X, std::vector<cplx>& G) -> cudaError_t {
    tsqr_gram_partial<<<nparts, 256, smem_g, s>>>(X, m, ni, rpc, part);
    tsqr_gram_reduce<<<(ne + 255) / 256, 256, 0, s>>>(part, nparts, ni, dG);
    ctx->launches += 2;
    cudaError_t r = cudaMemcpyAsync(hG.data(), dG, (size_t)n * n * sizeof(double2), cudaMemcpyDeviceToHost, s);
    if (r == cudaSuccess) r = cudaStreamSynchronize(s);
    G.resize((size_t)n * n);
    for (size_t x = 0; x < G.size(); ++x) G[x] = cplx(hG[x].x, hG[x].y);
    return r;
  };
  auto solve = [&](const double2* X, const std::vector<cplx>& Rf, double2* Y) -> cudaError_t {
    std::vector<double2> h((size_t)n * n);
    for (size_t x = 0; x < h.size(); ++x) h[x] = make_double2(Rf[x].real(), Rf[x].imag());
    cudaError_t r = cudaMemcpyAsync(dRi, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, s);
    if (r == cudaSuccess) r = cudaStreamSynchronize(s);  // h is released on return
    if (r != cudaSuccess) return r;
    tsqr_trsm<<<nparts, 256, smem_r, s>>>(X, dRi, m, ni, rpc, Y);
    ctx->launches++;
    return cudaGetLastError();
  };
  std::vector<cplx> G, Rp, Rtot;
  // pass 0 (shifted) A -> Q, pass 1 Q -> T, pass 2 T -> Q
  const double2* src[3] = {A, Q, T};
  double2* dst[3] = {Q, T, Q};
  for (int pass = 0; pass < 3; ++pass) {
    e = gram(src[pass], G);
    if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("qr: ") + cudaGetErrorString(e));
    if (pass == 0) {
      double tr = 0.0;
      for (int j = 0; j < ni; ++j) tr += G[(size_t)j * n + j].real();
      const double shift = 11.0 * ((double)m * n + (double)n * (n + 1)) * std::ldexp(1.0, -53) * tr;
      for (int j = 0; j < ni; ++j) G[(size_t)j * n + j] += shift;
    }
    if (!host_cholesky(G, ni, Rp)) return GTN_ERR_UNSUPPORTED;
    e = solve(src[pass], Rp, dst[pass]);
    if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("qr: ") + cudaGetErrorString(e));
    Rtot = pass == 0 ? Rp : host_upper_mul(Rp, Rtot, ni);
  }
  e = gram(Q, G);  // acceptance: Q^H Q = I to 1e-12
  if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("qr: ") + cudaGetErrorString(e));
  for (int i = 0; i < ni; ++i)
    for (int j = 0; j < ni; ++j)
      if (!(std::abs(G[(size_t)i * n + j] - (i == j ? 1.0 : 0.0)) <= 1e-12)) return GTN_ERR_UNSUPPORTED;
  std::vector<double2> hR((size_t)n * n);
  for (size_t x = 0; x < hR.size(); ++x) hR[x] = make_double2(Rtot[x].real(), Rtot[x].imag());
  e = cudaMemcpyAsync(R, hR.data(), hR.size() * sizeof(double2), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("qr: ") + cudaGetErrorString(e));
  return GTN_OK;
}
