// Thin QR of tall-skinny complex matrices (m >= 2n, n <= 64): the gauge moves, the
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
