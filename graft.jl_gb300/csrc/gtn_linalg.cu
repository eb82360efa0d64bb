// FP64 factorisations on device through cuSOLVER runtime calls: truncated SVD for the
// two-site split (lib/GraftFoundation/src/Backend/Backend.jl:466-505,
// lib/GraftContractions/src/Contractions/effective.jl:852-876) and thin QR for the gauge
// moves (Backend.jl:602-630, lib/GraftNetworks/src/Networks/ttns.jl:181-203).
// cuSOLVER is loaded on first use with dlopen so that the rest of the library does not
// depend on it being installed.
#include "gtn_internal.h"

#include <cusolverDn.h>
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace {

struct Solver {
  void* lib = nullptr;
  decltype(&cusolverDnCreate) create = nullptr;
  decltype(&cusolverDnDestroy) destroy = nullptr;
  decltype(&cusolverDnSetStream) set_stream = nullptr;
  decltype(&cusolverDnZgesvd_bufferSize) gesvd_bs = nullptr;
  decltype(&cusolverDnZgesvd) gesvd = nullptr;
  decltype(&cusolverDnZgeqrf_bufferSize) geqrf_bs = nullptr;
  decltype(&cusolverDnZgeqrf) geqrf = nullptr;
  decltype(&cusolverDnZungqr_bufferSize) ungqr_bs = nullptr;
  decltype(&cusolverDnZungqr) ungqr = nullptr;
  decltype(&cusolverDnZheevd_bufferSize) heevd_bs = nullptr;
  decltype(&cusolverDnZheevd) heevd = nullptr;
  bool ok = false;
};

Solver& solver() {
  static Solver s;
  static bool tried = false;
  if (tried) return s;
  tried = true;
  const char* names[] = {"libcusolver.so.12", "libcusolver.so.11", "libcusolver.so.13", "libcusolver.so"};
  for (const char* nm : names) {
    s.lib = dlopen(nm, RTLD_NOW | RTLD_LOCAL);
    if (s.lib) break;
  }
  if (!s.lib) return s;
#define LOAD(field, sym) s.field = reinterpret_cast<decltype(s.field)>(dlsym(s.lib, #sym))
  LOAD(create, cusolverDnCreate);
  LOAD(destroy, cusolverDnDestroy);
  LOAD(set_stream, cusolverDnSetStream);
  LOAD(gesvd_bs, cusolverDnZgesvd_bufferSize);
  LOAD(gesvd, cusolverDnZgesvd);
  LOAD(geqrf_bs, cusolverDnZgeqrf_bufferSize);
  LOAD(geqrf, cusolverDnZgeqrf);
  LOAD(ungqr_bs, cusolverDnZungqr_bufferSize);
  LOAD(ungqr, cusolverDnZungqr);
  LOAD(heevd_bs, cusolverDnZheevd_bufferSize);
  LOAD(heevd, cusolverDnZheevd);
#undef LOAD
  s.ok = s.create && s.destroy && s.set_stream && s.gesvd_bs && s.gesvd && s.geqrf_bs && s.geqrf &&
         s.ungqr_bs && s.ungqr && s.heevd_bs && s.heevd;
  return s;
}

int handle(gtn_ctx ctx, cusolverDnHandle_t* h) {
  Solver& s = solver();
  if (!s.ok) return set_err(ctx, GTN_ERR_UNSUPPORTED, "cuSOLVER could not be loaded");
  if (!ctx->cusolver) {
    cusolverDnHandle_t hh;
    if (s.create(&hh) != CUSOLVER_STATUS_SUCCESS) return set_err(ctx, GTN_ERR_CUDA, "cusolverDnCreate failed");
    ctx->cusolver = hh;
  }
  *h = static_cast<cusolverDnHandle_t>(ctx->cusolver);
  if (s.set_stream(*h, ctx->stream) != CUSOLVER_STATUS_SUCCESS) return set_err(ctx, GTN_ERR_CUDA, "cusolverDnSetStream failed");
  return GTN_OK;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

void linalg_release(gtn_ctx ctx) {
  if (ctx->cusolver) {
    Solver& s = solver();
    if (s.ok) s.destroy(static_cast<cusolverDnHandle_t>(ctx->cusolver));
    ctx->cusolver = nullptr;
  }
}

namespace {

// Truncation rank (truncrank & trunctol & truncerror, Backend.jl:466-483) from singular
// values sorted descending.  tot_sq >= 0 gives the squared Frobenius norm of the whole
// matrix when hs holds only the leading part of its spectrum; the discarded weight of a
// cut at i is then tot_sq minus the kept weight.
int64_t trunc_rank(const std::vector<double>& hs, int64_t maxdim, double atol, double rtol, double dw,
                   double tot_sq = -1.0) {
  const int64_t k = (int64_t)hs.size();
  int64_t r = k;
  if (maxdim > 0) r = std::min(r, maxdim);
  if (atol > 0 || rtol > 0) {
    const double thr = std::max(atol, rtol * hs[0]);
    int64_t c = 0;
    for (int64_t i = 0; i < k; ++i) c += hs[i] > thr ? 1 : 0;
    r = std::min(r, c);
  }
  if (dw > 0 && tot_sq >= 0) {
    std::vector<double> prefix(k + 1, 0.0);
    for (int64_t i = 0; i < k; ++i) prefix[i + 1] = prefix[i] + hs[i] * hs[i];
    int64_t rr = k;
    for (int64_t i = k - 1; i >= 0; --i) {
      if (std::sqrt(std::max(tot_sq - prefix[i], 0.0)) <= dw * std::sqrt(tot_sq)) rr = i;
      else break;
    }
    r = std::min(r, rr);
  } else if (dw > 0) {
    double tot = 0;
    for (double v : hs) tot += v * v;
    double tail = 0;
    int64_t rr = k;
    for (int64_t i = k - 1; i >= 0; --i) {
      tail += hs[i] * hs[i];
      if (std::sqrt(tail) <= dw * std::sqrt(tot)) rr = i;
      else break;
    }
    r = std::min(r, rr);
  }
  return std::max<int64_t>(r, 1);
}

// C[n][m] = sum_k X[m][k] Y'[n][k] for row-major X (M x K) and Y (N x K), Y' = conj(Y) when
// conj_y: FP64 SIMT, or the FP64-grade tensor-core GEMM (a one-shot contraction) when the
// context's linear-algebra precision is GTN_PREC_FP64E.  tmp (M x K when conj_y, SIMT only)
// holds conj(Y).
int linalg_gemm(gtn_ctx ctx, const double2* X, const double2* Y, double2* C, int64_t M, int64_t N, int64_t K,
                bool conj_y, double2* tmp) {
  cudaStream_t s = ctx->stream;
  if (ctx->linalg_prec == GTN_PREC_FP64E) {
    const int ranks[2] = {2, 2};
    const int64_t dims[4] = {M, K, N, K};
    const int labels[4] = {-2, 1, -1, 1};
    const int conj[2] = {0, conj_y ? 1 : 0};
    const int order[2] = {0, 1};
    const void* ops[2] = {X, Y};
    return gtn_contract(ctx, 2, ranks, dims, labels, conj, order, ops, C, GTN_PREC_FP64E);
  }
  const double2* Yc = Y;
  if (conj_y) {
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(tmp, Y, N * K * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    GTN_CUDA_TRY(ctx, launch_conj_inplace(tmp, N * K, s));
    ctx->launches++;
    Yc = tmp;
  }
  GTN_CUDA_TRY(ctx, launch_zgemm_simt(X, Yc, C, M, N, K, s));
  ctx->launches++;
  return GTN_OK;
}

// Thin SVD of a wide row-major m x n matrix (m <= n) through its Gram matrix:
// G = A A^H (FP64 GEMM), G = W diag(w) W^H (cuSOLVER Zheevd), U = W reversed (descending),
// S = sqrt(w), Vh = S^-1 U^H A (FP64 GEMM).  Used above the size where LAPACK-style
// bidiagonalisation (gesvd) is slow on a GPU with a weak FP64 rate; singular values below
// ~1e-8 of the largest lose relative accuracy, far below any kept weight that matters.
int svd_gram(gtn_ctx ctx, cusolverDnHandle_t h, int64_t m, int64_t n, const double2* A, int64_t maxdim,
             double atol, double rtol, double dw, double2* U, double* S, double2* Vh, int64_t* rank,
             double* discarded) {
  Solver& sv = solver();
  cudaStream_t s = ctx->stream;
  int lwork = 0;
  if (sv.heevd_bs(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)m, nullptr, (int)m, nullptr, &lwork) !=
      CUSOLVER_STATUS_SUCCESS)
    return set_err(ctx, GTN_ERR_CUDA, "heevd_bufferSize failed");
  const size_t bC = align256(m * n * sizeof(double2)), bG = align256(m * m * sizeof(double2)),
               bw = align256(m * sizeof(double)), bW = align256((size_t)lwork * sizeof(double2)),
               bT = align256(n * m * sizeof(double2)), bUt = align256(m * m * sizeof(double2));
  void* ws = nullptr;
  GTN_CUDA_TRY(ctx, ctx_workspace(ctx, bC + bG + bw + bW + bT + bUt + 256, &ws));
  char* p = static_cast<char*>(ws);
  double2* conjA = reinterpret_cast<double2*>(p); p += bC;
  double2* G = reinterpret_cast<double2*>(p); p += bG;
  double* w = reinterpret_cast<double*>(p); p += bw;
  double2* work = reinterpret_cast<double2*>(p); p += bW;
  double2* At = reinterpret_cast<double2*>(p); p += bT;
  double2* Ut = reinterpret_cast<double2*>(p); p += bUt;
  int* dinfo = reinterpret_cast<int*>(p);
  // G (column-major) : C[j][i] = sum_l A[i][l] conj(A[j][l]) = G[i][j]
  {
    const int st = linalg_gemm(ctx, A, A, G, m, m, n, true, conjA);
    if (st != GTN_OK) return st;
  }
  if (sv.heevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)m, reinterpret_cast<cuDoubleComplex*>(G),
               (int)m, w, reinterpret_cast<cuDoubleComplex*>(work), lwork, dinfo) != CUSOLVER_STATUS_SUCCESS)
    return set_err(ctx, GTN_ERR_CUDA, "cusolverDnZheevd failed");
  std::vector<double> hw(m);
  int hinfo = 0;
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(hw.data(), w, m * sizeof(double), cudaMemcpyDeviceToHost, s));
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
  GTN_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  if (hinfo != 0) return set_err(ctx, GTN_ERR_CUDA, "heevd info = " + std::to_string(hinfo));
  std::vector<double> hs(m);
  for (int64_t i = 0; i < m; ++i) hs[i] = std::sqrt(std::max(hw[m - 1 - i], 0.0));
  const int64_t r = trunc_rank(hs, maxdim, atol, rtol, dw);
  double disc = 0;
  for (int64_t i = r; i < m; ++i) disc += hs[i] * hs[i];
  for (int64_t i = 0; i < r; ++i) S[i] = hs[i];
  *rank = r;
  if (discarded) *discarded = std::sqrt(disc);
  // U[a][i] = W[a + (m-1-i) m]  (W column-major): gather with a negative column stride
  GroupSpec mg, kg;
  std::memset(&mg, 0, sizeof(mg));
  std::memset(&kg, 0, sizeof(kg));
  mg.n = 1; mg.dim[0] = m; mg.str[0] = 1;
  kg.n = 1; kg.dim[0] = r; kg.str[0] = -m;
  GTN_CUDA_TRY(ctx, launch_gather_c128_to_c128(G + (m - 1) * m, mg, kg, m, r, r, U, s));
  // Ut[i][a] = conj(U[a][i]) : r x m
  mg.dim[0] = r; mg.str[0] = -m;
  kg.dim[0] = m; kg.str[0] = 1;
  GTN_CUDA_TRY(ctx, launch_gather_c128_to_c128(G + (m - 1) * m, mg, kg, r, m, m, Ut, s));
  GTN_CUDA_TRY(ctx, launch_conj_inplace(Ut, r * m, s));
  // Vh[i][l] = sum_a Ut[i][a] A[a][l]: C[nn=i][mm=l] = sum_k X[l][k] Y[i][k], X = A^T, Y = Ut
  GTN_CUDA_TRY(ctx, launch_transpose_c128(A, m, n, At, s));
  {
    const int st = linalg_gemm(ctx, At, Ut, Vh, n, r, m, false, nullptr);
    if (st != GTN_OK) return st;
  }
  // s_i = ||A^H u_i|| (absolute accuracy ~ eps * s_max instead of the eigenvalues'
  // sqrt(eps) * s_max, so singular values of a rank-deficient A come out near zero)
  double* dnorm = reinterpret_cast<double*>(conjA);  // conjA is no longer needed
  GTN_CUDA_TRY(ctx, launch_row_norms(Vh, r, n, dnorm, s));
  ctx->launches += 7;
  std::vector<double> inv(r);
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(inv.data(), dnorm, r * sizeof(double), cudaMemcpyDeviceToHost, s));
  GTN_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  for (int64_t i = 0; i < r; ++i) {
    S[i] = inv[i];
    inv[i] = inv[i] > 0 ? 1.0 / inv[i] : 0.0;
  }
  double* dinv = dnorm;
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(dinv, inv.data(), r * sizeof(double), cudaMemcpyHostToDevice, s));
  GTN_CUDA_TRY(ctx, launch_diag_scale(Vh, r, n, dinv, 1, s));
  ctx->launches++;
  return gtn_ctx_sync(ctx);
}

// Device buffers of one call, freed (after the stream drains) on every return path.
struct CallBuffers {
  cudaStream_t s;
  std::vector<void*> ptrs;
  explicit CallBuffers(cudaStream_t st) : s(st) {}
  ~CallBuffers() {
    cudaStreamSynchronize(s);
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  T* get(size_t count) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
};

// Subspace dimension of the subspace-iteration route for a wide m x n matrix (m <= n)
// truncated to maxdim, or 0 when the Gram route is the better choice: the route pays off
// when maxdim plus its oversampling is small next to m.  GTN_SVD_SUBSPACE=0 switches it off.
int64_t subspace_dim(int64_t m, int64_t maxdim) {
  const char* env = std::getenv("GTN_SVD_SUBSPACE");
  if (env && env[0] == '0') return 0;
  if (maxdim <= 0) return 0;
  const int64_t kk = maxdim + std::max<int64_t>(32, maxdim / 2);
  return 4 * kk <= m ? kk : 0;
}

// Truncated SVD of a wide row-major m x n matrix (m <= n) by subspace iteration: the
// randomised range finder with power iterations (Halko, Martinsson and Tropp, SIAM Review
// 2011, algorithm 4.4) on a kk-dimensional subspace, iterated until the leading maxdim
// Rayleigh-Ritz singular values stop moving (1e-13 of the largest).  Their vectors have
// then converged to ~1e-7 in angle; the split is the exact orthogonal projection of A on
// the kept left vectors whatever the angle.  Every product is an FP64 SIMT GEMM of
// m x n x kk (two per iteration) instead of the m x m x n Gram product and an m x m
// eigenproblem.  *done is false when the values have not settled within the iteration
// cap, or when the truncation would keep the whole subspace; the caller then takes the
// Gram route.  Outputs and conventions as svd_gram.
int svd_subspace(gtn_ctx ctx, cusolverDnHandle_t h, int64_t m, int64_t n, const double2* A, int64_t maxdim,
                 int64_t kk, double atol, double rtol, double dw, double2* U, double* S, double2* Vh,
                 int64_t* rank, double* discarded, bool* done) {
  *done = false;
  Solver& sv = solver();
  cudaStream_t s = ctx->stream;
  const int ik = (int)kk;
  const int max_it = (int)std::max<int64_t>(4, std::min<int64_t>(40, m / (4 * kk)));
  // squared Frobenius norm of A
  const int nblk = multidot_blocks(ctx);
  GTN_CUDA_TRY(ctx, ctx_red(ctx, (size_t)nblk + 8));
  GTN_CUDA_TRY(ctx, launch_multidot(A, 0, 1, A, m * n, ctx->d_red, ctx->d_red + 8, nblk, s));
  double2 tot2;
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(&tot2, ctx->d_red, sizeof(double2), cudaMemcpyDeviceToHost, s));
  GTN_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  const double tot = tot2.x;
  const int sk1 = gemm_splitk_slices(m, kk, n), sk2 = gemm_splitk_slices(n, kk, m);
  const size_t pcap = (size_t)std::max(sk1 > 1 ? sk1 : 0, sk2 > 1 ? sk2 : 0) * std::max(m, n) * kk;
  CallBuffers buf(s);
  double2* Ah = buf.get<double2>(m * n);     // conj(A)^T, n x m
  double2* Qt = buf.get<double2>(kk * m);    // basis of the range, rows of length m
  double2* Zt = buf.get<double2>(kk * n);    // Z = A^H Q, rows of length n
  double2* Zc = buf.get<double2>(kk * n);    // conj(Z) rows, later Z^T
  double2* Gc = buf.get<double2>(kk * kk);   // Z^H Z (column-major), then its eigenvectors
  double2* Wr = buf.get<double2>(kk * kk);
  double2* Qr = buf.get<double2>(m * kk);    // Q row-major m x kk
  double* w = buf.get<double>(kk);
  double* dnorm = buf.get<double>(kk);
  double2* tau = buf.get<double2>(kk);
  double2* P = pcap ? buf.get<double2>(pcap) : nullptr;
  int* dinfo = buf.get<int>(1);
  if (!Ah || !Qt || !Zt || !Zc || !Gc || !Wr || !Qr || !w || !dnorm || !tau || !dinfo || (pcap && !P))
    return set_err(ctx, GTN_ERR_MEMORY, "svd subspace: staging allocation failed");
  int lq = 0, lq2 = 0, lu = 0, lu2 = 0, le = 0;
  if (sv.geqrf_bs(h, (int)m, ik, reinterpret_cast<cuDoubleComplex*>(Qt), (int)m, &lq) != CUSOLVER_STATUS_SUCCESS ||
      sv.geqrf_bs(h, (int)n, ik, reinterpret_cast<cuDoubleComplex*>(Zt), (int)n, &lq2) != CUSOLVER_STATUS_SUCCESS ||
      sv.ungqr_bs(h, (int)m, ik, ik, reinterpret_cast<cuDoubleComplex*>(Qt), (int)m,
                  reinterpret_cast<cuDoubleComplex*>(tau), &lu) != CUSOLVER_STATUS_SUCCESS ||
      sv.ungqr_bs(h, (int)n, ik, ik, reinterpret_cast<cuDoubleComplex*>(Zt), (int)n,
                  reinterpret_cast<cuDoubleComplex*>(tau), &lu2) != CUSOLVER_STATUS_SUCCESS ||
      sv.heevd_bs(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, ik, reinterpret_cast<cuDoubleComplex*>(Gc), ik,
                  w, &le) != CUSOLVER_STATUS_SUCCESS)
    return set_err(ctx, GTN_ERR_CUDA, "svd subspace: bufferSize failed");
  const int lwork = std::max({lq, lq2, lu, lu2, le, 1});
  double2* work = buf.get<double2>(lwork);
  if (!work) return set_err(ctx, GTN_ERR_MEMORY, "svd subspace: workspace allocation failed");
  auto gemm = [&](const double2* X, const double2* Y, double2* C, int64_t M, int64_t N, int64_t K) {
    const int sl = gemm_splitk_slices(M, N, K);
    ctx->launches += sl > 1 ? 2 : 1;
    if (sl > 1 && P && (size_t)sl * M * N <= pcap) return launch_zgemm_simt_splitk(X, Y, C, M, N, K, sl, P, s);
    return launch_zgemm_simt(X, Y, C, M, N, K, s);
  };
  // Householder QR of a column-major rows x kk block (a row-major kk x rows one), in place: Q
  auto orth = [&](double2* Y, int64_t rows) -> int {
    if (sv.geqrf(h, (int)rows, ik, reinterpret_cast<cuDoubleComplex*>(Y), (int)rows,
                 reinterpret_cast<cuDoubleComplex*>(tau), reinterpret_cast<cuDoubleComplex*>(work), lwork,
                 dinfo) != CUSOLVER_STATUS_SUCCESS ||
        sv.ungqr(h, (int)rows, ik, ik, reinterpret_cast<cuDoubleComplex*>(Y), (int)rows,
                 reinterpret_cast<cuDoubleComplex*>(tau), reinterpret_cast<cuDoubleComplex*>(work), lwork,
                 dinfo) != CUSOLVER_STATUS_SUCCESS)
      return set_err(ctx, GTN_ERR_CUDA, "svd subspace: QR failed");
    return GTN_OK;
  };
  GTN_CUDA_TRY(ctx, launch_transpose_c128(A, m, n, Ah, s));
  GTN_CUDA_TRY(ctx, launch_conj_inplace(Ah, m * n, s));
  GTN_CUDA_TRY(ctx, launch_fill_uniform_c128(Zt, kk * n, 0x5eed5eedull + (uint64_t)m * 131 + (uint64_t)n, s));
  ctx->launches += 3;
  GTN_CUDA_TRY(ctx, gemm(A, Zt, Qt, m, kk, n));  // Y = A Omega
  int st = orth(Qt, m);
  if (st != GTN_OK) return st;
  std::vector<double> hw(kk), sig(kk), prev;
  const int64_t rchk = std::min(maxdim, kk);
  bool settled = false;
  for (int it = 0; it <= max_it; ++it) {
    GTN_CUDA_TRY(ctx, gemm(Ah, Qt, Zt, n, kk, m));  // Z = A^H Q
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(Zc, Zt, kk * n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    GTN_CUDA_TRY(ctx, launch_conj_inplace(Zc, kk * n, s));
    GTN_CUDA_TRY(ctx, gemm(Zc, Zt, Gc, kk, kk, n));  // Z^H Z, column-major
    ctx->launches++;
    if (sv.heevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, ik, reinterpret_cast<cuDoubleComplex*>(Gc), ik, w,
                 reinterpret_cast<cuDoubleComplex*>(work), lwork, dinfo) != CUSOLVER_STATUS_SUCCESS)
      return set_err(ctx, GTN_ERR_CUDA, "svd subspace: heevd failed");
    int hinfo = 0;
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(hw.data(), w, kk * sizeof(double), cudaMemcpyDeviceToHost, s));
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
    GTN_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (hinfo != 0) return set_err(ctx, GTN_ERR_CUDA, "svd subspace: info = " + std::to_string(hinfo));
    for (int64_t i = 0; i < kk; ++i) sig[i] = std::sqrt(std::max(hw[kk - 1 - i], 0.0));
    if (!prev.empty()) {
      double dmax = 0;
      for (int64_t i = 0; i < rchk; ++i) dmax = std::max(dmax, std::fabs(sig[i] - prev[i]));
      if (dmax <= 1e-13 * sig[0]) {
        settled = true;
        break;
      }
    }
    if (it == max_it) break;
    prev = sig;
    st = orth(Zt, n);  // P = orth(Z)
    if (st != GTN_OK) return st;
    GTN_CUDA_TRY(ctx, gemm(A, Zt, Qt, m, kk, n));  // Y = A P
    st = orth(Qt, m);
    if (st != GTN_OK) return st;
  }
  if (!settled) return GTN_OK;
  const int64_t r = trunc_rank(sig, maxdim, atol, rtol, dw, tot);
  if (r >= kk) return GTN_OK;
  double kept = 0;
  for (int64_t i = 0; i < r; ++i) kept += sig[i] * sig[i];
  *rank = r;
  if (discarded) *discarded = std::sqrt(std::max(tot - kept, 0.0));
  // Wr[c][j] = W[j][kk-1-c]: eigenvectors in descending order, one per row
  GroupSpec mg, kg;
  std::memset(&mg, 0, sizeof(mg));
  std::memset(&kg, 0, sizeof(kg));
  mg.n = 1; mg.dim[0] = r; mg.str[0] = -kk;
  kg.n = 1; kg.dim[0] = kk; kg.str[0] = 1;
  GTN_CUDA_TRY(ctx, launch_gather_c128_to_c128(Gc + (kk - 1) * kk, mg, kg, r, kk, kk, Wr, s));
  // U = Q W (m x r)
  GTN_CUDA_TRY(ctx, launch_transpose_c128(Qt, kk, m, Qr, s));
  GTN_CUDA_TRY(ctx, gemm(Wr, Qr, U, r, m, kk));
  // Vh = S^-1 W^H Q^H A = S^-1 conj(W^T Z^T): C[c][l] = sum_j Z^T[l][j] Wr[c][j], conjugated
  GTN_CUDA_TRY(ctx, launch_transpose_c128(Zt, kk, n, Zc, s));
  GTN_CUDA_TRY(ctx, gemm(Zc, Wr, Vh, n, r, kk));
  GTN_CUDA_TRY(ctx, launch_conj_inplace(Vh, r * n, s));
  GTN_CUDA_TRY(ctx, launch_row_norms(Vh, r, n, dnorm, s));
  ctx->launches += 5;
  std::vector<double> inv(r);
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(inv.data(), dnorm, r * sizeof(double), cudaMemcpyDeviceToHost, s));
  GTN_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  for (int64_t i = 0; i < r; ++i) {
    S[i] = inv[i];
    inv[i] = inv[i] > 0 ? 1.0 / inv[i] : 0.0;
  }
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(dnorm, inv.data(), r * sizeof(double), cudaMemcpyHostToDevice, s));
  GTN_CUDA_TRY(ctx, launch_diag_scale(Vh, r, n, dnorm, 1, s));
  ctx->launches++;
  st = gtn_ctx_sync(ctx);
  if (st == GTN_OK) *done = true;
  return st;
}

// Thin truncated SVD of a wide row-major m x n matrix (m <= n): the subspace-iteration
// route where maxdim is small next to m and its values settle, else the Gram route.
int svd_wide(gtn_ctx ctx, cusolverDnHandle_t h, int64_t m, int64_t n, const double2* A, int64_t maxdim,
             double atol, double rtol, double dw, double2* U, double* S, double2* Vh, int64_t* rank,
             double* discarded) {
  const int64_t kk = subspace_dim(m, maxdim);
  if (kk > 0) {
    bool done = false;
    const int st = svd_subspace(ctx, h, m, n, A, maxdim, kk, atol, rtol, dw, U, S, Vh, rank, discarded, &done);
    if (st != GTN_OK || done) return st;
  }
  return svd_gram(ctx, h, m, n, A, maxdim, atol, rtol, dw, U, S, Vh, rank, discarded);
}

constexpr int64_t kGramMin = 384;

}  // namespace

// Rows of Vh (r x n, r <= n) made orthonormal.  The Gram route forms Vh = S^-1 U^H A, whose
// rows for singular values near sqrt(eps) * s_max (or zero) lose orthogonality; a thin
// Householder QR Vh^H = Q R restores it.  Where the rows were already orthonormal Q equals
// them up to the phase of R's diagonal, which is put back (Vh = (Q diag(ph))^H); for the
// rest Q completes the orthonormal set, so U S Vh changes only at the level of those
// singular values.
static int orthonormalize_rows(gtn_ctx ctx, int64_t r, int64_t n, double2* Vh) {
  cudaStream_t s = ctx->stream;
  double2 *Y = nullptr, *Q = nullptr, *R = nullptr, *ph = nullptr;
  if (cudaMalloc(&Y, n * r * sizeof(double2)) != cudaSuccess || cudaMalloc(&Q, n * r * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&R, r * r * sizeof(double2)) != cudaSuccess || cudaMalloc(&ph, r * sizeof(double2)) != cudaSuccess) {
    cudaFree(Y);
    cudaFree(Q);
    cudaFree(R);
    return set_err(ctx, GTN_ERR_MEMORY, "svd: orthonormalisation staging");
  }
  int st = GTN_OK;
  cudaError_t e = launch_transpose_c128(Vh, r, n, Y, s);
  if (e == cudaSuccess) e = launch_conj_inplace(Y, n * r, s);
  ctx->launches += 2;
  if (e != cudaSuccess) st = set_err(ctx, GTN_ERR_CUDA, cudaGetErrorString(e));
  if (st == GTN_OK) st = gtn_qr(ctx, n, r, Y, Q, R);
  std::vector<double2> d(r);
  if (st == GTN_OK) {
    e = cudaMemcpy2DAsync(d.data(), sizeof(double2), R, (r + 1) * sizeof(double2), sizeof(double2), r,
                          cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = set_err(ctx, GTN_ERR_CUDA, cudaGetErrorString(e));
  }
  if (st == GTN_OK) {
    for (auto& v : d) {
      const double a = std::hypot(v.x, v.y);
      v = a > 0 ? make_double2(v.x / a, v.y / a) : make_double2(1.0, 0.0);
    }
    e = cudaMemcpyAsync(ph, d.data(), r * sizeof(double2), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_transpose_c128(Q, n, r, Vh, s);
    if (e == cudaSuccess) e = launch_row_phase_conj(Vh, r, n, ph, s);
    ctx->launches += 2;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = set_err(ctx, GTN_ERR_CUDA, cudaGetErrorString(e));
  }
  cudaStreamSynchronize(s);
  cudaFree(Y);
  cudaFree(Q);
  cudaFree(R);
  cudaFree(ph);
  return st;
}

extern "C" int gtn_svd_trunc(gtn_ctx ctx, int64_t m, int64_t n, const void* A, int64_t maxdim, double atol,
                             double rtol, double discarded_weight, void* U, double* S, void* Vh,
                             int64_t* rank, double* discarded) {
  if (!ctx || !A || !U || !S || !Vh || !rank || m <= 0 || n <= 0)
    return set_err(ctx, GTN_ERR_INVALID, "gtn_svd_trunc: bad argument");
  if (m > INT32_MAX || n > INT32_MAX) return set_err(ctx, GTN_ERR_UNSUPPORTED, "gtn_svd_trunc: matrix too large");
  cusolverDnHandle_t h;
  int st = handle(ctx, &h);
  if (st != GTN_OK) return st;
  Solver& sv = solver();
  cudaStream_t s = ctx->stream;
  const int64_t k = std::min(m, n);
  if (k >= kGramMin) {
    if (m <= n) {
      st = svd_wide(ctx, h, m, n, static_cast<const double2*>(A), maxdim, atol, rtol, discarded_weight,
                    static_cast<double2*>(U), S, static_cast<double2*>(Vh), rank, discarded);
      return st == GTN_OK ? orthonormalize_rows(ctx, *rank, n, static_cast<double2*>(Vh)) : st;
    }
    // tall: B = A^T (n x m, wide) = U_B S Vh_B  =>  U_A = Vh_B^T, Vh_A = U_B^T
    double2* B = nullptr;
    double2 *UB = nullptr, *VB = nullptr;
    if (cudaMalloc(&B, m * n * sizeof(double2)) != cudaSuccess || cudaMalloc(&UB, n * k * sizeof(double2)) != cudaSuccess ||
        cudaMalloc(&VB, k * m * sizeof(double2)) != cudaSuccess) {
      cudaFree(B);
      cudaFree(UB);
      return set_err(ctx, GTN_ERR_MEMORY, "svd transpose staging");
    }
    st = GTN_OK;
    cudaError_t e = launch_transpose_c128(static_cast<const double2*>(A), m, n, B, s);
    if (e == cudaSuccess) st = svd_wide(ctx, h, n, m, B, maxdim, atol, rtol, discarded_weight, UB, S, VB, rank, discarded);
    else st = set_err(ctx, GTN_ERR_CUDA, cudaGetErrorString(e));
    if (st == GTN_OK) st = orthonormalize_rows(ctx, *rank, m, VB);
    if (st == GTN_OK) {
      const int64_t r = *rank;
      e = launch_transpose_c128(VB, r, m, static_cast<double2*>(U), s);       // (r x m)^T = m x r
      if (e == cudaSuccess) e = launch_transpose_c128(UB, n, r, static_cast<double2*>(Vh), s);  // (n x r)^T
      ctx->launches += 3;
      if (e != cudaSuccess) st = set_err(ctx, GTN_ERR_CUDA, cudaGetErrorString(e));
      else st = gtn_ctx_sync(ctx);
    }
    cudaStreamSynchronize(s);
    cudaFree(B);
    cudaFree(UB);
    cudaFree(VB);
    return st;
  }
  const char* ssv = std::getenv("GTN_SMALL_SVD");
  if (small_svd_applies(m, n) && !(ssv && ssv[0] == '0')) {  // one-CTA Jacobi: no per-shape set-up
    const size_t bU = align256(m * k * sizeof(double2)), bV = align256(k * n * sizeof(double2)),
                 bS = align256(k * sizeof(double));
    void* ws = nullptr;
    GTN_CUDA_TRY(ctx, ctx_workspace(ctx, bU + bV + bS, &ws));
    double2* dU = static_cast<double2*>(ws);
    double2* dV = reinterpret_cast<double2*>(static_cast<char*>(ws) + bU);
    double* dS = reinterpret_cast<double*>(static_cast<char*>(ws) + bU + bV);
    st = svd_small_launch(ctx, m, n, static_cast<const double2*>(A), dS, dU, dV);
    if (st != GTN_OK) return st;
    std::vector<double> hs(k);
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(hs.data(), dS, k * sizeof(double), cudaMemcpyDeviceToHost, s));
    GTN_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    const int64_t r = trunc_rank(hs, maxdim, atol, rtol, discarded_weight);
    double disc = 0;
    for (int64_t i = r; i < k; ++i) disc += hs[i] * hs[i];
    for (int64_t i = 0; i < r; ++i) S[i] = hs[i];
    *rank = r;
    if (discarded) *discarded = std::sqrt(disc);
    GTN_CUDA_TRY(ctx, cudaMemcpy2DAsync(U, r * sizeof(double2), dU, k * sizeof(double2), r * sizeof(double2), m,
                                        cudaMemcpyDeviceToDevice, s));
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(Vh, dV, r * n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    return gtn_ctx_sync(ctx);
  }
  // Column-major problem B (rows >= cols): for n >= m, B = A^T (the same buffer); else B =
  // column-major copy of A (a transpose).
  const bool wide = n >= m;
  const int64_t br = wide ? n : m, bc = wide ? m : n;  // B is br x bc, br >= bc
  int lwork = 0;
  if (sv.gesvd_bs(h, (int)br, (int)bc, &lwork) != CUSOLVER_STATUS_SUCCESS)
    return set_err(ctx, GTN_ERR_CUDA, "gesvd_bufferSize failed");
  const size_t bB = align256(br * bc * sizeof(double2)), bU = align256(br * k * sizeof(double2)),
               bVT = align256(k * bc * sizeof(double2)), bS = align256(k * sizeof(double)),
               bW = align256((size_t)lwork * sizeof(double2)), bR = align256(k * sizeof(double)),
               bT = align256(std::max(m * k, k * n) * sizeof(double2));
  void* ws = nullptr;
  GTN_CUDA_TRY(ctx, ctx_workspace(ctx, bB + bU + bVT + bS + bW + bR + bT + 256, &ws));
  char* p = static_cast<char*>(ws);
  double2* dB = reinterpret_cast<double2*>(p); p += bB;
  double2* dU = reinterpret_cast<double2*>(p); p += bU;
  double2* dVT = reinterpret_cast<double2*>(p); p += bVT;
  double* dS = reinterpret_cast<double*>(p); p += bS;
  double2* dW = reinterpret_cast<double2*>(p); p += bW;
  double* dR = reinterpret_cast<double*>(p); p += bR;
  double2* dT = reinterpret_cast<double2*>(p); p += bT;
  int* dinfo = reinterpret_cast<int*>(p);
  if (wide) {
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(dB, A, m * n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  } else {
    GTN_CUDA_TRY(ctx, launch_transpose_c128(static_cast<const double2*>(A), m, n, dB, s));  // row-major n x m
    ctx->launches++;
  }
  if (sv.gesvd(h, 'S', 'S', (int)br, (int)bc, reinterpret_cast<cuDoubleComplex*>(dB), (int)br, dS,
               reinterpret_cast<cuDoubleComplex*>(dU), (int)br, reinterpret_cast<cuDoubleComplex*>(dVT), (int)k,
               reinterpret_cast<cuDoubleComplex*>(dW), lwork, dR, dinfo) != CUSOLVER_STATUS_SUCCESS)
    return set_err(ctx, GTN_ERR_CUDA, "cusolverDnZgesvd failed");
  int hinfo = 0;
  std::vector<double> hs(k);
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(hs.data(), dS, k * sizeof(double), cudaMemcpyDeviceToHost, s));
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
  GTN_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  if (hinfo != 0) return set_err(ctx, GTN_ERR_CUDA, "gesvd info = " + std::to_string(hinfo));
  const int64_t r = trunc_rank(hs, maxdim, atol, rtol, discarded_weight);
  double disc = 0;
  for (int64_t i = r; i < k; ++i) disc += hs[i] * hs[i];
  for (int64_t i = 0; i < r; ++i) S[i] = hs[i];
  *rank = r;
  if (discarded) *discarded = std::sqrt(disc);
  double2* Uo = static_cast<double2*>(U);
  double2* Vo = static_cast<double2*>(Vh);
  if (wide) {
    // U_A (m x k row-major) = VT buffer; Vh_A (k x n row-major) = U buffer.
    GTN_CUDA_TRY(ctx, cudaMemcpy2DAsync(Uo, r * sizeof(double2), dVT, k * sizeof(double2), r * sizeof(double2), m,
                                        cudaMemcpyDeviceToDevice, s));
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(Vo, dU, r * n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  } else {
    // A = U S VT column-major: U (m x k, ld m) -> row-major via transpose of the k x m
    // row-major view; VT (k x n, ld k) -> row-major via transpose of the n x k view.
    GTN_CUDA_TRY(ctx, launch_transpose_c128(dU, k, m, dT, s));  // dT: m x k row-major
    GTN_CUDA_TRY(ctx, cudaMemcpy2DAsync(Uo, r * sizeof(double2), dT, k * sizeof(double2), r * sizeof(double2), m,
                                        cudaMemcpyDeviceToDevice, s));
    GTN_CUDA_TRY(ctx, launch_transpose_c128(dVT, n, k, dT, s));  // dT: k x n row-major
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(Vo, dT, r * n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    ctx->launches += 2;
  }
  return gtn_ctx_sync(ctx);
}

extern "C" int gtn_qr(gtn_ctx ctx, int64_t m, int64_t n, const void* A, void* Q, void* R) {
  if (!ctx || !A || !Q || !R || m <= 0 || n <= 0) return set_err(ctx, GTN_ERR_INVALID, "gtn_qr: bad argument");
  if (m > INT32_MAX || n > INT32_MAX) return set_err(ctx, GTN_ERR_UNSUPPORTED, "gtn_qr: matrix too large");
  const char* ts = std::getenv("GTN_TSQR");
  const bool fast = !(ts && ts[0] == '0');
  if (fast && small_qr_applies(m, n))  // small: Householder in one CTA
    return qr_small(ctx, m, n, static_cast<const double2*>(A), static_cast<double2*>(Q), static_cast<double2*>(R));
  if (fast && tsqr_applies(m, n)) {  // tall-skinny: Cholesky QR, else Householder below
    const int r = qr_tall_cholesky(ctx, m, n, static_cast<const double2*>(A), static_cast<double2*>(Q),
                                   static_cast<double2*>(R));
    if (r != GTN_ERR_UNSUPPORTED) return r;
  }
  cusolverDnHandle_t h;
  int st = handle(ctx, &h);
  if (st != GTN_OK) return st;
  Solver& sv = solver();
  cudaStream_t s = ctx->stream;
  const int64_t k = std::min(m, n);
  int l1 = 0, l2 = 0;
  const size_t bA = align256(m * n * sizeof(double2)), btau = align256(k * sizeof(double2)),
               bT = align256(std::max(m * n, m * k) * sizeof(double2));
  void* ws = nullptr;
  GTN_CUDA_TRY(ctx, ctx_workspace(ctx, bA + btau + bT + 256, &ws));  // sized again below with lwork
  char* p = static_cast<char*>(ws);
  double2* dA = reinterpret_cast<double2*>(p);
  GTN_CUDA_TRY(ctx, launch_transpose_c128(static_cast<const double2*>(A), m, n, dA, s));  // column-major m x n
  ctx->launches++;
  if (sv.geqrf_bs(h, (int)m, (int)n, reinterpret_cast<cuDoubleComplex*>(dA), (int)m, &l1) != CUSOLVER_STATUS_SUCCESS ||
      sv.ungqr_bs(h, (int)m, (int)k, (int)k, reinterpret_cast<cuDoubleComplex*>(dA), (int)m, nullptr, &l2) !=
          CUSOLVER_STATUS_SUCCESS)
    return set_err(ctx, GTN_ERR_CUDA, "QR bufferSize failed");
  const size_t bW = align256((size_t)std::max(l1, l2) * sizeof(double2));
  const size_t need = bA + btau + bT + bW + 256;
  if (need > ctx->ws_bytes) {
    // grow while preserving the transposed copy
    void* tmp = nullptr;
    GTN_CUDA_TRY(ctx, cudaMalloc(&tmp, bA));
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(tmp, dA, m * n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    GTN_CUDA_TRY(ctx, ctx_workspace(ctx, need, &ws));
    p = static_cast<char*>(ws);
    dA = reinterpret_cast<double2*>(p);
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(dA, tmp, m * n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    GTN_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    cudaFree(tmp);
  }
  p = static_cast<char*>(ws) + bA;
  double2* dtau = reinterpret_cast<double2*>(p); p += btau;
  double2* dT = reinterpret_cast<double2*>(p); p += bT;
  double2* dW = reinterpret_cast<double2*>(p); p += bW;
  int* dinfo = reinterpret_cast<int*>(p);
  if (sv.geqrf(h, (int)m, (int)n, reinterpret_cast<cuDoubleComplex*>(dA), (int)m, reinterpret_cast<cuDoubleComplex*>(dtau),
               reinterpret_cast<cuDoubleComplex*>(dW), std::max(l1, l2), dinfo) != CUSOLVER_STATUS_SUCCESS)
    return set_err(ctx, GTN_ERR_CUDA, "cusolverDnZgeqrf failed");
  // R: rows 0..k-1 of the row-major form of the factored matrix, lower part zeroed
  GTN_CUDA_TRY(ctx, launch_transpose_c128(dA, n, m, dT, s));  // dT: m x n row-major
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(R, dT, k * n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  GTN_CUDA_TRY(ctx, launch_zero_lower(static_cast<double2*>(R), k, n, s));
  if (sv.ungqr(h, (int)m, (int)k, (int)k, reinterpret_cast<cuDoubleComplex*>(dA), (int)m,
               reinterpret_cast<cuDoubleComplex*>(dtau), reinterpret_cast<cuDoubleComplex*>(dW), std::max(l1, l2),
               dinfo) != CUSOLVER_STATUS_SUCCESS)
    return set_err(ctx, GTN_ERR_CUDA, "cusolverDnZungqr failed");
  GTN_CUDA_TRY(ctx, launch_transpose_c128(dA, k, m, static_cast<double2*>(Q), s));  // Q: m x k row-major
  ctx->launches += 3;
  int hinfo = 0;
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
  st = gtn_ctx_sync(ctx);
  if (st != GTN_OK) return st;
  if (hinfo != 0) return set_err(ctx, GTN_ERR_CUDA, "QR info = " + std::to_string(hinfo));
  return GTN_OK;
}
