// Device-resident Krylov solvers: the eigsolve / exponentiate hooks of the reference
// (lib/GraftGroundState/src/GroundState/GroundState.jl:25-39,
//  lib/GraftEvolution/src/Evolution/Evolution.jl:54-68).
//
// Krylov vectors live in HBM as complex FP64.  Each Lanczos step applies the map (in its
// precision mode), takes the local three-term step against the two newest vectors in FP64,
// then one reorthogonalisation pass against the whole basis (FP32 products for mixed-
// precision maps, FP64 otherwise; a second FP64 pass when the DGKS test asks for it), then
// normalises.  The first step of an expansion runs two full FP64 passes.  Only the projected
// coefficients cross to the host; the small symmetric eigenproblem is solved there by
// cyclic Jacobi rotations.  The eigensolver restarts thick: the lowest Ritz vectors are
// rotated in place at the front of the basis and the expansion continues from the residual
// direction.  Maps without the Hermitian trait take the Arnoldi exponential (two FP64
// passes per step, exp of the Hessenberg matrix on the host).
#include "gtn_internal.h"

#include <algorithm>
#include <cmath>
#include <complex>

namespace {

constexpr int kMaxKrylov = 63;

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major A, destroyed).
// On return w holds eigenvalues ascending and V's columns the matching eigenvectors.
void jacobi_eig(int n, std::vector<double>& A, std::vector<double>& w, std::vector<double>& V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  auto a = [&](int i, int j) -> double& { return A[(size_t)i * n + j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, diag = 0;
    for (int p = 0; p < n; ++p) {
      diag += a(p, p) * a(p, p);
      for (int q = p + 1; q < n; ++q) off += a(p, q) * a(p, q);
    }
    if (off <= 1e-32 * (diag + 1e-300)) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a(p, q);
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (a(q, q) - a(p, p)) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // columns p, q
          const double akp = a(k, p), akq = a(k, q);
          a(k, p) = c * akp - s * akq;
          a(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows p, q
          const double apk = a(p, k), aqk = a(q, k);
          a(p, k) = c * apk - s * aqk;
          a(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vkp - s * vkq;
          V[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
  std::vector<double> V2((size_t)n * n);
  w.resize(n);
  for (int j = 0; j < n; ++j) {
    w[j] = a(idx[j], idx[j]);
    for (int k = 0; k < n; ++k) V2[(size_t)k * n + j] = V[(size_t)k * n + idx[j]];
  }
  V.swap(V2);
}

struct Krylov {
  gtn_map map;
  gtn_ctx ctx;
  int64_t n;
  double2* V;       // (kd+1) x n
  double2* coef;    // device coefficient area: [0,64) h1, [64,128) h2, [128] norm^2, [192,256) lincomb,
                    // [256, 2304) kept-Ritz rotation matrix (doubles)
  double2* part;    // multidot partials
  int nblk;
  int64_t part_cap;  // entries in part (nblk * 64)
};

int krylov_setup(gtn_map map, int kd, Krylov* K) {
  gtn_ctx ctx = map->ctx;
  if (kd < 1 || kd > kMaxKrylov) return set_err(ctx, GTN_ERR_INVALID, "krylovdim must be in 1..63");
  if (map->x_elems != map->y_elems) return set_err(ctx, GTN_ERR_SHAPE, "Krylov solvers need a square map");
  K->map = map;
  K->ctx = ctx;
  K->n = map->x_elems;
  K->nblk = multidot_blocks(ctx);
  if (map->kv_cap < kd + 1) {
    if (map->kv) cudaFree(map->kv);
    map->kv = nullptr;
    map->kv_cap = 0;
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    const size_t need = (size_t)(kd + 1) * K->n * sizeof(double2);
    if (need + (size_t(1) << 30) > freeb)
      return set_err(ctx, GTN_ERR_MEMORY, "memory admission refused: Krylov basis needs " +
                                              std::to_string(need >> 20) + " MiB");
    if (cudaMalloc(&map->kv, need) != cudaSuccess) return set_err(ctx, GTN_ERR_MEMORY, "Krylov basis allocation failed");
    map->kv_cap = kd + 1;
  }
  if (!map->kcoef) {
    // [0, 256): coefficient slots; [256, 256 + 2048): kept-Ritz rotation (kMaxKrylov^2 doubles)
    if (cudaMalloc(&map->kcoef, (256 + 2048) * sizeof(double2)) != cudaSuccess)
      return set_err(ctx, GTN_ERR_MEMORY, "Krylov coefficient allocation failed");
    map->owned.push_back(map->kcoef);
  }
  if (map->kscratch_cap < K->nblk * 64) {
    if (map->kscratch) cudaFree(map->kscratch);
    if (cudaMalloc(&map->kscratch, (size_t)K->nblk * 64 * sizeof(double2)) != cudaSuccess)
      return set_err(ctx, GTN_ERR_MEMORY, "Krylov scratch allocation failed");
    map->kscratch_cap = K->nblk * 64;
  }
  K->V = map->kv;
  K->coef = map->kcoef;
  K->part = map->kscratch;
  K->part_cap = map->kscratch_cap;
  GTN_CUDA_TRY(ctx, ctx_red(ctx, 64));
  return GTN_OK;
}

// ||x||^2 into coef[slot] (device)
cudaError_t norm2_dev(Krylov& K, const double2* x, double2* dst) {
  K.ctx->launches += 2;
  return launch_multidot(x, 0, 1, x, K.n, dst, K.part, K.nblk, K.ctx->stream, K.part_cap);
}

// Copy `cnt` double2 from device to host and wait; reports device-side wait timeouts.
int fetch(Krylov& K, const double2* dsrc, int cnt, double2* out) {
  gtn_ctx ctx = K.ctx;
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_red, dsrc, cnt * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
  int st = gtn_ctx_sync(ctx);
  if (st != GTN_OK) return st;
  for (int i = 0; i < cnt; ++i) out[i] = ctx->h_red[i];
  return GTN_OK;
}

int push(Krylov& K, const std::vector<double2>& c, double2* ddst) {
  gtn_ctx ctx = K.ctx;
  for (size_t i = 0; i < c.size(); ++i) ctx->h_red[64 + i] = c[i];
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(ddst, ctx->h_red + 64, c.size() * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
  // the pinned staging area is reused on the next call: wait for the copy
  GTN_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return GTN_OK;
}

// x <- x / ||x||, returns the norm.
int normalize(Krylov& K, double2* x, double* nrm) {
  GTN_CUDA_TRY(K.ctx, norm2_dev(K, x, K.coef + 128));
  double2 h;
  int st = fetch(K, K.coef + 128, 1, &h);
  if (st != GTN_OK) return st;
  *nrm = std::sqrt(std::max(h.x, 0.0));
  if (*nrm > 0) {
    GTN_CUDA_TRY(K.ctx, launch_axpby(K.n, make_double2(1.0 / *nrm, 0.0), x, make_double2(0.0, 0.0), x, K.ctx->stream));
    K.ctx->launches++;
  }
  return GTN_OK;
}

// Lanczos expansion of the basis from column j0 (V[j0] unit norm and orthogonal to V[0..j0))
// up to kd columns.  Fills a[j0..m), b[j0..m) and returns m (the number of basis vectors);
// V[m] then holds the normalised residual direction and b[m-1] its norm.  Stops early at an
// invariant subspace, or when `stop` says so.
template <class Stop>
int lanczos_expand(Krylov& K, int j0, int kd, int precision, std::vector<double>& a, std::vector<double>& b,
                   int* m_out, int* matvecs, bool* breakdown, Stop stop) {
  gtn_ctx ctx = K.ctx;
  cudaStream_t s = ctx->stream;
  a.resize(kd, 0.0);
  b.resize(kd, 0.0);
  for (int j = j0; j < kd; ++j) a[j] = b[j] = 0.0;
  *breakdown = false;
  const bool fast_reorth = precision != GTN_PREC_FP64;
  int m = kd;
  for (int j = j0; j < kd; ++j) {
    double2* vj = K.V + (int64_t)j * K.n;
    double2* w = K.V + (int64_t)(j + 1) * K.n;
    int st = map_run(K.map, precision, vj, w);
    if (st != GTN_OK) return st;
    (*matvecs)++;
    double2 hbuf[130];
    double hh = 0.0;  // squared norm of the full-pass coefficients (local steps only)
    if (j == j0) {
      // first vector of an expansion (couples to every kept Ritz vector): two classical
      // Gram-Schmidt passes against V[0..j] in FP64
      GTN_CUDA_TRY(ctx, launch_multidot(K.V, K.n, j + 1, w, K.n, K.coef, K.part, K.nblk, s, K.part_cap));
      GTN_CUDA_TRY(ctx, launch_lincomb(w, make_double2(1.0, 0.0), K.V, K.n, j + 1, K.coef, make_double2(-1.0, 0.0), K.n, s));
      GTN_CUDA_TRY(ctx, launch_multidot(K.V, K.n, j + 1, w, K.n, K.coef + 64, K.part, K.nblk, s, K.part_cap));
      GTN_CUDA_TRY(ctx, launch_lincomb(w, make_double2(1.0, 0.0), K.V, K.n, j + 1, K.coef + 64, make_double2(-1.0, 0.0), K.n, s));
      ctx->launches += 2 * (multidot_launch_count(j + 1) + 1);
    } else {
      // local three-term step against V[j-1], V[j] in FP64, then one full reorthogonalisation
      // pass (FP32 products for mixed-precision maps, whose error sits far above the
      // coefficients this pass removes)
      const double2* vprev = K.V + (int64_t)(j - 1) * K.n;
      GTN_CUDA_TRY(ctx, launch_multidot(vprev, K.n, 2, w, K.n, K.coef, K.part, K.nblk, s, K.part_cap));
      GTN_CUDA_TRY(ctx, launch_lincomb(w, make_double2(1.0, 0.0), vprev, K.n, 2, K.coef, make_double2(-1.0, 0.0), K.n, s));
      if (fast_reorth) {
        GTN_CUDA_TRY(ctx, launch_multidot_f32(K.V, K.n, j + 1, w, K.n, K.coef + 64, K.part, K.nblk, s, K.part_cap));
        GTN_CUDA_TRY(ctx, launch_reorth_update_f32(w, K.V, K.n, j + 1, K.coef + 64, K.n, s));
      } else {
        GTN_CUDA_TRY(ctx, launch_multidot(K.V, K.n, j + 1, w, K.n, K.coef + 64, K.part, K.nblk, s, K.part_cap));
        GTN_CUDA_TRY(ctx, launch_lincomb(w, make_double2(1.0, 0.0), K.V, K.n, j + 1, K.coef + 64, make_double2(-1.0, 0.0), K.n, s));
      }
      ctx->launches += multidot_launch_count(2) + multidot_launch_count(j + 1) + 2;
    }
    GTN_CUDA_TRY(ctx, norm2_dev(K, w, K.coef + 128));
    int st2 = fetch(K, K.coef, 130, hbuf);  // h (0..63), h2 (64..127), |w|^2 (128)
    if (st2 != GTN_OK) return st2;
    double nn = hbuf[128].x;
    if (j == j0) {
      a[j] = hbuf[j].x + hbuf[64 + j].x;
    } else {
      a[j] = hbuf[1].x + hbuf[64 + j].x;
      for (int i = 0; i <= j; ++i) hh += hbuf[64 + i].x * hbuf[64 + i].x + hbuf[64 + i].y * hbuf[64 + i].y;
      if (nn < hh) {
        // DGKS criterion: the pass removed more than half of |w|^2, so V[0..j] and w were far
        // from orthogonal; repeat it in FP64
        GTN_CUDA_TRY(ctx, launch_multidot(K.V, K.n, j + 1, w, K.n, K.coef + 64, K.part, K.nblk, s, K.part_cap));
        GTN_CUDA_TRY(ctx, launch_lincomb(w, make_double2(1.0, 0.0), K.V, K.n, j + 1, K.coef + 64, make_double2(-1.0, 0.0), K.n, s));
        GTN_CUDA_TRY(ctx, norm2_dev(K, w, K.coef + 128));
        ctx->launches += multidot_launch_count(j + 1) + 1;
        st2 = fetch(K, K.coef + 64, 65, hbuf + 64);
        if (st2 != GTN_OK) return st2;
        a[j] += hbuf[64 + j].x;
        nn = hbuf[128].x;
      }
    }
    const double beta = std::sqrt(std::max(nn, 0.0));
    b[j] = beta;
    if (beta <= 1e-13 * std::max(1.0, std::fabs(a[j]))) {
      m = j + 1;
      *breakdown = true;
      break;
    }
    GTN_CUDA_TRY(ctx, launch_axpby(K.n, make_double2(1.0 / beta, 0.0), w, make_double2(0.0, 0.0), w, s));
    ctx->launches++;
    if (stop(j + 1, a, b)) {
      m = j + 1;
      break;
    }
  }
  *m_out = m;
  return GTN_OK;
}

// Eigen-decomposition of the projected matrix of a thick-restarted Lanczos basis: the first k
// columns are kept Ritz vectors (diagonal a[i], coupled to column k by the arrow entries
// s[i]), the rest a Lanczos tridiagonal (diagonal a, off-diagonal b).  k = 0 is the plain
// tridiagonal case.
void projected_eig(int m, int k, const std::vector<double>& a, const std::vector<double>& b,
                   const std::vector<double>& s, std::vector<double>& w, std::vector<double>& Q) {
  std::vector<double> T((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) {
    T[(size_t)i * m + i] = a[i];
    if (i >= k && i + 1 < m) {
      T[(size_t)i * m + i + 1] = b[i];
      T[(size_t)(i + 1) * m + i] = b[i];
    }
  }
  if (k < m)
    for (int i = 0; i < k; ++i) {
      T[(size_t)i * m + k] = s[i];
      T[(size_t)k * m + i] = s[i];
    }
  jacobi_eig(m, T, w, Q);
}

void tridiag_eig(int m, const std::vector<double>& a, const std::vector<double>& b, std::vector<double>& w,
                 std::vector<double>& Q) {
  projected_eig(m, 0, a, b, {}, w, Q);
}

// Kept Ritz vectors per restart: about three fifths of the Krylov dimension, as KrylovKit
// (0.10) keeps in its restarted Lanczos eigsolve, the solver behind the reference's hook.
int thick_keep(int kd, int m) { return std::max(0, std::min((3 * kd + 2) / 5, m - 1)); }

}  // namespace

extern "C" int gtn_lanczos_min(gtn_map map, void* xv, int krylovdim, double tol, int maxiter, int rq_fp64,
                               double* energy, int* info, double* resid) {
  if (!map || !xv || !energy) return GTN_ERR_INVALID;
  MapUse use(map);
  if (!use.ok) return map_busy_error(map);
  Krylov K;
  int st = krylov_setup(map, std::min<int64_t>(krylovdim, std::max<int64_t>(map->x_elems, 1)), &K);
  if (st != GTN_OK) return st;
  gtn_ctx ctx = K.ctx;
  double2* x = static_cast<double2*>(xv);
  const int kd = (int)std::min<int64_t>(krylovdim, K.n);
  int matvecs = 0, restarts = 0;
  // Convergence as KrylovKit's eigsolve judges it: the residual norm |beta_m q_m| of the
  // lowest Ritz pair against the absolute tolerance.  A mixed-precision map is accurate to
  // ~1e-5 (bf16x6) relative to |H|: its Ritz residual cannot drop below that level, so the
  // tolerance is floored there, relative to the Ritz value; the energy is then the FP64
  // Rayleigh quotient, whose error is quadratic in the vector error.
  const double floor_rel = (map->precision == GTN_PREC_BF16X6 || map->precision == GTN_PREC_FP16X3) ? 5e-6
                           : map->precision == GTN_PREC_BF16X3 ? 5e-4
                           : map->precision == GTN_PREC_FP32 ? 5e-6 : 0.0;
  auto small_enough = [&](double r, double th) { return r <= std::max(tol, floor_rel * std::max(1.0, std::fabs(th))); };
  bool converged = false;
  double theta = 0, res = 0;
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(K.V, x, K.n * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
  double nrm;
  st = normalize(K, K.V, &nrm);
  if (st != GTN_OK) return st;
  if (nrm == 0) return set_err(ctx, GTN_ERR_INVALID, "zero start vector");
  // Thick-restarted Lanczos (Wu and Simon, 2000): a restart keeps the lowest Ritz vectors
  // (rotated in place at the front of the basis) and the residual direction, so that each
  // restart adds kd - keep matvecs instead of rebuilding the basis from one vector.
  std::vector<double> a, b, s, w, Q;
  int k = 0;  // kept Ritz vectors at the front of V
  const int maxit = std::max(1, maxiter);
  for (int it = 0; it < maxit; ++it) {
    restarts = it + 1;
    int m = 0;
    bool brk = false;
    auto stop = [&](int mm, const std::vector<double>& aa, const std::vector<double>& bb) {
      if (mm < 2 && kd > 1) return false;
      std::vector<double> ww, QQ;
      projected_eig(mm, k, aa, bb, s, ww, QQ);
      const double r = std::fabs(bb[mm - 1] * QQ[(size_t)(mm - 1) * mm + 0]);
      return small_enough(r, ww[0]);
    };
    st = lanczos_expand(K, k, kd, map->precision, a, b, &m, &matvecs, &brk, stop);
    if (st != GTN_OK) return st;
    projected_eig(m, k, a, b, s, w, Q);
    theta = w[0];
    res = brk ? 0.0 : std::fabs(b[m - 1] * Q[(size_t)(m - 1) * m + 0]);
    converged = brk || small_enough(res, theta) || m == K.n;
    const int keep = thick_keep(kd, m);
    if (converged || it + 1 == maxit || keep == 0) {
      // Ritz vector x = sum_i Q[i,0] V_i
      std::vector<double2> c(m);
      for (int i = 0; i < m; ++i) c[i] = make_double2(Q[(size_t)i * m + 0], 0.0);
      st = push(K, c, K.coef + 192);
      if (st != GTN_OK) return st;
      GTN_CUDA_TRY(ctx, launch_lincomb(x, make_double2(0.0, 0.0), K.V, K.n, m, K.coef + 192, make_double2(1.0, 0.0), K.n, ctx->stream));
      ctx->launches++;
      st = normalize(K, x, &nrm);
      if (st != GTN_OK) return st;
      if (converged || it + 1 == maxit) break;
      GTN_CUDA_TRY(ctx, cudaMemcpyAsync(K.V, x, K.n * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
      k = 0;
      continue;
    }
    // V[:, :keep] <- V[:, :m] Q[:, :keep]; the residual direction V[m] becomes column keep.
    std::vector<double> qk((size_t)m * keep);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < keep; ++j) qk[(size_t)i * keep + j] = Q[(size_t)i * m + j];
    double* dq = reinterpret_cast<double*>(K.coef + 256);
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(dq, qk.data(), qk.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    GTN_CUDA_TRY(ctx, launch_basis_rotate(K.V, K.n, m, keep, dq, K.n, ctx->stream));
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(K.V + (int64_t)keep * K.n, K.V + (int64_t)m * K.n, K.n * sizeof(double2),
                                      cudaMemcpyDeviceToDevice, ctx->stream));
    GTN_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // qk is pageable host memory
    ctx->launches++;
    s.assign(keep, 0.0);
    for (int i = 0; i < keep; ++i) {
      a[i] = w[i];
      s[i] = b[m - 1] * Q[(size_t)(m - 1) * m + i];
    }
    k = keep;
  }
  double E = theta;
  if (rq_fp64) {
    double2* y = K.V + K.n;  // scratch slot
    st = map_run(map, GTN_PREC_FP64, x, y);
    if (st != GTN_OK) return st;
    matvecs++;
    GTN_CUDA_TRY(ctx, launch_multidot(x, 0, 1, y, K.n, K.coef + 130, K.part, K.nblk, ctx->stream));
    ctx->launches += 2;
    double2 h;
    st = fetch(K, K.coef + 130, 1, &h);
    if (st != GTN_OK) return st;
    E = h.x;
  }
  *energy = E;
  if (info) {
    info[0] = restarts;
    info[1] = matvecs;
    info[2] = converged ? 1 : 0;
  }
  if (resid) *resid = res;
  return converged ? GTN_OK : set_err(ctx, GTN_ERR_NOT_CONVERGED, "Lanczos reached maxiter");
}

// Iterative refinement of an approximate lowest eigenvector in FP64 accuracy, with the
// bulk of the work on the map's (mixed-precision) arithmetic.  Each outer step:
//   1. y = H v with the FP64 plan, theta = <v, y>, r = y - theta v (all FP64): the only
//      FP64 application of the step; stop when |r| <= tol.
//   2. A mixed-precision Lanczos basis q_1 = r / |r|, q_2, ... of the map restricted to the
//      complement of v (every new vector orthogonalised against v and the basis).
//   3. Rayleigh-Ritz on span(v, q_1..q_m).  The projected matrix is an arrow: T[0,0] = theta
//      and T[0,1] = |r| come from the FP64 residual exactly (<q_j, H v> = <q_j, r> = 0 for
//      j > 1), the q-block is the mixed tridiagonal.  v <- the lowest Ritz vector.
// The mixed error E (|E| ~ 2e-5 |H|) enters only through the q-block, which acts on the
// correction: each step shrinks the error of v by about |E| / gap, against a floor of
// |E| / gap for the mixed solve alone.  The returned energy is the FP64 Rayleigh quotient
// of the returned vector.  This is the classical defect-correction scheme for eigenpairs
// (residual in high precision, correction in low precision; Dongarra, Moler and Wilkinson,
// SIAM J. Numer. Anal. 20 (1983)) with a Davidson-style projected correction.
extern "C" int gtn_lanczos_refine(gtn_map map, void* xv, int inner_dim, double tol, int max_outer, double* energy,
                                  int* info, double* resid) {
  if (!map || !xv || !energy) return GTN_ERR_INVALID;
  MapUse use(map);
  if (!use.ok) return map_busy_error(map);
  if (inner_dim < 1 || max_outer < 0) return set_err(map->ctx, GTN_ERR_INVALID, "inner_dim >= 1, max_outer >= 0");
  Krylov K;
  const int kd = (int)std::min<int64_t>(inner_dim + 1, std::max<int64_t>(map->x_elems, 1));
  int st = krylov_setup(map, std::min(kd, kMaxKrylov), &K);
  if (st != GTN_OK) return st;
  gtn_ctx ctx = K.ctx;
  cudaStream_t s = ctx->stream;
  double2* x = static_cast<double2*>(xv);
  const int m_max = std::min(kd, kMaxKrylov);
  int mixed_mv = 0, fp64_mv = 0, outer = 0;
  // V[0] = v (normalised)
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(K.V, x, K.n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  double nrm;
  st = normalize(K, K.V, &nrm);
  if (st != GTN_OK) return st;
  if (nrm == 0) return set_err(ctx, GTN_ERR_INVALID, "zero start vector");
  double theta = 0.0, rnorm = 0.0;
  bool converged = false;
  std::vector<double> a, b, sarr, w, Q;
  for (;;) {
    // FP64 residual of v: y in V[1], r = y - theta v in V[1]
    double2* v = K.V;
    double2* r = K.V + K.n;
    st = map_run(map, GTN_PREC_FP64, v, r);
    if (st != GTN_OK) return st;
    fp64_mv++;
    GTN_CUDA_TRY(ctx, launch_multidot(v, 0, 1, r, K.n, K.coef + 130, K.part, K.nblk, s, K.part_cap));
    ctx->launches += 2;
    double2 h;
    st = fetch(K, K.coef + 130, 1, &h);
    if (st != GTN_OK) return st;
    theta = h.x;
    GTN_CUDA_TRY(ctx, launch_axpby(K.n, make_double2(-theta, 0.0), v, make_double2(1.0, 0.0), r, s));
    ctx->launches++;
    // |r| may be far below |H|: remove the rounding-level component along v explicitly (two
    // passes) so that q_1 is orthogonal to v to working accuracy
    for (int pass = 0; pass < 2; ++pass) {
      GTN_CUDA_TRY(ctx, launch_multidot(v, 0, 1, r, K.n, K.coef, K.part, K.nblk, s, K.part_cap));
      GTN_CUDA_TRY(ctx, launch_lincomb(r, make_double2(1.0, 0.0), v, K.n, 1, K.coef, make_double2(-1.0, 0.0), K.n, s));
      ctx->launches += multidot_launch_count(1) + 1;
    }
    st = normalize(K, r, &rnorm);  // q_1 = r / |r|
    if (st != GTN_OK) return st;
    if (rnorm <= tol || rnorm == 0.0) {
      converged = true;
      break;
    }
    if (outer >= max_outer || m_max < 2) break;
    ++outer;
    // mixed Lanczos on the complement of v, from q_1; stop once the lowest Ritz pair of the
    // arrow matrix has a residual below 1 % of |r| (or the tolerance)
    a.assign(m_max, 0.0);
    b.assign(m_max, 0.0);
    sarr.assign(1, rnorm);
    int m = 0;
    bool brk = false;
    auto stop = [&](int mm, const std::vector<double>& aa, const std::vector<double>& bb) {
      if (mm < 3) return false;
      std::vector<double> a2(aa), ww, QQ;
      a2[0] = theta;
      projected_eig(mm, 1, a2, bb, sarr, ww, QQ);
      const double rin = std::fabs(bb[mm - 1] * QQ[(size_t)(mm - 1) * mm + 0]);
      return rin <= std::max(tol, 1e-2 * rnorm);
    };
    int mv = 0;
    st = lanczos_expand(K, 1, m_max, map->precision, a, b, &m, &mv, &brk, stop);
    if (st != GTN_OK) return st;
    mixed_mv += mv;
    a[0] = theta;
    projected_eig(m, 1, a, b, sarr, w, Q);
    // v <- sum_i Q[i, 0] V_i, normalised (into x, then back to V[0])
    std::vector<double2> c(m);
    for (int i = 0; i < m; ++i) c[i] = make_double2(Q[(size_t)i * m + 0], 0.0);
    st = push(K, c, K.coef + 192);
    if (st != GTN_OK) return st;
    GTN_CUDA_TRY(ctx, launch_lincomb(x, make_double2(0.0, 0.0), K.V, K.n, m, K.coef + 192, make_double2(1.0, 0.0), K.n, s));
    ctx->launches++;
    st = normalize(K, x, &nrm);
    if (st != GTN_OK) return st;
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(K.V, x, K.n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  }
  // the returned vector is V[0] (normalised); its FP64 Rayleigh quotient is theta
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(x, K.V, K.n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  GTN_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  *energy = theta;
  if (info) {
    info[0] = outer;
    info[1] = mixed_mv;
    info[2] = fp64_mv;
    info[3] = converged ? 1 : 0;
  }
  if (resid) *resid = rnorm;
  return converged ? GTN_OK : set_err(ctx, GTN_ERR_NOT_CONVERGED, "refinement reached max_outer");
}

extern "C" int gtn_expm_apply(gtn_map map, double dz_re, double dz_im, void* xv, int krylovdim, double tol,
                              int* info) {
  if (!map || !xv) return GTN_ERR_INVALID;
  MapUse use(map);
  if (!use.ok) return map_busy_error(map);
  Krylov K;
  int st = krylov_setup(map, std::min<int64_t>(krylovdim, std::max<int64_t>(map->x_elems, 1)), &K);
  if (st != GTN_OK) return st;
  gtn_ctx ctx = K.ctx;
  double2* x = static_cast<double2*>(xv);
  const int kd = (int)std::min<int64_t>(krylovdim, K.n);
  const std::complex<double> dz(dz_re, dz_im);
  double remaining = 1.0, frac = 1.0;
  int matvecs = 0, substeps = 0;
  std::vector<double> a, b, w, Q;
  while (remaining > 1e-14) {
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(K.V, x, K.n * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
    double beta0;
    st = normalize(K, K.V, &beta0);
    if (st != GTN_OK) return st;
    if (beta0 == 0) break;
    int m = 0;
    bool brk = false;
    st = lanczos_expand(K, 0, kd, map->precision, a, b, &m, &matvecs, &brk,
                        [](int, const std::vector<double>&, const std::vector<double>&) { return false; });
    if (st != GTN_OK) return st;
    tridiag_eig(m, a, b, w, Q);
    double step = std::min(frac, remaining);
    std::vector<std::complex<double>> c(m);
    for (int tries = 0; tries < 60; ++tries) {
      for (int i = 0; i < m; ++i) {
        std::complex<double> acc = 0;
        for (int k = 0; k < m; ++k)
          acc += Q[(size_t)i * m + k] * std::exp(dz * (step * w[k])) * Q[(size_t)0 * m + k];
        c[i] = acc;
      }
      const double err = (brk || m < kd) ? 0.0 : beta0 * std::fabs(b[m - 1]) * std::abs(c[m - 1]);
      if (err <= tol || step < 1e-12) break;
      step *= 0.5;
    }
    std::vector<double2> cd(m);
    for (int i = 0; i < m; ++i) cd[i] = make_double2(beta0 * c[i].real(), beta0 * c[i].imag());
    st = push(K, cd, K.coef + 192);
    if (st != GTN_OK) return st;
    GTN_CUDA_TRY(ctx, launch_lincomb(x, make_double2(0.0, 0.0), K.V, K.n, m, K.coef + 192, make_double2(1.0, 0.0), K.n, ctx->stream));
    ctx->launches++;
    remaining -= step;
    frac = step;
    substeps++;
    if (substeps > 4096) return set_err(ctx, GTN_ERR_NOT_CONVERGED, "expm: too many substeps");
  }
  if (info) {
    info[0] = substeps;
    info[1] = matvecs;
  }
  return gtn_ctx_sync(ctx);
}

namespace {

using cplx = std::complex<double>;

// exp(A) of a small dense complex matrix (row-major m x m) by scaling and squaring with a
// truncated Taylor series (Moler and Van Loan, SIAM Review 45 (2003), method 3): A is
// scaled by 2^-s so that its 1-norm is at most 1/2, the series is summed until a term
// falls below 2^-60 of the partial sum (at most 40 terms), and the result is squared s times.
void expm_small(int m, const std::vector<cplx>& A, std::vector<cplx>& E) {
  double nrm = 0;
  for (int j = 0; j < m; ++j) {
    double col = 0;
    for (int i = 0; i < m; ++i) col += std::abs(A[(size_t)i * m + j]);
    nrm = std::max(nrm, col);
  }
  int s = 0;
  while (nrm > 0.5 && s < 1000) {
    nrm *= 0.5;
    ++s;
  }
  const double scale = std::ldexp(1.0, -s);
  std::vector<cplx> As(A.size()), term((size_t)m * m, 0.0), next((size_t)m * m);
  for (size_t i = 0; i < A.size(); ++i) As[i] = A[i] * scale;
  E.assign((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) {
    E[(size_t)i * m + i] = 1.0;
    term[(size_t)i * m + i] = 1.0;
  }
  for (int k = 1; k <= 40; ++k) {
    double tn = 0, en = 0;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        cplx acc = 0;
        for (int l = 0; l < m; ++l) acc += term[(size_t)i * m + l] * As[(size_t)l * m + j];
        next[(size_t)i * m + j] = acc / (double)k;
      }
    term.swap(next);
    for (size_t i = 0; i < E.size(); ++i) {
      E[i] += term[i];
      tn = std::max(tn, std::abs(term[i]));
      en = std::max(en, std::abs(E[i]));
    }
    if (tn <= std::ldexp(en, -60)) break;
  }
  for (int q = 0; q < s; ++q) {
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        cplx acc = 0;
        for (int l = 0; l < m; ++l) acc += E[(size_t)i * m + l] * E[(size_t)l * m + j];
        next[(size_t)i * m + j] = acc;
      }
    E.swap(next);
  }
}

// Arnoldi expansion from V[0] (unit norm) for a map that is not Hermitian: two FP64
// classical Gram-Schmidt passes against the whole basis per step.  Hm (row-major
// (kd+1) x kd) receives the projections H[i][j] = <v_i, A v_j> and the subdiagonal norms.
int arnoldi_expand(Krylov& K, int kd, int precision, std::vector<cplx>& Hm, int* m_out, int* matvecs,
                   bool* breakdown) {
  gtn_ctx ctx = K.ctx;
  cudaStream_t s = ctx->stream;
  Hm.assign((size_t)(kd + 1) * kd, 0.0);
  *breakdown = false;
  int m = kd;
  for (int j = 0; j < kd; ++j) {
    double2* vj = K.V + (int64_t)j * K.n;
    double2* w = K.V + (int64_t)(j + 1) * K.n;
    int st = map_run(K.map, precision, vj, w);
    if (st != GTN_OK) return st;
    (*matvecs)++;
    GTN_CUDA_TRY(ctx, launch_multidot(K.V, K.n, j + 1, w, K.n, K.coef, K.part, K.nblk, s, K.part_cap));
    GTN_CUDA_TRY(ctx, launch_lincomb(w, make_double2(1.0, 0.0), K.V, K.n, j + 1, K.coef, make_double2(-1.0, 0.0), K.n, s));
    GTN_CUDA_TRY(ctx, launch_multidot(K.V, K.n, j + 1, w, K.n, K.coef + 64, K.part, K.nblk, s, K.part_cap));
    GTN_CUDA_TRY(ctx, launch_lincomb(w, make_double2(1.0, 0.0), K.V, K.n, j + 1, K.coef + 64, make_double2(-1.0, 0.0), K.n, s));
    GTN_CUDA_TRY(ctx, norm2_dev(K, w, K.coef + 128));
    ctx->launches += 2 * (multidot_launch_count(j + 1) + 1);
    double2 hbuf[130];
    st = fetch(K, K.coef, 130, hbuf);
    if (st != GTN_OK) return st;
    double colmax = 0;
    for (int i = 0; i <= j; ++i) {
      Hm[(size_t)i * kd + j] = cplx(hbuf[i].x + hbuf[64 + i].x, hbuf[i].y + hbuf[64 + i].y);
      colmax = std::max(colmax, std::abs(Hm[(size_t)i * kd + j]));
    }
    const double beta = std::sqrt(std::max(hbuf[128].x, 0.0));
    Hm[(size_t)(j + 1) * kd + j] = beta;
    if (beta <= 1e-13 * std::max(1.0, colmax)) {
      m = j + 1;
      *breakdown = true;
      break;
    }
    GTN_CUDA_TRY(ctx, launch_axpby(K.n, make_double2(1.0 / beta, 0.0), w, make_double2(0.0, 0.0), w, s));
    ctx->launches++;
  }
  *m_out = m;
  return GTN_OK;
}

}  // namespace

extern "C" int gtn_expm_small(int m, const double* A, double* E) {
  if (m < 1 || m > 256 || !A || !E) return GTN_ERR_INVALID;
  std::vector<cplx> a((size_t)m * m), e;
  for (size_t i = 0; i < a.size(); ++i) a[i] = cplx(A[2 * i], A[2 * i + 1]);
  expm_small(m, a, e);
  for (size_t i = 0; i < e.size(); ++i) {
    E[2 * i] = e[i].real();
    E[2 * i + 1] = e[i].imag();
  }
  return GTN_OK;
}

extern "C" int gtn_expm_apply_arnoldi(gtn_map map, double dz_re, double dz_im, void* xv, int krylovdim, double tol,
                                      int* info) {
  if (!map || !xv) return GTN_ERR_INVALID;
  MapUse use(map);
  if (!use.ok) return map_busy_error(map);
  Krylov K;
  int st = krylov_setup(map, std::min<int64_t>(krylovdim, std::max<int64_t>(map->x_elems, 1)), &K);
  if (st != GTN_OK) return st;
  gtn_ctx ctx = K.ctx;
  double2* x = static_cast<double2*>(xv);
  const int kd = (int)std::min<int64_t>(krylovdim, K.n);
  const cplx dz(dz_re, dz_im);
  double remaining = 1.0, frac = 1.0;
  int matvecs = 0, substeps = 0;
  std::vector<cplx> Hm, T, E;
  while (remaining > 1e-14) {
    GTN_CUDA_TRY(ctx, cudaMemcpyAsync(K.V, x, K.n * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
    double beta0;
    st = normalize(K, K.V, &beta0);
    if (st != GTN_OK) return st;
    if (beta0 == 0) break;
    int m = 0;
    bool brk = false;
    st = arnoldi_expand(K, kd, map->precision, Hm, &m, &matvecs, &brk);
    if (st != GTN_OK) return st;
    double step = std::min(frac, remaining);
    std::vector<cplx> c(m);
    T.assign((size_t)m * m, 0.0);
    for (int tries = 0; tries < 60; ++tries) {
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) T[(size_t)i * m + j] = dz * step * Hm[(size_t)i * kd + j];
      expm_small(m, T, E);
      for (int i = 0; i < m; ++i) c[i] = E[(size_t)i * m + 0];
      const double err = (brk || m < kd) ? 0.0 : beta0 * std::abs(Hm[(size_t)m * kd + m - 1]) * std::abs(c[m - 1]);
      if (err <= tol || step < 1e-12) break;
      step *= 0.5;
    }
    std::vector<double2> cd(m);
    for (int i = 0; i < m; ++i) cd[i] = make_double2(beta0 * c[i].real(), beta0 * c[i].imag());
    st = push(K, cd, K.coef + 192);
    if (st != GTN_OK) return st;
    GTN_CUDA_TRY(ctx, launch_lincomb(x, make_double2(0.0, 0.0), K.V, K.n, m, K.coef + 192, make_double2(1.0, 0.0), K.n, ctx->stream));
    ctx->launches++;
    remaining -= step;
    frac = step;
    substeps++;
    if (substeps > 4096) return set_err(ctx, GTN_ERR_NOT_CONVERGED, "expm: too many substeps");
  }
  if (info) {
    info[0] = substeps;
    info[1] = matvecs;
  }
  return gtn_ctx_sync(ctx);
}
