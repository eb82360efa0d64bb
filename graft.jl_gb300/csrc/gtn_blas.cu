// Vector kernels for the device-resident Krylov solvers: batched Gram-Schmidt projections
// h = V^H w, linear combinations w = b*w + s*V*c, their FP32-product variants, the thick-
// restart basis rotation, and small helpers for the factorisation paths.  In FP64 a complex
// multiply-add per element and vector costs four DFMA, which on this part bounds the
// projections near 1.5 TB/s of streamed data, below HBM; the FP32 variants and the
// one-to-two-vector kernels are bound by memory latency and HBM.
#include "gtn_internal.h"

namespace {

constexpr int kMaxJ = 64;
constexpr int kDotThreads = 256;

__device__ __forceinline__ double2 cmul_conj(double2 a, double2 b) {  // conj(a) * b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// double -> float by bit manipulation on the integer pipe: mantissa truncated to 23 bits,
// magnitudes below float's normal range flushed to signed zero, finite values above it
// clamped to the largest float.  Inf stays Inf and NaN stays NaN (a quiet NaN), so a
// non-finite basis entry propagates into the projections instead of being hidden.  The
// hardware F2F conversion runs at the FP64 rate on this part, which would make the
// FP32-product kernels as slow as FP64 ones.
__device__ __forceinline__ float dtof_trunc(double d) {
  const unsigned hi = (unsigned)__double2hiint(d);
  const unsigned lo = (unsigned)__double2loint(d);
  const unsigned sign = hi & 0x80000000u;
  const unsigned ebits = (hi >> 20) & 0x7ffu;
  const int e = (int)ebits - 1023 + 127;
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const bool nonfinite = ebits == 0x7ffu;
  const bool nan = nonfinite && (((hi & 0xfffffu) | lo) != 0u);
  const unsigned bits = nonfinite ? (sign | 0x7f800000u | (nan ? 0x00400000u : 0u))
                        : e <= 0  ? sign
                        : e >= 255 ? (sign | 0x7f7fffffu)
                                   : (sign | ((unsigned)e << 23) | mant);
  return __uint_as_float(bits);
}

// Per-block partial sums of conj(V_j) . w for j < J, written to part[block * J + j].
template <int JB>
__global__ void __launch_bounds__(kDotThreads) multidot_partial_kernel(const double2* __restrict__ V,
                                                                       int64_t ldv, int J, int j0,
                                                                       const double2* __restrict__ w,
                                                                       int64_t n,
                                                                       double2* __restrict__ part) {
  double2 acc[JB];
#pragma unroll
  for (int j = 0; j < JB; ++j) acc[j] = make_double2(0.0, 0.0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 wi = w[i];
#pragma unroll
    for (int j = 0; j < JB; ++j) {
      if (j0 + j < J) {
        const double2 v = V[(int64_t)(j0 + j) * ldv + i];
        const double2 p = cmul_conj(v, wi);
        acc[j].x += p.x;
        acc[j].y += p.y;
      }
    }
  }
  __shared__ double2 red[kDotThreads / 32][JB];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < JB; ++j) {
    double x = acc[j].x, y = acc[j].y;
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_down_sync(0xffffffffu, x, o);
      y += __shfl_down_sync(0xffffffffu, y, o);
    }
    if (lane == 0) red[wid][j] = make_double2(x, y);
  }
  __syncthreads();
  if (threadIdx.x < JB && j0 + (int)threadIdx.x < J) {
    double x = 0, y = 0;
    for (int q = 0; q < kDotThreads / 32; ++q) {
      x += red[q][threadIdx.x].x;
      y += red[q][threadIdx.x].y;
    }
    part[(int64_t)blockIdx.x * J + j0 + threadIdx.x] = make_double2(x, y);
  }
}

// The same projections with FP32 products (inputs rounded to float, per-thread sums in
// float, block sums in double): for reorthogonalisation passes of mixed-precision Krylov
// bases, whose coefficients only need to be accurate well below the map's own error.  The
// vector kernels are FP64-ALU bound on this part, not HBM bound.
template <int JB>
__global__ void __launch_bounds__(kDotThreads) multidot_f32_partial_kernel(const double2* __restrict__ V,
                                                                           int64_t ldv, int J, int j0,
                                                                           const double2* __restrict__ w,
                                                                           int64_t n,
                                                                           double2* __restrict__ part) {
  float2 acc[JB];
#pragma unroll
  for (int j = 0; j < JB; ++j) acc[j] = make_float2(0.f, 0.f);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 wd = w[i];
    const float wx = dtof_trunc(wd.x), wy = dtof_trunc(wd.y);
#pragma unroll
    for (int j = 0; j < JB; ++j) {
      if (j0 + j < J) {
        const double2 vd = V[(int64_t)(j0 + j) * ldv + i];
        const float vx = dtof_trunc(vd.x), vy = dtof_trunc(vd.y);
        acc[j].x = fmaf(vx, wx, fmaf(vy, wy, acc[j].x));
        acc[j].y = fmaf(vx, wy, fmaf(-vy, wx, acc[j].y));
      }
    }
  }
  __shared__ double2 red[kDotThreads / 32][JB];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < JB; ++j) {
    double x = acc[j].x, y = acc[j].y;
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_down_sync(0xffffffffu, x, o);
      y += __shfl_down_sync(0xffffffffu, y, o);
    }
    if (lane == 0) red[wid][j] = make_double2(x, y);
  }
  __syncthreads();
  if (threadIdx.x < JB && j0 + (int)threadIdx.x < J) {
    double x = 0, y = 0;
    for (int q = 0; q < kDotThreads / 32; ++q) {
      x += red[q][threadIdx.x].x;
      y += red[q][threadIdx.x].y;
    }
    part[(int64_t)blockIdx.x * J + j0 + threadIdx.x] = make_double2(x, y);
  }
}

// w -= sum_j coef[j] V_j with FP32 products and one FP64 subtraction per element: the
// update of a reorthogonalisation pass, whose coefficients are small next to |w|.
__global__ void reorth_update_f32_kernel(double2* __restrict__ w, const double2* __restrict__ V, int64_t ldv,
                                         int J, const double2* __restrict__ coef, int64_t n) {
  __shared__ float2 c[kMaxJ];
  if ((int)threadIdx.x < J) {
    const double2 a = coef[threadIdx.x];
    c[threadIdx.x] = make_float2((float)a.x, (float)a.y);
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float ax = 0.f, ay = 0.f;
    for (int j = 0; j < J; ++j) {
      const double2 vd = V[(int64_t)j * ldv + i];
      const float vx = dtof_trunc(vd.x), vy = dtof_trunc(vd.y);
      ax = fmaf(c[j].x, vx, fmaf(-c[j].y, vy, ax));
      ay = fmaf(c[j].x, vy, fmaf(c[j].y, vx, ay));
    }
    double2 wi = w[i];
    wi.x -= (double)ax;
    wi.y -= (double)ay;
    w[i] = wi;
  }
}

// out[j] = sum over blocks of part[b * J + j] (fixed order: deterministic).
__global__ void multidot_final_kernel(const double2* __restrict__ part, int nblk, int J,
                                      double2* __restrict__ out) {
  const int j = blockIdx.x;
  double x = 0, y = 0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    x += part[(int64_t)b * J + j].x;
    y += part[(int64_t)b * J + j].y;
  }
  __shared__ double sx[256], sy[256];
  sx[threadIdx.x] = x;
  sy[threadIdx.x] = y;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sx[threadIdx.x] += sx[threadIdx.x + o];
      sy[threadIdx.x] += sy[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[j] = make_double2(sx[0], sy[0]);
}

// w = beta*w + cscale * sum_j coef[j] V_j
__global__ void lincomb_kernel(double2* __restrict__ w, double2 beta, const double2* __restrict__ V,
                               int64_t ldv, int J, const double2* __restrict__ coef, double2 cscale,
                               int64_t n) {
  __shared__ double2 c[kMaxJ];
  if ((int)threadIdx.x < J) {
    const double2 a = coef[threadIdx.x];
    c[threadIdx.x] = make_double2(a.x * cscale.x - a.y * cscale.y, a.x * cscale.y + a.y * cscale.x);
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double2 acc;
    if (beta.x == 0.0 && beta.y == 0.0) {
      acc = make_double2(0.0, 0.0);
    } else if (beta.x == 1.0 && beta.y == 0.0) {  // the Gram-Schmidt update: no FP64 multiply
      acc = w[i];
    } else {
      const double2 wi = w[i];
      acc = make_double2(beta.x * wi.x - beta.y * wi.y, beta.x * wi.y + beta.y * wi.x);
    }
    for (int j = 0; j < J; ++j) {
      const double2 v = V[(int64_t)j * ldv + i];
      acc.x += c[j].x * v.x - c[j].y * v.y;
      acc.y += c[j].x * v.y + c[j].y * v.x;
    }
    w[i] = acc;
  }
}

__global__ void axpby_kernel(int64_t n, double2 a, const double2* __restrict__ x, double2 b,
                             double2* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 xi = x[i];
    if (a.y == 0.0 && b.x == 0.0 && b.y == 0.0) {  // real scaling (normalisation): 2 FP64 multiplies
      y[i] = make_double2(a.x * xi.x, a.x * xi.y);
      continue;
    }
    double2 yi = make_double2(0.0, 0.0);
    if (b.x != 0.0 || b.y != 0.0) {
      const double2 t = y[i];
      yi = make_double2(b.x * t.x - b.y * t.y, b.x * t.y + b.y * t.x);
    }
    yi.x += a.x * xi.x - a.y * xi.y;
    yi.y += a.x * xi.y + a.y * xi.x;
    y[i] = yi;
  }
}

__global__ void c64_to_c128_kernel(const float2* __restrict__ x, double2* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = make_double2(x[i].x, x[i].y);
}

__global__ void fill_kernel(double2* __restrict__ x, double2 v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = v;
}

// out[a][j][b] = in[a][idx[j]][b]: one leg of a row-major tensor restricted to a list of
// indices (a = outer legs, b = inner legs).
__global__ void restrict_leg_kernel(const double2* __restrict__ in, double2* __restrict__ out, int64_t A,
                                    int64_t Lin, int64_t nsel, int64_t B, const int64_t* __restrict__ idx) {
  const int64_t total = A * nsel * B;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i % B;
    const int64_t r = i / B;
    const int64_t j = r % nsel;
    const int64_t a = r / nsel;
    out[i] = in[(a * Lin + idx[j]) * B + b];
  }
}

__global__ void conj_kernel(double2* __restrict__ x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i].y = -x[i].y;
}

__global__ void transpose_kernel(const double2* __restrict__ in, int64_t rows, int64_t cols,
                                 double2* __restrict__ out) {
  __shared__ double2 tile[32][33];
  const int64_t c0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int64_t rr = r0 + r, cc = c0 + threadIdx.x;
    if (rr < rows && cc < cols) tile[r][threadIdx.x] = in[rr * cols + cc];
  }
  __syncthreads();
  for (int c = threadIdx.y; c < 32; c += 8) {
    const int64_t cc = c0 + c, rr = r0 + threadIdx.x;
    if (rr < rows && cc < cols) out[cc * rows + rr] = tile[threadIdx.x][c];
  }
}

__global__ void zero_lower_kernel(double2* __restrict__ R, int64_t rows, int64_t cols) {
  const int64_t total = rows * cols;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / cols, c = i - r * cols;
    if (c < r) R[i] = make_double2(0.0, 0.0);
  }
}

__global__ void diag_scale_kernel(double2* __restrict__ A, int64_t rows, int64_t cols,
                                  const double* __restrict__ d, int side) {
  const int64_t total = rows * cols;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / cols;
    const double f = side == 0 ? d[i - r * cols] : d[r];
    A[i].x *= f;
    A[i].y *= f;
  }
}

// out[r] = ||A[r][:]||_2, one CTA per row
__global__ void __launch_bounds__(256) row_norms_kernel(const double2* __restrict__ A, int64_t cols,
                                                        double* __restrict__ out) {
  __shared__ double red[256];
  const double2* a = A + (int64_t)blockIdx.x * cols;
  double acc = 0.0;
  for (int64_t c = threadIdx.x; c < cols; c += 256) acc += a[c].x * a[c].x + a[c].y * a[c].y;
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sqrt(red[0]);
}

// A[r][c] = conj(ph[r] * A[r][c])
__global__ void row_phase_conj_kernel(double2* __restrict__ A, int64_t rows, int64_t cols,
                                      const double2* __restrict__ ph) {
  const int64_t total = rows * cols;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 p = ph[i / cols], a = A[i];
    A[i] = make_double2(p.x * a.x - p.y * a.y, -(p.x * a.y + p.y * a.x));
  }
}

// Thick-restart basis rotation, in place.  A block stages its kRotRows rows of all m basis
// vectors in shared memory before it writes any of them, and blocks own disjoint rows, so the
// kept combinations can overwrite the leading columns directly.
constexpr int kRotRows = 32;
constexpr int kRotThreads = 128;

__global__ void __launch_bounds__(kRotThreads) basis_rotate_kernel(double2* __restrict__ V, int64_t ldv, int m,
                                                                   int k, const double* __restrict__ Q,
                                                                   int64_t n) {
  __shared__ double2 tile[kMaxJ][kRotRows];
  const int64_t row0 = (int64_t)blockIdx.x * kRotRows;
  const int r = threadIdx.x % kRotRows, g = threadIdx.x / kRotRows;
  constexpr int kGroups = kRotThreads / kRotRows;
  const bool live = row0 + r < n;
  for (int i = g; i < m; i += kGroups)
    tile[i][r] = live ? V[(int64_t)i * ldv + row0 + r] : make_double2(0.0, 0.0);
  __syncthreads();
  if (!live) return;
  for (int j = g; j < k; j += kGroups) {
    double2 acc = make_double2(0.0, 0.0);
    for (int i = 0; i < m; ++i) {
      const double q = __ldg(Q + (int64_t)i * k + j);
      acc.x += q * tile[i][r].x;
      acc.y += q * tile[i][r].y;
    }
    V[(int64_t)j * ldv + row0 + r] = acc;
  }
}

// Counter-based uniform fill in [-1, 1) for both parts: the SplitMix64 finaliser (Steele,
// Lea and Flood, 2014) of seed + index, top 53 bits as a double.  Deterministic for a seed.
__device__ __forceinline__ double splitmix_unit(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

__global__ void fill_uniform_kernel(double2* __restrict__ x, int64_t n, uint64_t seed) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = make_double2(splitmix_unit(seed + 2 * (uint64_t)i), splitmix_unit(seed + 2 * (uint64_t)i + 1));
}

inline unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

int multidot_blocks(gtn_ctx ctx) { return (ctx->sm_count > 0 ? ctx->sm_count : 152) * 2; }

int multidot_launch_count(int J) {
  int c = J > 0 ? 1 : 0;  // the final reduction
  for (int j0 = 0; j0 < J;) {
    const int rem = J - j0;
    j0 += rem >= 8 ? 8 : rem >= 4 ? 4 : rem >= 2 ? 2 : 1;
    ++c;
  }
  return c;
}

// Grid widening for latency-bound projections: the FP32 kernels and the 1-2 vector FP64 ones
// keep too few loads in flight with 2 CTAs per SM.  The partials need nb * J entries, so the
// grid only widens as far as the caller's scratch capacity allows (0: exactly nblk * J).
int widened_blocks(int nblk, int J, int64_t scratch_cap, bool f32) {
  if (scratch_cap <= 0 || (!f32 && J > 2)) return nblk;
  for (int f : {4, 2})
    if ((int64_t)nblk * f * J <= scratch_cap) return nblk * f;
  return nblk;
}

cudaError_t launch_multidot(const double2* V, int64_t ldv, int J, const double2* w, int64_t n,
                            double2* out, double2* scratch, int nblk, cudaStream_t s, int64_t scratch_cap) {
  if (J <= 0) return cudaSuccess;
  if (J > kMaxJ) return cudaErrorInvalidValue;
  nblk = widened_blocks(nblk, J, scratch_cap, false);
  // vectors in groups of 8, 4, 2, 1: a guarded slot of a wider kernel still costs its FP64 work
  for (int j0 = 0; j0 < J;) {
    const int rem = J - j0;
    if (rem >= 8) multidot_partial_kernel<8><<<nblk, kDotThreads, 0, s>>>(V, ldv, J, j0, w, n, scratch);
    else if (rem >= 4) multidot_partial_kernel<4><<<nblk, kDotThreads, 0, s>>>(V, ldv, J, j0, w, n, scratch);
    else if (rem >= 2) multidot_partial_kernel<2><<<nblk, kDotThreads, 0, s>>>(V, ldv, J, j0, w, n, scratch);
    else multidot_partial_kernel<1><<<nblk, kDotThreads, 0, s>>>(V, ldv, J, j0, w, n, scratch);
    j0 += rem >= 8 ? 8 : rem >= 4 ? 4 : rem >= 2 ? 2 : 1;
  }
  multidot_final_kernel<<<J, 256, 0, s>>>(scratch, nblk, J, out);
  return cudaGetLastError();
}

cudaError_t launch_multidot_f32(const double2* V, int64_t ldv, int J, const double2* w, int64_t n,
                                double2* out, double2* scratch, int nblk, cudaStream_t s, int64_t scratch_cap) {
  if (J <= 0) return cudaSuccess;
  if (J > kMaxJ) return cudaErrorInvalidValue;
  nblk = widened_blocks(nblk, J, scratch_cap, true);
  for (int j0 = 0; j0 < J;) {
    const int rem = J - j0;
    if (rem >= 8) multidot_f32_partial_kernel<8><<<nblk, kDotThreads, 0, s>>>(V, ldv, J, j0, w, n, scratch);
    else if (rem >= 4) multidot_f32_partial_kernel<4><<<nblk, kDotThreads, 0, s>>>(V, ldv, J, j0, w, n, scratch);
    else if (rem >= 2) multidot_f32_partial_kernel<2><<<nblk, kDotThreads, 0, s>>>(V, ldv, J, j0, w, n, scratch);
    else multidot_f32_partial_kernel<1><<<nblk, kDotThreads, 0, s>>>(V, ldv, J, j0, w, n, scratch);
    j0 += rem >= 8 ? 8 : rem >= 4 ? 4 : rem >= 2 ? 2 : 1;
  }
  multidot_final_kernel<<<J, 256, 0, s>>>(scratch, nblk, J, out);
  return cudaGetLastError();
}

cudaError_t launch_reorth_update_f32(double2* w, const double2* V, int64_t ldv, int J, const double2* coef,
                                     int64_t n, cudaStream_t s) {
  if (J > kMaxJ) return cudaErrorInvalidValue;
  if (J <= 0) return cudaSuccess;
  reorth_update_f32_kernel<<<grid_for(n), 256, 0, s>>>(w, V, ldv, J, coef, n);
  return cudaGetLastError();
}

cudaError_t launch_lincomb(double2* w, double2 beta, const double2* V, int64_t ldv, int J,
                           const double2* coef, double2 cscale, int64_t n, cudaStream_t s) {
  if (J > kMaxJ) return cudaErrorInvalidValue;
  lincomb_kernel<<<grid_for(n), 256, 0, s>>>(w, beta, V, ldv, J, coef, cscale, n);
  return cudaGetLastError();
}

cudaError_t launch_basis_rotate(double2* V, int64_t ldv, int m, int k, const double* Q, int64_t n,
                                cudaStream_t s) {
  if (m > kMaxJ || k > m || k < 0) return cudaErrorInvalidValue;
  if (k == 0 || n <= 0) return cudaSuccess;
  const int64_t blocks = (n + kRotRows - 1) / kRotRows;
  if (blocks > 0x7fffffff) return cudaErrorInvalidValue;
  basis_rotate_kernel<<<(unsigned)blocks, kRotThreads, 0, s>>>(V, ldv, m, k, Q, n);
  return cudaGetLastError();
}

cudaError_t launch_axpby(int64_t n, double2 a, const double2* x, double2 b, double2* y, cudaStream_t s) {
  axpby_kernel<<<grid_for(n), 256, 0, s>>>(n, a, x, b, y);
  return cudaGetLastError();
}
cudaError_t launch_c64_to_c128(const float2* x, double2* y, int64_t n, cudaStream_t s) {
  c64_to_c128_kernel<<<grid_for(n), 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}
cudaError_t launch_fill_uniform_c128(double2* x, int64_t n, uint64_t seed, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  fill_uniform_kernel<<<grid_for(n), 256, 0, s>>>(x, n, seed);
  return cudaGetLastError();
}

cudaError_t launch_fill_c128(double2* x, double2 v, int64_t n, cudaStream_t s) {
  fill_kernel<<<grid_for(n), 256, 0, s>>>(x, v, n);
  return cudaGetLastError();
}
cudaError_t launch_restrict_leg(const double2* in, double2* out, int64_t A, int64_t Lin, int64_t nsel, int64_t B,
                                const int64_t* idx, cudaStream_t s) {
  const int64_t total = A * nsel * B;
  if (total <= 0) return cudaSuccess;
  restrict_leg_kernel<<<grid_for(total), 256, 0, s>>>(in, out, A, Lin, nsel, B, idx);
  return cudaGetLastError();
}

cudaError_t launch_conj_inplace(double2* x, int64_t n, cudaStream_t s) {
  conj_kernel<<<grid_for(n), 256, 0, s>>>(x, n);
  return cudaGetLastError();
}
cudaError_t launch_transpose_c128(const double2* in, int64_t rows, int64_t cols, double2* out,
                                  cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const int64_t gy = (rows + 31) / 32;
  if (gy > 65535) return cudaErrorInvalidConfiguration;
  transpose_kernel<<<dim3((unsigned)((cols + 31) / 32), (unsigned)gy), dim3(32, 8), 0, s>>>(in, rows, cols, out);
  return cudaGetLastError();
}
cudaError_t launch_zero_lower(double2* R, int64_t rows, int64_t cols, cudaStream_t s) {
  zero_lower_kernel<<<grid_for(rows * cols), 256, 0, s>>>(R, rows, cols);
  return cudaGetLastError();
}
cudaError_t launch_diag_scale(double2* A, int64_t rows, int64_t cols, const double* d, int side,
                              cudaStream_t s) {
  diag_scale_kernel<<<grid_for(rows * cols), 256, 0, s>>>(A, rows, cols, d, side);
  return cudaGetLastError();
}
cudaError_t launch_row_phase_conj(double2* A, int64_t rows, int64_t cols, const double2* ph, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  row_phase_conj_kernel<<<grid_for(rows * cols), 256, 0, s>>>(A, rows, cols, ph);
  return cudaGetLastError();
}
cudaError_t launch_row_norms(const double2* A, int64_t rows, int64_t cols, double* out, cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  if (rows > 2147483647LL) return cudaErrorInvalidConfiguration;
  row_norms_kernel<<<(unsigned)rows, 256, 0, s>>>(A, cols, out);
  return cudaGetLastError();
}
