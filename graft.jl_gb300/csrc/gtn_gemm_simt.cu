// Complex SIMT GEMMs for the FP64 path (DFMA) and the FP32 diagnostic path (FFMA).
//   C[n][m] = sum_k A[m][k] * B[n][k]      A: [M][K], B: [N][K], C: [N][M] (row-major)
// The output is written m-fastest so that each warp's stores are contiguous.
#include "gtn_internal.h"

#include <algorithm>
#include <cstring>

namespace {

template <typename T> struct CT;
template <> struct CT<double2> {
  using R = double;
  __device__ static double2 zero() { return make_double2(0.0, 0.0); }
};
template <> struct CT<float2> {
  using R = float;
  __device__ static float2 zero() { return make_float2(0.f, 0.f); }
};

constexpr int BM = 64, BN = 64, BK = 16;

// 256 threads; thread (tx = tid % 16, ty = tid / 16) owns m = tx + 16*i, n = ty + 16*j.
template <typename T>
__device__ __forceinline__ void gemm_simt_tile(const T* __restrict__ A, const T* __restrict__ B,
                                               T* __restrict__ C, int64_t M, int64_t N, int64_t K,
                                               int64_t m0, int64_t n0, int64_t kb = 0, int64_t ke = -1) {
  // k range [kb, ke) of the row pitch K (split-K slices); ke < 0 means K
  if (ke < 0) ke = K;
  using R = typename CT<T>::R;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  R acc_r[4][4], acc_i[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) { acc_r[i][j] = 0; acc_i[i][j] = 0; }

  for (int64_t k0 = kb; k0 < ke; k0 += BK) {
    // load A tile: BM rows x BK cols = 1024 elements, 4 per thread; lanes walk k.
#pragma unroll
    for (int l = 0; l < (BM * BK) / 256; ++l) {
      const int e = tid + l * 256;
      const int r = e / BK, c = e % BK;
      const int64_t m = m0 + r, k = k0 + c;
      As[c][r] = (m < M && k < ke) ? A[m * K + k] : CT<T>::zero();
    }
#pragma unroll
    for (int l = 0; l < (BN * BK) / 256; ++l) {
      const int e = tid + l * 256;
      const int r = e / BK, c = e % BK;
      const int64_t n = n0 + r, k = k0 + c;
      Bs[c][r] = (n < N && k < ke) ? B[n * K + k] : CT<T>::zero();
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc_r[i][j] = fma(a[i].x, b[j].x, acc_r[i][j]);
          acc_r[i][j] = fma(-a[i].y, b[j].y, acc_r[i][j]);
          acc_i[i][j] = fma(a[i].x, b[j].y, acc_i[i][j]);
          acc_i[i][j] = fma(a[i].y, b[j].x, acc_i[i][j]);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int64_t n = n0 + ty + 16 * j;
    if (n >= N) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t m = m0 + tx + 16 * i;
      if (m < M) {
        T v;
        v.x = acc_r[i][j];
        v.y = acc_i[i][j];
        C[n * M + m] = v;
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) gemm_simt_kernel(const T* __restrict__ A, const T* __restrict__ B,
                                                        T* __restrict__ C, int64_t M, int64_t N,
                                                        int64_t K) {
  gemm_simt_tile<T>(A, B, C, M, N, K, (int64_t)blockIdx.x * BM, (int64_t)blockIdx.y * BN);
}

struct GemmJobsP {
  GemmJob j[kGemmJobMax];
  int tile_start[kGemmJobMax + 1];
  int tiles_m[kGemmJobMax];
  int n;
};

template <typename T>
__global__ void __launch_bounds__(256) gemm_simt_grouped_kernel(const __grid_constant__ GemmJobsP g) {
  const int b = blockIdx.x;
  int p = 0;
  while (p + 1 < g.n && g.tile_start[p + 1] <= b) ++p;
  const GemmJob& J = g.j[p];
  const int t = b - g.tile_start[p];
  gemm_simt_tile<T>(static_cast<const T*>(J.A), static_cast<const T*>(J.B), static_cast<T*>(J.C), J.M, J.N, J.K,
                    (int64_t)(t % g.tiles_m[p]) * BM, (int64_t)(t / g.tiles_m[p]) * BN);
}

template <typename T>
cudaError_t launch_grouped(const GemmJob* jobs, int njobs, cudaStream_t s) {
  for (int base = 0; base < njobs; base += kGemmJobMax) {
    const int cnt = std::min(kGemmJobMax, njobs - base);
    GemmJobsP g;
    std::memset(&g, 0, sizeof(g));
    int tiles = 0;
    for (int q = 0; q < cnt; ++q) {
      const GemmJob& J = jobs[base + q];
      g.j[q] = J;
      g.tiles_m[q] = (int)((J.M + BM - 1) / BM);
      g.tile_start[q] = tiles;
      tiles += (J.M > 0 && J.N > 0) ? g.tiles_m[q] * (int)((J.N + BN - 1) / BN) : 0;
    }
    g.tile_start[cnt] = tiles;
    g.n = cnt;
    if (tiles == 0) continue;
    gemm_simt_grouped_kernel<T><<<tiles, 256, 0, s>>>(g);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Skinny variant for N <= 32 (coupled-charge problems with a few output columns): B lives
// in shared memory, A is staged in 128-row x 16-column chunks through shared memory, and
// thread (r, g) of a 128*ng-thread CTA owns row r and the 8 columns n = 8g .. 8g+7.
constexpr int SK_ROWS = 128, SK_KC = 16, kSkinnyMaxN = 32;

struct SkinnyJobsP {
  GemmJob j[kGemmJobMax];
  int blk_start[kGemmJobMax + 1];
  int n;
};

template <typename T>
__global__ void __launch_bounds__(512) gemm_skinny_grouped_kernel(const __grid_constant__ SkinnyJobsP g) {
  extern __shared__ __align__(16) unsigned char sk_smem[];
  const int b = blockIdx.x;
  int p = 0;
  while (p + 1 < g.n && g.blk_start[p + 1] <= b) ++p;
  const GemmJob& J = g.j[p];
  const int64_t blk = b - g.blk_start[p], nblk = g.blk_start[p + 1] - g.blk_start[p];
  const T* __restrict__ A = static_cast<const T*>(J.A);
  const T* __restrict__ B = static_cast<const T*>(J.B);
  T* __restrict__ C = static_cast<T*>(J.C);
  const int64_t M = J.M;
  const int N = (int)J.N, K = (int)J.K;
  T* Bs = reinterpret_cast<T*>(sk_smem);
  T* As = Bs + (size_t)N * K;  // [SK_ROWS][SK_KC + 1]
  const int nthr = blockDim.x, tid = threadIdx.x;
  const int r = tid & (SK_ROWS - 1), n0 = (tid >> 7) * 8;
  for (int i = tid; i < N * K; i += nthr) Bs[i] = B[i];
  for (int64_t c0 = blk * SK_ROWS; c0 < M; c0 += nblk * SK_ROWS) {
    const int rows = (int)(M - c0 < SK_ROWS ? M - c0 : SK_ROWS);
    T acc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = CT<T>::zero();
    for (int k0 = 0; k0 < K; k0 += SK_KC) {
      const int kc = K - k0 < SK_KC ? K - k0 : SK_KC;
      __syncthreads();
      for (int e = tid; e < SK_ROWS * SK_KC; e += nthr) {
        const int rr = e >> 4, kk = e & (SK_KC - 1);
        As[rr * (SK_KC + 1) + kk] = (rr < rows && kk < kc) ? A[(c0 + rr) * K + k0 + kk] : CT<T>::zero();
      }
      __syncthreads();
      for (int kk = 0; kk < kc; ++kk) {
        const T a = As[r * (SK_KC + 1) + kk];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (n0 + j < N) {
            const T bv = Bs[(n0 + j) * K + k0 + kk];
            acc[j].x = fma(a.x, bv.x, acc[j].x);
            acc[j].x = fma(-a.y, bv.y, acc[j].x);
            acc[j].y = fma(a.x, bv.y, acc[j].y);
            acc[j].y = fma(a.y, bv.x, acc[j].y);
          }
        }
      }
    }
    if (r < rows) {
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (n0 + j < N) C[(int64_t)(n0 + j) * M + c0 + r] = acc[j];
    }
  }
}

template <typename T>
size_t skinny_smem(const GemmJob& J) {
  return ((size_t)J.N * J.K + (size_t)SK_ROWS * (SK_KC + 1)) * sizeof(T);
}

template <typename T>
cudaError_t launch_skinny(const GemmJob* jobs, int njobs, cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(gemm_skinny_grouped_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kSkinnyMaxSmem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  for (int base = 0; base < njobs; base += kGemmJobMax) {
    const int cnt = std::min(kGemmJobMax, njobs - base);
    SkinnyJobsP g;
    std::memset(&g, 0, sizeof(g));
    int blocks = 0, maxn = 1;
    size_t smem = 0;
    for (int q = 0; q < cnt; ++q) {
      const GemmJob& J = jobs[base + q];
      if (J.N > kSkinnyMaxN || skinny_smem<T>(J) > (size_t)kSkinnyMaxSmem) return cudaErrorInvalidValue;
      g.j[q] = J;
      g.blk_start[q] = blocks;
      int64_t nb = (J.M + SK_ROWS - 1) / SK_ROWS;
      if (nb > 1024) nb = 1024;
      blocks += (J.M > 0 && J.N > 0) ? (int)nb : 0;
      smem = std::max(smem, skinny_smem<T>(J));
      maxn = std::max(maxn, (int)J.N);
    }
    g.blk_start[cnt] = blocks;
    g.n = cnt;
    if (blocks == 0) continue;
    const int threads = SK_ROWS * ((maxn + 7) / 8);
    gemm_skinny_grouped_kernel<T><<<blocks, threads, smem, s>>>(g);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Narrow tile for split-K products with few output columns: 64 x 16, thread (tx, ty) of
// 16 x 16 owns m = tx + 16 i (i < 4) and n = ty.
template <typename T>
__device__ __forceinline__ void gemm_simt_tile_n16(const T* __restrict__ A, const T* __restrict__ B,
                                                   T* __restrict__ C, int64_t M, int64_t N, int64_t K, int64_t m0,
                                                   int64_t kb, int64_t ke) {
  using R = typename CT<T>::R;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][16 + 1];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  R acc_r[4], acc_i[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) { acc_r[i] = 0; acc_i[i] = 0; }
  for (int64_t k0 = kb; k0 < ke; k0 += BK) {
#pragma unroll
    for (int l = 0; l < (BM * BK) / 256; ++l) {
      const int e = tid + l * 256;
      const int r = e / BK, c = e % BK;
      const int64_t m = m0 + r, k = k0 + c;
      As[c][r] = (m < M && k < ke) ? A[m * K + k] : CT<T>::zero();
    }
    {
      const int r = tid / BK, c = tid % BK;
      const int64_t k = k0 + c;
      Bs[c][r] = (r < N && k < ke) ? B[(int64_t)r * K + k] : CT<T>::zero();
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      const T b = Bs[kk][ty];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const T a = As[kk][tx + 16 * i];
        acc_r[i] = fma(a.x, b.x, acc_r[i]);
        acc_r[i] = fma(-a.y, b.y, acc_r[i]);
        acc_i[i] = fma(a.x, b.y, acc_i[i]);
        acc_i[i] = fma(a.y, b.x, acc_i[i]);
      }
    }
    __syncthreads();
  }
  if (ty < N) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t m = m0 + tx + 16 * i;
      if (m < M) {
        T v;
        v.x = acc_r[i];
        v.y = acc_i[i];
        C[(int64_t)ty * M + m] = v;
      }
    }
  }
}

// Split-K: slice z of gridDim.z computes the partial product over its k range into
// P[z][N][M]; splitk_reduce_kernel sums the slices in order (deterministic).
template <typename T, bool N16>
__global__ void __launch_bounds__(256) gemm_simt_splitk_kernel(const T* __restrict__ A, const T* __restrict__ B,
                                                               T* __restrict__ P, int64_t M, int64_t N, int64_t K,
                                                               int64_t kchunk) {
  const int64_t kb = (int64_t)blockIdx.z * kchunk;
  const int64_t ke = kb + kchunk < K ? kb + kchunk : K;
  if (N16)
    gemm_simt_tile_n16<T>(A, B, P + (int64_t)blockIdx.z * M * N, M, N, K, (int64_t)blockIdx.x * BM, kb, ke);
  else
    gemm_simt_tile<T>(A, B, P + (int64_t)blockIdx.z * M * N, M, N, K, (int64_t)blockIdx.x * BM,
                      (int64_t)blockIdx.y * BN, kb, ke);
}

template <typename T>
__global__ void splitk_reduce_kernel(const T* __restrict__ P, int S, int64_t MN, T* __restrict__ C) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < MN; i += (int64_t)gridDim.x * blockDim.x) {
    T acc = P[i];
    for (int z = 1; z < S; ++z) {
      const T v = P[(int64_t)z * MN + i];
      acc.x += v.x;
      acc.y += v.y;
    }
    C[i] = acc;
  }
}

template <typename T>
cudaError_t launch(const T* A, const T* B, T* C, int64_t M, int64_t N, int64_t K, cudaStream_t s) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  const int64_t gx = (M + BM - 1) / BM, gy = (N + BN - 1) / BN;
  if (gy > 65535) return cudaErrorInvalidConfiguration;
  gemm_simt_kernel<T><<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(A, B, C, M, N, K);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_splitk(const T* A, const T* B, T* C, int64_t M, int64_t N, int64_t K, int S, T* P,
                          cudaStream_t s) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  const int64_t gx = (M + BM - 1) / BM, gy = (N + BN - 1) / BN;
  if (gy > 65535 || S < 1 || S > 65535) return cudaErrorInvalidConfiguration;
  int64_t kchunk = (K + S - 1) / S;
  kchunk = (kchunk + BK - 1) / BK * BK;
  const int Se = (int)((K + kchunk - 1) / kchunk);
  if (N <= 16)
    gemm_simt_splitk_kernel<T, true><<<dim3((unsigned)gx, 1u, (unsigned)Se), 256, 0, s>>>(A, B, P, M, N, K, kchunk);
  else
    gemm_simt_splitk_kernel<T, false><<<dim3((unsigned)gx, (unsigned)gy, (unsigned)Se), 256, 0, s>>>(A, B, P, M, N, K,
                                                                                                   kchunk);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int64_t MN = M * N;
  int64_t blocks = (MN + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  splitk_reduce_kernel<T><<<(unsigned)(blocks < 1 ? 1 : blocks), 256, 0, s>>>(P, Se, MN, C);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_zgemm_simt(const double2* A, const double2* B, double2* C, int64_t M, int64_t N,
                              int64_t K, cudaStream_t s) {
  return launch(A, B, C, M, N, K, s);
}
int gemm_splitk_slices(int64_t M, int64_t N, int64_t K) {
  const int64_t tiles = ((M + BM - 1) / BM) * (N <= 16 ? 1 : (N + BN - 1) / BN);
  if (tiles >= 2 * 152 || K < 8 * BK * 16) return 1;
  int64_t S = (2 * 152) / tiles;
  const int64_t kmax = K / (BK * 16);  // at least 256 k per slice
  if (S > kmax) S = kmax;
  if (S > 256) S = 256;
  return S < 2 ? 1 : (int)S;
}
cudaError_t launch_zgemm_simt_splitk(const double2* A, const double2* B, double2* C, int64_t M, int64_t N, int64_t K,
                                     int S, double2* P, cudaStream_t s) {
  return launch_splitk(A, B, C, M, N, K, S, P, s);
}
cudaError_t launch_cgemm_simt_splitk(const float2* A, const float2* B, float2* C, int64_t M, int64_t N, int64_t K,
                                     int S, float2* P, cudaStream_t s) {
  return launch_splitk(A, B, C, M, N, K, S, P, s);
}
cudaError_t launch_gemm_simt_grouped(const GemmJob* jobs, int njobs, int is64, cudaStream_t s) {
  return is64 ? launch_grouped<double2>(jobs, njobs, s) : launch_grouped<float2>(jobs, njobs, s);
}
cudaError_t launch_gemm_skinny_grouped(const GemmJob* jobs, int njobs, int is64, cudaStream_t s) {
  return is64 ? launch_skinny<double2>(jobs, njobs, s) : launch_skinny<float2>(jobs, njobs, s);
}
bool gemm_skinny_fits(int64_t N, int64_t K, int is64) {
  const size_t e = is64 ? sizeof(double2) : sizeof(float2);
  return N >= 1 && N <= kSkinnyMaxN && ((size_t)N * K + (size_t)SK_ROWS * (SK_KC + 1)) * e <= (size_t)kSkinnyMaxSmem;
}
cudaError_t launch_cgemm_simt(const float2* A, const float2* B, float2* C, int64_t M, int64_t N,
                              int64_t K, cudaStream_t s) {
  return launch(A, B, C, M, N, K, s);
}
