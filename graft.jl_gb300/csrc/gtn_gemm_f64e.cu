// FP64-grade complex GEMM on the bf16 tensor cores (tcgen05), for the contractions that
// must stay FP64-accurate: environment updates, the Rayleigh quotients and residuals of the
// Krylov refinement.  On this part FP64 runs at about 1.2 TFLOP/s, more than a thousand
// times below the bf16 tensor rate; this kernel trades that for exact integer arithmetic.
//
// Method (the fixed-point splitting of Ozaki, Ogita, Oishi and Rump, Numer. Algorithms 59
// (2012), with exact chunked accumulation):
//   * every row of the real-expanded A (and every complex row of B') is scaled by a power
//     of two 2^k so that its entries lie in (-1, 1), then written as S = 7 signed base-128
//     digits, a = sum_i d_i 2^{-7(i+1)}, |d_0| <= 128, |d_i| <= 64; each digit is an integer
//     that bf16 holds exactly (the digit planes are built by split_i7 / pack_b_planes_i7);
//   * the digit products d_i e_j with i + j <= 6 (28 of them) are summed on the tensor
//     cores, one TMEM accumulator per level s = i + j (7 levels x 64 columns).  Every
//     product of two digits is an integer below 2^14 and a level gets at most
//     2 * 2^13 + 5 * 2^12 per k, so over a chunk of 256 k the FP32 sums are exact integers;
//   * after each chunk the epilogue warps read the levels and add 2^{-7(s+2)} L_s into a
//     double-float accumulator (pairs of FP32 with error-free TwoSum updates, about 48
//     significant bits); the result is scaled back by 2^{-(k_row + k_col)} into FP64.
// The terms left out (i + j >= 7) and the digits beyond the seventh are below 2^-49 of the
// row maxima, so each output is accurate to about 1e-14 relative to sum_k |a_k| |b_k|.
//
// Tile: 128 rows x 64 real columns (32 complex) per CTA; stages of 16 k (SWIZZLE_32B rows
// of 32 bytes) holding all 7 digit planes of A and of B'; warp 0 issues TMA, warp 1 the
// MMAs (tcgen05.mma.cta_group::1.kind::f16, bf16 x bf16 -> f32), warps 2-9 drain the
// levels (warp w reads TMEM lanes 32 (w % 4) .. + 31, columns (w - 2) / 4 * 32 .. + 31).
// Every mbarrier wait is bounded as in the other tcgen05 kernels.
#include "gtn_internal.h"
#include "gtn_tcgen05.h"

#include <algorithm>

namespace {
using namespace gtn_tc;

constexpr int kS = kF64eSlices;                  // digits per value
constexpr int kLevels = kS;                      // levels s = i + j <= kS - 1
constexpr int kBM = 128;
constexpr int kBN = 64;                          // real columns (32 complex outputs)
constexpr int kBK = 16;                          // real k per stage (one 32-byte row)
constexpr int kPlaneA = kBM * kBK * 2;           // 4 KB
constexpr int kPlaneB = kBN * kBK * 2;           // 2 KB
constexpr int kStageBytes = kS * (kPlaneA + kPlaneB);
constexpr int kStages = (228352 - 4096) / kStageBytes > 8 ? 8 : (228352 - 4096) / kStageBytes;
constexpr int kSmem = kStages * kStageBytes + 1024;
constexpr int kChunkStages = 16;                 // 256 real k per exact chunk
constexpr uint32_t kTmemCols = 512;              // 7 levels x 64 columns = 448
constexpr int kThreads = 320;
static_assert(kStages >= 3, "operand ring");
static_assert(kLevels * kBN <= (int)kTmemCols, "TMEM columns");

// Power-of-two exponent k with |x| 2^k < 1 for every |x| <= mx (mx a float row maximum).
__device__ __forceinline__ int row_exp(float mx) {
  const uint32_t b = __float_as_uint(mx);
  const int e = (int)((b >> 23) & 0xffu);
  return mx > 0.f ? 126 - e : 0;
}

// x = hi + lo (double-float) += v, error-free (Knuth TwoSum) with the error kept in lo.
__device__ __forceinline__ void df_add(float& hi, float& lo, float v) {
  const float s = hi + v;
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (v - bb);
  hi = s;
  lo += err;
}

__global__ void __launch_bounds__(kThreads, 1)
    f64e_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     double2* __restrict__ C, int64_t M, int64_t N, int nkb, const float* __restrict__ amax,
                     const float* __restrict__ bmax, int* __restrict__ errflag, int tiles_n) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  __shared__ __align__(8) uint64_t full_bar[kStages];
  __shared__ __align__(8) uint64_t empty_bar[kStages];
  __shared__ __align__(8) uint64_t chunk_full, chunk_empty;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  __shared__ int n_issued, n_consumed;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = (int)(blockIdx.x / tiles_n) * kBM, r0 = (int)(blockIdx.x % tiles_n) * kBN;
  const int nchunks = (nkb + kChunkStages - 1) / kChunkStages;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&chunk_full, 1);
    mbar_init(&chunk_empty, 8);
    abort_flag = 0;
    n_issued = 0;
    n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem_base = tmem_slot;

  if (warp == 0 && lane == 0) {
    int it = 0;
    for (; it < nkb; ++it) {
      const int s = it % kStages;
      const uint32_t ph = (uint32_t)(it / kStages) & 1u;
      if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_flag)) {
        abort_flag = 1;
        atomicCAS(errflag, 0, DEVERR_TMA_TIMEOUT);
        break;
      }
      const uint32_t sa = smem_u32(smem + s * kStageBytes);
      const uint32_t sb = sa + kS * kPlaneA;
      mbar_expect_tx(&full_bar[s], kStageBytes);
#pragma unroll
      for (int p = 0; p < kS; ++p) {
        tma_load_3d(sa + p * kPlaneA, &tmA, &full_bar[s], it * kBK, m0, p);
        tma_load_3d(sb + p * kPlaneB, &tmB, &full_bar[s], it * kBK, r0, p);
      }
    }
    n_issued = it;
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = idesc_bf16(kBM, kBN);
    int it = 0;
    bool stop = false;
    for (int c = 0; c < nchunks && !stop; ++c) {
      // the levels are free once the epilogue drained the previous chunk
      if (!mbar_wait(&chunk_empty, ((uint32_t)c & 1u) ^ 1u, &abort_flag)) {
        abort_flag = 1;
        atomicCAS(errflag, 0, DEVERR_MMA_TIMEOUT);
        break;
      }
      fence_after();
      bool started[kLevels];
#pragma unroll
      for (int l = 0; l < kLevels; ++l) started[l] = false;
      const int kb_end = std::min(nkb, (c + 1) * kChunkStages);
      for (; it < kb_end; ++it) {
        const int s = it % kStages;
        const uint32_t ph = (uint32_t)(it / kStages) & 1u;
        if (!mbar_wait(&full_bar[s], ph, &abort_flag)) {
          abort_flag = 1;
          atomicCAS(errflag, 0, DEVERR_MMA_TIMEOUT);
          stop = true;
          break;
        }
        fence_after();
        const uint32_t sa = smem_u32(smem + s * kStageBytes);
        const uint32_t sb = sa + kS * kPlaneA;
#pragma unroll
        for (int i = 0; i < kS; ++i) {
#pragma unroll
          for (int j = 0; j + i < kLevels; ++j) {
            const int l = i + j;
            umma_bf16(tmem_base + (uint32_t)(l * kBN), sdesc32(sa + i * kPlaneA), sdesc32(sb + j * kPlaneB), idesc,
                      started[l] ? 1u : 0u);
            started[l] = true;
          }
        }
        umma_commit(&empty_bar[s]);
      }
      umma_commit(&chunk_full);  // the chunk's levels are complete once its MMAs are
    }
    n_consumed = it;
  } else if (warp >= 2) {
    const int q4 = warp & 3;             // TMEM lane quarter
    const int half = (warp - 2) >> 2;    // column half
    const int row = q4 * 32 + lane;
    const int64_t m = (int64_t)m0 + row;
    float hi[32], lo[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) hi[j] = lo[j] = 0.f;
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
      if (!mbar_wait(&chunk_full, (uint32_t)c & 1u, &abort_flag)) {
        if (lane == 0) {
          abort_flag = 1;
          atomicCAS(errflag, 0, DEVERR_EPI_TIMEOUT);
        }
        ok = false;
        break;
      }
      __syncwarp();
      fence_after();
#pragma unroll 1
      for (int l = 0; l < kLevels; ++l) {
        uint32_t v[32];
        tmem_ld32(tmem_base + (uint32_t)(l * kBN + half * 32) + ((uint32_t)(q4 * 32) << 16), v);
        const float w = __uint_as_float((uint32_t)(127 - 7 * (l + 2)) << 23);  // 2^{-7(l+2)}, exact
#pragma unroll
        for (int j = 0; j < 32; ++j) df_add(hi[j], lo[j], __uint_as_float(v[j]) * w);
      }
#pragma unroll
      for (int j = 0; j < 32; ++j) {  // renormalise (FastTwoSum, |hi| >= |lo|)
        const float s = hi[j] + lo[j];
        lo[j] = lo[j] - (s - hi[j]);
        hi[j] = s;
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive_local(&chunk_empty);
    }
    if (ok && m < M) {
      const int ka = row_exp(amax[m]);
      const int64_t nb = (int64_t)(r0 + half * 32) >> 1;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int64_t n = nb + j;
        if (n < N) {
          const int kb = row_exp(bmax[n]);
          const double sc = ldexp(1.0, -(ka + kb));
          C[n * M + m] = make_double2(((double)hi[2 * j] + (double)lo[2 * j]) * sc,
                                      ((double)hi[2 * j + 1] + (double)lo[2 * j + 1]) * sc);
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {  // copies issued but never consumed (abort path only) land before exit
    for (int it = n_consumed; it < n_issued; ++it) {
      volatile int no_abort = 0;
      mbar_wait(&full_bar[it % kStages], (uint32_t)(it / kStages) & 1u, &no_abort);
    }
  }
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(kTmemCols) : "memory");
  }
}

// 3-D map over the digit planes: (2Kp elements, rows, planes), box (16, box_rows, 1), 32B swizzle.
bool make_map32(CUtensorMap* tm, const void* base, int64_t Kp, int64_t rows, int planes, int box_rows,
                std::string* why) {
  EncodeTiledFn enc = get_encode();
  if (!enc) {
    if (why) *why = "cuTensorMapEncodeTiled unavailable";
    return false;
  }
  cuuint64_t gdim[3] = {(cuuint64_t)(2 * Kp), (cuuint64_t)rows, (cuuint64_t)planes};
  cuuint64_t gstr[2] = {(cuuint64_t)(2 * Kp * 2), (cuuint64_t)(rows * 2 * Kp * 2)};
  cuuint32_t box[3] = {(cuuint32_t)kBK, (cuuint32_t)box_rows, 1u};
  cuuint32_t estr[3] = {1u, 1u, 1u};
  CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), gdim, gstr, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    if (why) *why = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
    return false;
  }
  return true;
}

}  // namespace

cudaError_t launch_f64e_gemm(const F64eGemmArgs& a, int* errflag, cudaStream_t s, std::string* why) {
  if (a.M <= 0 || a.N <= 0) return cudaSuccess;
  if (a.Kp % 32 != 0 || !a.A || !a.B || !a.C || !a.a_max || !a.b_max) {
    if (why) *why = "f64e_gemm: Kp must be a multiple of 32 and every operand given";
    return cudaErrorInvalidValue;
  }
  if (reinterpret_cast<uintptr_t>(a.A) % 16 || reinterpret_cast<uintptr_t>(a.B) % 16) {
    if (why) *why = "f64e_gemm: digit planes must be 16-byte aligned";
    return cudaErrorInvalidValue;
  }
  CUtensorMap tmA, tmB;
  if (!make_map32(&tmA, a.A, a.Kp, a.M, kS, kBM, why)) return cudaErrorInvalidValue;
  if (!make_map32(&tmB, a.B, a.Kp, 2 * a.N, kS, kBN, why)) return cudaErrorInvalidValue;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(f64e_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const int nkb = (int)(2 * a.Kp / kBK);
  const int64_t gx = (a.M + kBM - 1) / kBM;
  const int64_t gy = (2 * a.N + kBN - 1) / kBN;
  if (gx * gy > 2147483647LL) return cudaErrorInvalidConfiguration;
  f64e_gemm_kernel<<<(unsigned)(gx * gy), kThreads, kSmem, s>>>(tmA, tmB, a.C, a.M, a.N, nkb, a.a_max, a.b_max,
                                                               errflag, (int)gy);
  return cudaGetLastError();
}
