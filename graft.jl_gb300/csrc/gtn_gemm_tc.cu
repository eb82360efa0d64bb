// tcgen05 split-precision GEMM for sm_103a.
//
// Real GEMM  C_real[M x 2N] = A_real[M x 2K] * B'_real[2N x 2K]^T  on bf16 slice planes,
// FP32 accumulation in TMEM.  A_real is the complex operand with (re, im) interleaved
// along K; B' is the expanded static operand [[Br, -Bi], [Bi, Br]] so that column pair
// (2n, 2n+1) of C_real is the complex output n.  Split precision: A ~ sum_p A_p,
// B' ~ sum_q B_q (bf16 slices); the product list (p, q) is accumulated into one TMEM
// accumulator as a longer K loop.
//
// One CTA (128 threads) per 128 x BN output tile:
//   warp 0 lane 0 : TMA producer (cp.async.bulk.tensor.3d, SWIZZLE_128B; each CTA loads its own tiles)
//   warp 1 lane 0 : tcgen05.mma issuer (kind::f16, bf16 x bf16 -> f32)
//   warp 2        : TMEM allocator
//   warps 0-3     : epilogue (tcgen05.ld 32x32b -> complex FP32 stores, m-fastest)
// Every mbarrier wait is bounded (globaltimer, 4 s); on timeout the CTA records an error
// code in the context's device flag, drains its own copies and MMAs, frees TMEM, returns.
#include "gtn_internal.h"
#include "gtn_tcgen05.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

namespace {
using namespace gtn_tc;

constexpr int BM = 128;
constexpr int BKE = 64;  // bf16 elements per k-block = 128 bytes = one SW128 row
constexpr int A_BYTES = BM * BKE * 2;

constexpr int kTcGroupMax = 56;

struct ProdList {
  int n;
  int a[9];
  int b[9];
};

// A wait that runs out: an mbarrier expecting one arrival that never comes.
__global__ void wait_selftest_kernel(int* __restrict__ errflag, uint64_t timeout_ns) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ volatile int no_abort;
  mbar_init(&bar, 1);
  no_abort = 0;
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  if (!mbar_wait(&bar, 0u, &no_abort, timeout_ns)) atomicCAS(errflag, 0, DEVERR_SELFTEST_TIMEOUT);
}

template <int BN> struct Cfg {
  static constexpr int B_BYTES = BN * BKE * 2;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int STAGES = (196608 / STAGE_BYTES) > 8 ? 8 : (196608 / STAGE_BYTES);
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024;
  static constexpr uint32_t TMEM_COLS = BN < 32 ? 32 : BN;
};

// One 128 x BN output tile of C = A * B'^T (all roles of the CTA).
template <int BN>
__device__ __forceinline__ void tc_tile(const CUtensorMap* tmA, const CUtensorMap* tmB, float2* __restrict__ C,
                                        int64_t M, int64_t N, int nkb, const ProdList& prods, int m0, int r0,
                                        int* __restrict__ errflag) {
  using CF = Cfg<BN>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  __shared__ __align__(8) uint64_t full_bar[CF::STAGES];
  __shared__ __align__(8) uint64_t empty_bar[CF::STAGES];
  __shared__ __align__(8) uint64_t accum_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  __shared__ int n_issued, n_consumed;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < CF::STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&accum_bar, 1);
    abort_flag = 0;
    n_issued = 0;
    n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tmA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tmB)) : "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(CF::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem_d = tmem_slot;

  const int total = prods.n * nkb;

  if (warp == 0 && lane == 0) {
    int it = 0;
    for (; it < total; ++it) {
      const int s = it % CF::STAGES;
      const uint32_t ph = (uint32_t)(it / CF::STAGES) & 1u;
      if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_flag)) {
        abort_flag = 1;
        atomicCAS(errflag, 0, DEVERR_TMA_TIMEOUT);
        break;
      }
      const int p = it / nkb, kb = it - p * nkb;
      const uint32_t sa = smem_u32(smem + s * CF::STAGE_BYTES);
      const uint32_t sb = sa + A_BYTES;
      mbar_expect_tx(&full_bar[s], CF::STAGE_BYTES);
      tma_load_3d(sa, tmA, &full_bar[s], kb * BKE, m0, prods.a[p]);
      tma_load_3d(sb, tmB, &full_bar[s], kb * BKE, r0, prods.b[p]);
    }
    n_issued = it;
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = idesc_bf16(BM, BN);
    int it = 0;
    for (; it < total; ++it) {
      const int s = it % CF::STAGES;
      const uint32_t ph = (uint32_t)(it / CF::STAGES) & 1u;
      if (!mbar_wait(&full_bar[s], ph, &abort_flag)) {
        abort_flag = 1;
        atomicCAS(errflag, 0, DEVERR_MMA_TIMEOUT);
        break;
      }
      fence_after();
      const uint32_t sa = smem_u32(smem + s * CF::STAGE_BYTES);
      const uint32_t sb = sa + A_BYTES;
#pragma unroll
      for (int kk = 0; kk < BKE / 16; ++kk) {
        umma_bf16(tmem_d, sdesc(sa + kk * 32), sdesc(sb + kk * 32), idesc,
                  (it > 0 || kk > 0) ? 1u : 0u);
      }
      umma_commit(&empty_bar[s]);
    }
    n_consumed = it;
    umma_commit(&accum_bar);  // arrives once every MMA issued above has completed
  }
  __syncwarp();

  // ---- epilogue: TMEM -> registers -> complex FP32 stores (C[n][m], m fastest) ----------
  const bool ok = mbar_wait(&accum_bar, 0u, &abort_flag);
  if (!ok && lane == 0) {
    abort_flag = 1;
    atomicCAS(errflag, 0, DEVERR_EPI_TIMEOUT);
  }
  __syncwarp();
  fence_after();
  if (ok) {
    const int row = warp * 32 + lane;
    const int64_t m = (int64_t)m0 + row;
    const uint32_t taddr = tmem_d + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c = 0; c < BN; c += 16) {
      uint32_t v[16];
      tmem_ld16(taddr + (uint32_t)c, v);
      if (m < M) {
        const int64_t nb = (int64_t)(r0 + c) >> 1;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int64_t n = nb + j;
          if (n < N) C[n * M + m] = make_float2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]));
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  // Drain: copies issued but never consumed (abort path only) must land before exit.
  if (threadIdx.x == 0) {
    for (int it = n_consumed; it < n_issued; ++it) {
      volatile int no_abort = 0;
      mbar_wait(&full_bar[it % CF::STAGES], (uint32_t)(it / CF::STAGES) & 1u, &no_abort);
    }
  }
  __syncthreads();
  if (warp == 2) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d),
                 "r"(CF::TMEM_COLS)
                 : "memory");
  }
}

// Variant: every stage holds all P slice planes of A and of B' for one 32-wide k-block
// (SWIZZLE_64B rows of 64 B), and the MMA thread issues every slice product from that
// stage.  Operand bytes per MAC drop by the number of products that share a plane
// (6 products from 3+3 planes for bf16x6), relieving L2->SM bandwidth.  Because the
// products of one k-block are interleaved, the leading product (plane 0 x plane 0) and
// the correction products accumulate in two TMEM accumulators that the epilogue adds:
// the corrections then never round against the leading product's running sum.
constexpr int BKE2 = 32;
// CPS = CTAs resident per SM: with 2, one CTA's epilogue overlaps the other's mainloop
// (short-K steps, where the prologue and epilogue of a one-tile CTA dominate).
// Threads of a split-plane tile CTA: warps 0-3 hold the TMA, MMA and TMEM-allocation roles
// (one lane each), and all 8 warps drain the accumulators (two per TMEM lane quarter).
constexpr int kPsThreads = 256;

template <int BN, int P, int CPS = 1> struct Cfg2 {
  static constexpr int A_PLANE = BM * BKE2 * 2;   // 8 KB
  static constexpr int B_PLANE = BN * BKE2 * 2;
  static constexpr int STAGE_BYTES = P * (A_PLANE + B_PLANE);
  static constexpr int ST = (228352 / CPS - 2048) / STAGE_BYTES;
  static constexpr int STAGES = ST > 8 ? 8 : ST;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024;
  static constexpr uint32_t ACC_COLS = BN < 32 ? 32 : BN;   // column offset of the correction accumulator
  static constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;
  static_assert(STAGES >= 2, "the operand ring needs two stages");
  static_assert(CPS * TMEM_COLS <= 512, "TMEM columns of the resident CTAs");
};

// Optional fp16 row scales of the slice planes (the scale that was applied to each row
// of A and complex row of B, divided out in the epilogue).
struct PlaneScales {
  const float* amax;
  const float* bmax;
  int fp16;
};

template <int BN, int P, int CPS>
__device__ __forceinline__ void tc_tile_ps(const CUtensorMap* tmA, const CUtensorMap* tmB, float2* __restrict__ C,
                                           int64_t M, int64_t N, int nkb, const ProdList& prods, int m0, int r0,
                                           int* __restrict__ errflag, const PlaneScales& sc) {
  using CF = Cfg2<BN, P, CPS>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  __shared__ __align__(8) uint64_t full_bar[CF::STAGES];
  __shared__ __align__(8) uint64_t empty_bar[CF::STAGES];
  __shared__ __align__(8) uint64_t accum_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  __shared__ int n_issued, n_consumed;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < CF::STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&accum_bar, 1);
    abort_flag = 0;
    n_issued = 0;
    n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tmA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tmB)) : "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(CF::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  // inverse fp16 scales of the tile's complex columns, read once here instead of per output
  __shared__ float s_binv[BN / 2 > 0 ? BN / 2 : 1];
  if (sc.bmax)
    for (int t = threadIdx.x; t < BN / 2; t += blockDim.x) {
      const int64_t n = (int64_t)(r0 >> 1) + t;
      s_binv[t] = n < N ? fp16_row_scale_inv(sc.bmax[n]) : 1.0f;
    }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem_d = tmem_slot;
  const int total = nkb;

  if (warp == 0 && lane == 0) {
    int it = 0;
    for (; it < total; ++it) {
      const int s = it % CF::STAGES;
      const uint32_t ph = (uint32_t)(it / CF::STAGES) & 1u;
      if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_flag)) {
        abort_flag = 1;
        atomicCAS(errflag, 0, DEVERR_TMA_TIMEOUT);
        break;
      }
      const uint32_t sa = smem_u32(smem + s * CF::STAGE_BYTES);
      const uint32_t sb = sa + P * CF::A_PLANE;
      mbar_expect_tx(&full_bar[s], CF::STAGE_BYTES);
#pragma unroll
      for (int p = 0; p < P; ++p) {
        tma_load_3d(sa + p * CF::A_PLANE, tmA, &full_bar[s], it * BKE2, m0, p);
        tma_load_3d(sb + p * CF::B_PLANE, tmB, &full_bar[s], it * BKE2, r0, p);
      }
    }
    n_issued = it;
  } else if (warp == 1 && lane == 0) {
    const uint32_t idesc = sc.fp16 ? idesc_f16(BM, BN) : idesc_bf16(BM, BN);
    bool lead_started = false, corr_started = false;
    int it = 0;
    for (; it < total; ++it) {
      const int s = it % CF::STAGES;
      const uint32_t ph = (uint32_t)(it / CF::STAGES) & 1u;
      if (!mbar_wait(&full_bar[s], ph, &abort_flag)) {
        abort_flag = 1;
        atomicCAS(errflag, 0, DEVERR_MMA_TIMEOUT);
        break;
      }
      fence_after();
      const uint32_t sa = smem_u32(smem + s * CF::STAGE_BYTES);
      const uint32_t sb = sa + P * CF::A_PLANE;
      for (int q = 0; q < prods.n; ++q) {
        const uint32_t a0 = sa + prods.a[q] * CF::A_PLANE;
        const uint32_t b0 = sb + prods.b[q] * CF::B_PLANE;
        const bool lead = prods.a[q] == 0 && prods.b[q] == 0;
        const uint32_t d = lead ? tmem_d : tmem_d + CF::ACC_COLS;
#pragma unroll
        for (int kk = 0; kk < BKE2 / 16; ++kk) {
          umma_bf16(d, sdesc64(a0 + kk * 32), sdesc64(b0 + kk * 32), idesc,
                    (lead ? lead_started : corr_started) ? 1u : 0u);
          if (lead) lead_started = true; else corr_started = true;
        }
      }
      umma_commit(&empty_bar[s]);
    }
    n_consumed = it;
    umma_commit(&accum_bar);
  }
  __syncwarp();

  const bool ok = mbar_wait(&accum_bar, 0u, &abort_flag);
  if (!ok && lane == 0) {
    abort_flag = 1;
    atomicCAS(errflag, 0, DEVERR_EPI_TIMEOUT);
  }
  __syncwarp();
  fence_after();
  if (ok) {
    // 8 warps: warp w drains TMEM lane quarter w % 4, columns of half w / 4 of the tile
    const int q4 = warp & 3, c0 = (warp >> 2) * (BN / 2);
    const int row = q4 * 32 + lane;
    const int64_t m = (int64_t)m0 + row;
    const uint32_t taddr = tmem_d + ((uint32_t)(q4 * 32) << 16);
    bool has_corr = false;
    for (int q = 0; q < prods.n; ++q) has_corr |= !(prods.a[q] == 0 && prods.b[q] == 0);
    const float ainv = (sc.amax && m < M) ? fp16_row_scale_inv(sc.amax[m]) : 1.0f;
#pragma unroll 1
    for (int c = c0; c < c0 + BN / 2; c += 16) {
      uint32_t v[16], w[16];
      tmem_ld16(taddr + (uint32_t)c, v);
      if (has_corr) {
        tmem_ld16(taddr + CF::ACC_COLS + (uint32_t)c, w);
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) w[j] = 0u;
      }
      if (m < M) {
        const int64_t nb = (int64_t)(r0 + c) >> 1;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int64_t n = nb + j;
          if (n < N) {
            const float f = sc.bmax ? ainv * s_binv[(c >> 1) + j] : ainv;
            C[n * M + m] = make_float2((__uint_as_float(v[2 * j]) + __uint_as_float(w[2 * j])) * f,
                                       (__uint_as_float(v[2 * j + 1]) + __uint_as_float(w[2 * j + 1])) * f);
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int it = n_consumed; it < n_issued; ++it) {
      volatile int no_abort = 0;
      mbar_wait(&full_bar[it % CF::STAGES], (uint32_t)(it / CF::STAGES) & 1u, &no_abort);
    }
  }
  __syncthreads();
  if (warp == 2) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d),
                 "r"(CF::TMEM_COLS)
                 : "memory");
  }
}

template <int BN, int P, int CPS>
__global__ void __launch_bounds__(kPsThreads, CPS)
    tc_gemm_ps_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      float2* __restrict__ C, int64_t M, int64_t N, int nkb, ProdList prods,
                      int* __restrict__ errflag, PlaneScales sc, int tiles_n) {
  // N tile fastest: the CTAs that run together share their A tiles through L2
  tc_tile_ps<BN, P, CPS>(&tmA, &tmB, C, M, N, nkb, prods, (int)(blockIdx.x / tiles_n) * BM, (int)(blockIdx.x % tiles_n) * BN,
                    errflag, sc);
}

// ---- SM pairs: tcgen05.mma.cta_group::2 ------------------------------------------------
// A cluster of two CTAs on two SMs computes one 256 x 256 tile of the real product as
// M = 256 MMAs.  Each CTA stages its own 128 rows of A and its own 128 rows of B' (half of
// the N tile) for every slice plane of a k-block; the even CTA (the leader) issues every
// MMA, which reads both CTAs' shared memory at the same offsets and writes each CTA's 128
// rows of the accumulators into that CTA's TMEM (all 256 columns).  Per SM the operand
// bytes per MAC are 2/3 of a one-CTA 128 x 256 tile: 256 rows of operands per k-block
// against 384.  Both TMEM accumulators (leading product, corrections) take 256 columns.
//
// Cross-CTA hand-offs (no copy or commit goes to several CTAs at once):
//   * both CTAs' TMA copies of a stage complete on the leader's full barrier (the
//     .cta_group::2 form of cp.async.bulk.tensor); the leader's producer announces the
//     bytes of both halves;
//   * the leader's MMA thread commits each stage to the empty barriers of both CTAs (one
//     commit per barrier) and the finished accumulators to both accumulator barriers.
// Every wait is bounded like the one-CTA kernel's; cluster barriers at the end keep either
// CTA from leaving while the other may still use its memory.
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Address of the same shared-memory object in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t peer_addr(const void* p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
__device__ __forceinline__ bool mbar_try_wait_cl(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait with cluster-scope acquire (barriers that receive arrivals from the peer).
__device__ bool mbar_wait_cl(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                             uint64_t timeout_ns = kTimeoutNs) {
  uint64_t t0 = 0;
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait_cl(bar, parity)) return true;
    if ((it & 255u) == 255u) {
      if (*abort_flag) return false;
      const uint64_t now = globaltimer();
      if (t0 == 0) t0 = now;
      else if (now - t0 > timeout_ns) return false;
    }
  }
}
__device__ __forceinline__ void umma_pair(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}
// Arrive on the mbarrier at shared::cluster address `bar` (this CTA's or the peer's) once
// every MMA issued so far has completed.
__device__ __forceinline__ void umma_commit_pair(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// TMA tile load into this CTA's shared memory whose completion is counted on the mbarrier
// at shared::cluster address `bar`, which may be the peer CTA's (.cta_group::2).
__device__ __forceinline__ void tma_load_3d_pair(uint32_t dst, const CUtensorMap* tm, uint32_t bar, int x, int y,
                                                 int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.cta_group::2 "
      "[%0], [%1, {%3, %4, %5}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(bar), "r"(x), "r"(y), "r"(z)
      : "memory");
}

template <int P> struct CfgPair {
  static constexpr int ROWS = 128;                 // rows of A and of B' staged per CTA
  static constexpr int A_PLANE = ROWS * BKE2 * 2;  // 8 KB
  static constexpr int B_PLANE = ROWS * BKE2 * 2;  // 8 KB
  static constexpr int STAGE_BYTES = P * (A_PLANE + B_PLANE);
  static constexpr int ST = (228352 - 2048) / STAGE_BYTES;
  static constexpr int STAGES = ST > 8 ? 8 : ST;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024;
  static constexpr int TILE_N = 256;               // real columns of the pair's tile
  static constexpr uint32_t ACC_COLS = 256;
  static constexpr uint32_t TMEM_COLS = 512;
  static_assert(STAGES >= 2, "the operand ring needs two stages");
};

template <int P>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(128, 1)
    tc_gemm_pair_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                        float2* __restrict__ C, int64_t M, int64_t N, int nkb, ProdList prods,
                        int* __restrict__ errflag, PlaneScales sc, int tiles_n) {
  using CF = CfgPair<P>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  __shared__ __align__(8) uint64_t full_bar[CF::STAGES];
  __shared__ __align__(8) uint64_t empty_bar[CF::STAGES];
  __shared__ __align__(8) uint64_t accum_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  __shared__ int n_issued, n_consumed, peer_issued;

  const uint32_t rank = cluster_ctarank();
  const bool leader = rank == 0;
  const uint32_t peer = rank ^ 1u;
  const int pair = (int)(blockIdx.x >> 1);
  const int tm = pair / tiles_n, tn = pair % tiles_n;  // N tile fastest
  const int m0 = tm * 256 + (int)rank * CF::ROWS;     // this CTA's rows of A and of C
  const int n0 = tn * CF::TILE_N;                      // the pair's first real column
  const int rb = n0 + (int)rank * CF::ROWS;            // this CTA's rows of B'

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < CF::STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&accum_bar, 1);
    abort_flag = 0;
    n_issued = 0;
    n_consumed = 0;
    peer_issued = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
  }
  if (warp == 2) {  // one warp of each CTA allocates the pair's columns together
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(CF::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  // inverse fp16 scales of the pair's complex columns (every CTA writes all TILE_N columns)
  __shared__ float s_binv[CF::TILE_N / 2];
  if (sc.bmax)
    for (int t = threadIdx.x; t < CF::TILE_N / 2; t += blockDim.x) {
      const int64_t n = (int64_t)(n0 >> 1) + t;
      s_binv[t] = n < N ? fp16_row_scale_inv(sc.bmax[n]) : 1.0f;
    }
  fence_before();
  __syncthreads();
  cluster_sync();  // both CTAs' barriers exist before either side signals the other's
  fence_after();
  const uint32_t tmem_d = tmem_slot;

  if (warp == 0 && lane == 0) {
    const uint32_t leader_full0 = peer_addr(&full_bar[0], 0u);
    int it = 0;
    for (; it < nkb; ++it) {
      const int s = it % CF::STAGES;
      const uint32_t ph = (uint32_t)(it / CF::STAGES) & 1u;
      if (!mbar_wait_cl(&empty_bar[s], ph ^ 1u, &abort_flag)) {
        abort_flag = 1;
        atomicCAS(errflag, 0, DEVERR_TMA_TIMEOUT);
        break;
      }
      const uint32_t sa = smem_u32(smem + s * CF::STAGE_BYTES);
      const uint32_t sb = sa + P * CF::A_PLANE;
      const uint32_t fb = leader_full0 + (uint32_t)(s * sizeof(uint64_t));
      if (leader) mbar_expect_tx(&full_bar[s], 2 * CF::STAGE_BYTES);  // both halves
#pragma unroll
      for (int p = 0; p < P; ++p) {
        tma_load_3d_pair(sa + p * CF::A_PLANE, &tmA, fb, it * BKE2, m0, p);
        tma_load_3d_pair(sb + p * CF::B_PLANE, &tmB, fb, it * BKE2, rb, p);
      }
    }
    n_issued = it;
    if (!leader) {  // tell the leader how many stages this CTA issued (its drain covers them)
      const uint32_t dst = peer_addr(&peer_issued, 0u);
      asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(dst), "r"(it) : "memory");
    }
  } else if (warp == 1 && lane == 0 && leader) {
    const uint32_t idesc = sc.fp16 ? idesc_f16(256, CF::TILE_N) : idesc_bf16(256, CF::TILE_N);
    const uint32_t peer_empty0 = peer_addr(&empty_bar[0], peer);
    bool lead_started = false, corr_started = false;
    int it = 0;
    for (; it < nkb; ++it) {
      const int s = it % CF::STAGES;
      const uint32_t ph = (uint32_t)(it / CF::STAGES) & 1u;
      if (!mbar_wait_cl(&full_bar[s], ph, &abort_flag)) {
        abort_flag = 1;
        atomicCAS(errflag, 0, DEVERR_MMA_TIMEOUT);
        break;
      }
      fence_after();
      const uint32_t sa = smem_u32(smem + s * CF::STAGE_BYTES);
      const uint32_t sb = sa + P * CF::A_PLANE;
      for (int q = 0; q < prods.n; ++q) {
        const uint32_t a0 = sa + prods.a[q] * CF::A_PLANE;
        const uint32_t b0 = sb + prods.b[q] * CF::B_PLANE;
        const bool lead = prods.a[q] == 0 && prods.b[q] == 0;
        const uint32_t d = lead ? tmem_d : tmem_d + CF::ACC_COLS;
#pragma unroll
        for (int kk = 0; kk < BKE2 / 16; ++kk) {
          umma_pair(d, sdesc64(a0 + kk * 32), sdesc64(b0 + kk * 32), idesc,
                    (lead ? lead_started : corr_started) ? 1u : 0u);
          if (lead) lead_started = true; else corr_started = true;
        }
      }
      umma_commit_pair(smem_u32(&empty_bar[s]));
      umma_commit_pair(peer_empty0 + (uint32_t)(s * sizeof(uint64_t)));
    }
    n_consumed = it;
    umma_commit_pair(smem_u32(&accum_bar));
    umma_commit_pair(peer_addr(&accum_bar, peer));
  }
  __syncwarp();

  const bool ok = mbar_wait_cl(&accum_bar, 0u, &abort_flag);
  if (!ok && lane == 0) {
    abort_flag = 1;
    atomicCAS(errflag, 0, DEVERR_EPI_TIMEOUT);
  }
  __syncwarp();
  fence_after();
  if (ok) {
    const int row = warp * 32 + lane;
    const int64_t m = (int64_t)m0 + row;
    const uint32_t taddr = tmem_d + ((uint32_t)(warp * 32) << 16);
    bool has_corr = false;
    for (int q = 0; q < prods.n; ++q) has_corr |= !(prods.a[q] == 0 && prods.b[q] == 0);
    const float ainv = (sc.amax && m < M) ? fp16_row_scale_inv(sc.amax[m]) : 1.0f;
#pragma unroll 1
    for (int c = 0; c < CF::TILE_N; c += 16) {
      uint32_t v[16], w[16];
      tmem_ld16(taddr + (uint32_t)c, v);
      if (has_corr) {
        tmem_ld16(taddr + CF::ACC_COLS + (uint32_t)c, w);
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) w[j] = 0u;
      }
      if (m < M) {
        const int64_t nb = (int64_t)(n0 + c) >> 1;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int64_t n = nb + j;
          if (n < N) {
            const float f = sc.bmax ? ainv * s_binv[(c >> 1) + j] : ainv;
            C[n * M + m] = make_float2((__uint_as_float(v[2 * j]) + __uint_as_float(w[2 * j])) * f,
                                       (__uint_as_float(v[2 * j + 1]) + __uint_as_float(w[2 * j + 1])) * f);
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  cluster_sync();  // the odd CTA's issue count has reached the leader
  // drain: copies of either CTA that no MMA waited for (abort path only) land on the
  // leader's full barriers before anyone leaves
  if (leader && threadIdx.x == 0) {
    const int issued = n_issued > peer_issued ? n_issued : peer_issued;
    for (int it = n_consumed; it < issued; ++it) {
      volatile int no_abort = 0;
      mbar_wait_cl(&full_bar[it % CF::STAGES], (uint32_t)(it / CF::STAGES) & 1u, &no_abort, 50000000ull);
    }
  }
  __syncthreads();
  cluster_sync();  // neither CTA frees TMEM or leaves while the other may still use its memory
  if (warp == 2) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(CF::TMEM_COLS)
                 : "memory");
  }
}

template <int BN>
__global__ void __launch_bounds__(128, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   float2* __restrict__ C, int64_t M, int64_t N, int nkb, ProdList prods,
                   int* __restrict__ errflag, int tiles_n) {
  tc_tile<BN>(&tmA, &tmB, C, M, N, nkb, prods, (int)(blockIdx.x / tiles_n) * BM, (int)(blockIdx.x % tiles_n) * BN,
              errflag);
}

// Many independent problems in one launch: CTA b works on tile b - tile_start[p] of the
// problem p whose tile range holds b (problems listed largest K first).
struct GroupedTc {
  CUtensorMap tmA[kTcGroupMax];
  CUtensorMap tmB[kTcGroupMax];
  float2* C[kTcGroupMax];
  int64_t M[kTcGroupMax];
  int64_t N[kTcGroupMax];
  int nkb[kTcGroupMax];
  int tiles_n[kTcGroupMax];
  int tile_start[kTcGroupMax + 1];
  const float* amax[kTcGroupMax];
  const float* bmax[kTcGroupMax];
  int nprob;
  int fp16;
  ProdList prods;
};

template <int BN, int P>
__global__ void __launch_bounds__(kPsThreads, 1) tc_gemm_grouped_ps_kernel(const __grid_constant__ GroupedTc g,
                                                                    int* __restrict__ errflag) {
  constexpr int CPS = 1;
  const int b = blockIdx.x;
  int p = 0;
  while (p + 1 < g.nprob && g.tile_start[p + 1] <= b) ++p;
  const int t = b - g.tile_start[p];
  const int tn = t % g.tiles_n[p], tm = t / g.tiles_n[p];  // N tile fastest
  const PlaneScales sc{g.amax[p], g.bmax[p], g.fp16};
  tc_tile_ps<BN, P, CPS>(&g.tmA[p], &g.tmB[p], g.C[p], g.M[p], g.N[p], g.nkb[p], g.prods, tm * BM, tn * BN, errflag,
                         sc);
}

// ---- persistent grouped kernel -----------------------------------------------------------
// One launch of at most one CTA per SM runs every tile of every problem of the group (the
// coupled-charge GEMMs of a block-sparse step, or one dense problem): CTA c takes tiles c,
// c + grid, ...  Six warps with fixed roles:
//   warp 0 (one lane) : TMA producer over the CTA's (tile, k-block) sequence, one ring of
//                       stages shared by all its tiles (no pipeline drain between tiles)
//   warp 1 (one lane) : MMA issuer; warp 1 also allocates and frees TMEM
//   warps 2-9         : epilogue; warp w reads TMEM lanes 32 (w % 4) .. + 31 and one half of
//                       the tile's columns (two warps per lane quarter keep twice the
//                       TMEM loads and stores in flight)
// With 128-wide (or narrower) tiles TMEM holds two accumulator sets (lead + corrections
// each), so the epilogue of tile i runs while the MMAs of tile i + 1 proceed; 256-wide tiles
// fill TMEM with one set.  Accumulator hand-off: full barriers (one MMA commit) and empty
// barriers (one arrival per epilogue warp).  Every wait is bounded as in tc_tile_ps.
template <int BN, int P> struct CfgPersist {
  using Base = Cfg2<BN, P, 1>;
  static constexpr int STAGE_BYTES = Base::STAGE_BYTES;
  static constexpr int STAGES = Base::STAGES;
  static constexpr int SMEM = Base::SMEM;
  static constexpr uint32_t ACC_COLS = Base::ACC_COLS;
  static constexpr int NACC = (4 * ACC_COLS <= 512) ? 2 : 1;  // accumulator sets
  static constexpr uint32_t TMEM_COLS = (uint32_t)NACC * 2 * ACC_COLS;
};

__device__ __forceinline__ int find_problem(const GroupedTc& g, int t) {
  int p = 0;
  while (p + 1 < g.nprob && g.tile_start[p + 1] <= t) ++p;
  return p;
}

constexpr int kPersistEpiWarps = 8;
constexpr int kPersistThreads = 32 * (2 + kPersistEpiWarps);

template <int BN, int P>
__global__ void __launch_bounds__(kPersistThreads, 1) tc_gemm_persist_kernel(const __grid_constant__ GroupedTc g,
                                                                             int* __restrict__ errflag) {
  using CF = CfgPersist<BN, P>;
  using B2 = Cfg2<BN, P, 1>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  __shared__ __align__(8) uint64_t full_bar[CF::STAGES];
  __shared__ __align__(8) uint64_t empty_bar[CF::STAGES];
  __shared__ __align__(8) uint64_t accf_bar[2];
  __shared__ __align__(8) uint64_t acce_bar[2];
  __shared__ float s_binv[kPersistEpiWarps][BN / 4 > 0 ? BN / 4 : 1];
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  __shared__ int n_issued, n_consumed;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int total = g.tile_start[g.nprob];
  if (threadIdx.x == 0) {
    for (int s = 0; s < CF::STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf_bar[b], 1);
      mbar_init(&acce_bar[b], kPersistEpiWarps);
    }
    abort_flag = 0;
    n_issued = 0;
    n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(CF::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem_base = tmem_slot;

  if (warp == 0 && lane == 0) {
    int gk = 0;
    bool stop = false;
    for (int t = blockIdx.x; t < total && !stop; t += gridDim.x) {
      const int p = find_problem(g, t);
      const int tl = t - g.tile_start[p];
      const int m0 = (tl / g.tiles_n[p]) * BM, r0 = (tl % g.tiles_n[p]) * BN;
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&g.tmA[p])) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&g.tmB[p])) : "memory");
      for (int kb = 0; kb < g.nkb[p]; ++kb, ++gk) {
        const int s = gk % CF::STAGES;
        const uint32_t ph = (uint32_t)(gk / CF::STAGES) & 1u;
        if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_flag)) {
          abort_flag = 1;
          atomicCAS(errflag, 0, DEVERR_TMA_TIMEOUT);
          stop = true;
          break;
        }
        const uint32_t sa = smem_u32(smem + s * CF::STAGE_BYTES);
        const uint32_t sb = sa + P * B2::A_PLANE;
        mbar_expect_tx(&full_bar[s], CF::STAGE_BYTES);
#pragma unroll
        for (int pl = 0; pl < P; ++pl) {
          tma_load_3d(sa + pl * B2::A_PLANE, &g.tmA[p], &full_bar[s], kb * BKE2, m0, pl);
          tma_load_3d(sb + pl * B2::B_PLANE, &g.tmB[p], &full_bar[s], kb * BKE2, r0, pl);
        }
      }
    }
    n_issued = gk;
  } else if (warp == 1 && lane == 0) {
    const uint32_t idesc = g.fp16 ? idesc_f16(BM, BN) : idesc_bf16(BM, BN);
    int gk = 0, i = 0;
    bool stop = false;
    for (int t = blockIdx.x; t < total && !stop; t += gridDim.x, ++i) {
      const int p = find_problem(g, t);
      const int b = i % CF::NACC;
      const uint32_t use = (uint32_t)(i / CF::NACC);
      if (!mbar_wait(&acce_bar[b], (use & 1u) ^ 1u, &abort_flag)) {  // the epilogue freed set b
        abort_flag = 1;
        atomicCAS(errflag, 0, DEVERR_MMA_TIMEOUT);
        break;
      }
      fence_after();
      const uint32_t dlead = tmem_base + (uint32_t)b * 2u * CF::ACC_COLS, dcorr = dlead + CF::ACC_COLS;
      bool lead_started = false, corr_started = false;
      for (int kb = 0; kb < g.nkb[p]; ++kb, ++gk) {
        const int s = gk % CF::STAGES;
        const uint32_t ph = (uint32_t)(gk / CF::STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, &abort_flag)) {
          abort_flag = 1;
          atomicCAS(errflag, 0, DEVERR_MMA_TIMEOUT);
          stop = true;
          break;
        }
        fence_after();
        const uint32_t sa = smem_u32(smem + s * CF::STAGE_BYTES);
        const uint32_t sb = sa + P * B2::A_PLANE;
        for (int q = 0; q < g.prods.n; ++q) {
          const uint32_t a0 = sa + g.prods.a[q] * B2::A_PLANE;
          const uint32_t b0 = sb + g.prods.b[q] * B2::B_PLANE;
          const bool lead = g.prods.a[q] == 0 && g.prods.b[q] == 0;
#pragma unroll
          for (int kk = 0; kk < BKE2 / 16; ++kk) {
            umma_bf16(lead ? dlead : dcorr, sdesc64(a0 + kk * 32), sdesc64(b0 + kk * 32), idesc,
                      (lead ? lead_started : corr_started) ? 1u : 0u);
            if (lead) lead_started = true; else corr_started = true;
          }
        }
        umma_commit(&empty_bar[s]);
      }
      umma_commit(&accf_bar[b]);  // set b complete once every MMA issued so far has
    }
    n_consumed = gk;
  } else if (warp >= 2) {
    const int q4 = warp & 3;                // TMEM lane quarter of this warp
    const int c0 = ((warp - 2) >> 2) * (BN / 2);  // its half of the tile's columns
    int i = 0;
    bool has_corr = false;
    for (int q = 0; q < g.prods.n; ++q) has_corr |= !(g.prods.a[q] == 0 && g.prods.b[q] == 0);
    for (int t = blockIdx.x; t < total; t += gridDim.x, ++i) {
      const int p = find_problem(g, t);
      const int tl = t - g.tile_start[p];
      const int m0 = (tl / g.tiles_n[p]) * BM, r0 = (tl % g.tiles_n[p]) * BN;
      const int b = i % CF::NACC;
      const uint32_t use = (uint32_t)(i / CF::NACC);
      const bool ok = mbar_wait(&accf_bar[b], use & 1u, &abort_flag);
      if (!ok) {
        if (lane == 0) {
          abort_flag = 1;
          atomicCAS(errflag, 0, DEVERR_EPI_TIMEOUT);
        }
        break;
      }
      __syncwarp();
      fence_after();
      const int64_t M = g.M[p], N = g.N[p];
      float2* __restrict__ C = g.C[p];
      const int row = q4 * 32 + lane;
      const int64_t m = (int64_t)m0 + row;
      const uint32_t taddr = tmem_base + (uint32_t)b * 2u * CF::ACC_COLS + ((uint32_t)(q4 * 32) << 16);
      const float ainv = (g.amax[p] && m < M) ? fp16_row_scale_inv(g.amax[p][m]) : 1.0f;
      const float* bmx = g.bmax[p];
      // this warp's copy of its columns' inverse scales (read once per tile)
      float* binv = s_binv[warp - 2];
      if (bmx) {
        for (int t = lane; t < BN / 4; t += 32) {
          const int64_t n = (int64_t)((r0 + c0) >> 1) + t;
          binv[t] = n < N ? fp16_row_scale_inv(bmx[n]) : 1.0f;
        }
        __syncwarp();
      }
#pragma unroll 1
      for (int c = c0; c < c0 + BN / 2; c += 16) {
        uint32_t v[16], w[16];
        tmem_ld16(taddr + (uint32_t)c, v);
        if (has_corr) {
          tmem_ld16(taddr + CF::ACC_COLS + (uint32_t)c, w);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) w[j] = 0u;
        }
        if (m < M) {
          const int64_t nb = (int64_t)(r0 + c) >> 1;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int64_t n = nb + j;
            if (n < N) {
              const float f = bmx ? ainv * binv[((c - c0) >> 1) + j] : ainv;
              C[n * M + m] = make_float2((__uint_as_float(v[2 * j]) + __uint_as_float(w[2 * j])) * f,
                                         (__uint_as_float(v[2 * j + 1]) + __uint_as_float(w[2 * j + 1])) * f);
            }
          }
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive_local(&acce_bar[b]);
    }
  }
  fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {  // copies issued but never consumed (abort path only) land before exit
    for (int it = n_consumed; it < n_issued; ++it) {
      volatile int no_abort = 0;
      mbar_wait(&full_bar[it % CF::STAGES], (uint32_t)(it / CF::STAGES) & 1u, &no_abort);
    }
  }
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(CF::TMEM_COLS)
                 : "memory");
  }
}

template <int BN>
__global__ void __launch_bounds__(128, 1) tc_gemm_grouped_kernel(const __grid_constant__ GroupedTc g,
                                                                 int* __restrict__ errflag) {
  const int b = blockIdx.x;
  int p = 0;
  while (p + 1 < g.nprob && g.tile_start[p + 1] <= b) ++p;
  const int t = b - g.tile_start[p];
  const int tn = t % g.tiles_n[p], tm = t / g.tiles_n[p];  // N tile fastest
  tc_tile<BN>(&g.tmA[p], &g.tmB[p], g.C[p], g.M[p], g.N[p], g.nkb[p], g.prods, tm * BM, tn * BN, errflag);
}

// 3-D map over bf16 planes: (2Kp elements, rows, planes), box (64, box_rows, 1).
bool make_map(CUtensorMap* tm, const void* base, int64_t Kp, int64_t rows, int planes, int box_rows,
              std::string* why, int box_k = BKE) {
  EncodeTiledFn enc = get_encode();
  if (!enc) {
    if (why) *why = "cuTensorMapEncodeTiled unavailable";
    return false;
  }
  cuuint64_t gdim[3] = {(cuuint64_t)(2 * Kp), (cuuint64_t)rows, (cuuint64_t)planes};
  cuuint64_t gstr[2] = {(cuuint64_t)(2 * Kp * 2), (cuuint64_t)(rows * 2 * Kp * 2)};
  cuuint32_t box[3] = {(cuuint32_t)box_k, (cuuint32_t)box_rows, 1u};
  cuuint32_t estr[3] = {1u, 1u, 1u};
  CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), gdim, gstr, box,
                   estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   box_k == BKE ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    if (why) *why = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
    return false;
  }
  return true;
}

// Kernel variant: 1 = all slice planes per stage (SWIZZLE_64B), 0 = one product per stage
// (SWIZZLE_128B).  GTN_TC_VARIANT overrides the default.
int tc_variant() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("GTN_TC_VARIANT");
    v = (e && e[0] == '0') ? 0 : 1;
  }
  return v;
}

template <int BN, int P, int CPS = 1>
cudaError_t launch_ps(const TcGemmArgs& a, int* errflag, cudaStream_t s, std::string* why) {
  using CF = Cfg2<BN, P, CPS>;
  CUtensorMap tmA, tmB;
  if (!make_map(&tmA, a.A, a.Kp, a.M, a.a_planes, BM, why, BKE2)) return cudaErrorInvalidValue;
  if (!make_map(&tmB, a.B, a.Kp, 2 * a.N, a.b_planes, BN, why, BKE2)) return cudaErrorInvalidValue;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_ps_kernel<BN, P, CPS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         CF::SMEM);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  ProdList pl;
  pl.n = a.nprod;
  for (int i = 0; i < 9; ++i) {
    pl.a[i] = i < a.nprod ? a.prod_a[i] : 0;
    pl.b[i] = i < a.nprod ? a.prod_b[i] : 0;
  }
  const int nkb = (int)((2 * a.Kp + BKE2 - 1) / BKE2);
  const int64_t gx = (a.M + BM - 1) / BM;
  const int64_t gy = (2 * a.N + BN - 1) / BN;
  if (gx * gy > 2147483647LL) return cudaErrorInvalidConfiguration;
  const PlaneScales sc{a.a_max, a.b_max, a.fp16};
  tc_gemm_ps_kernel<BN, P, CPS><<<(unsigned)(gx * gy), kPsThreads, CF::SMEM, s>>>(tmA, tmB, a.C, a.M, a.N, nkb, pl, errflag, sc,
                                                                     (int)gy);
  return cudaGetLastError();
}

int device_sm_count() {
  static int sms[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (sms[dev] == 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 148;
    sms[dev] = v;
  }
  return sms[dev];
}

// Grouped problems, at most kTcGroupMax per launch.  Persist: one persistent launch of
// min(tiles, SM count) CTAs of 320 threads (tc_gemm_persist_kernel); otherwise one CTA per
// tile (tc_gemm_grouped_ps_kernel).
template <int BN, int P, bool Persist>
cudaError_t launch_grouped_ps(const TcGemmArgs* probs, int nprob, int* errflag, cudaStream_t s, std::string* why) {
  using CF = Cfg2<BN, P>;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = Persist ? cudaFuncSetAttribute(tc_gemm_persist_kernel<BN, P>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, CF::SMEM)
                            : cudaFuncSetAttribute(tc_gemm_grouped_ps_kernel<BN, P>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, CF::SMEM);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  for (int base = 0; base < nprob; base += kTcGroupMax) {
    const int cnt = std::min(kTcGroupMax, nprob - base);
    GroupedTc g;
    std::memset(&g, 0, sizeof(g));
    int tiles = 0;
    for (int q = 0; q < cnt; ++q) {
      const TcGemmArgs& a = probs[base + q];
      if (!make_map(&g.tmA[q], a.A, a.Kp, a.M, a.a_planes, BM, why, BKE2)) return cudaErrorInvalidValue;
      if (!make_map(&g.tmB[q], a.B, a.Kp, 2 * a.N, a.b_planes, BN, why, BKE2)) return cudaErrorInvalidValue;
      g.C[q] = a.C;
      g.M[q] = a.M;
      g.N[q] = a.N;
      g.amax[q] = a.a_max;
      g.bmax[q] = a.b_max;
      g.nkb[q] = (int)((2 * a.Kp + BKE2 - 1) / BKE2);
      g.tiles_n[q] = (int)((2 * a.N + BN - 1) / BN);
      g.tile_start[q] = tiles;
      tiles += (int)((a.M + BM - 1) / BM) * g.tiles_n[q];
    }
    g.tile_start[cnt] = tiles;
    g.nprob = cnt;
    g.fp16 = probs[base].fp16;
    g.prods.n = probs[base].nprod;
    for (int i = 0; i < 9; ++i) {
      g.prods.a[i] = i < probs[base].nprod ? probs[base].prod_a[i] : 0;
      g.prods.b[i] = i < probs[base].nprod ? probs[base].prod_b[i] : 0;
    }
    if (tiles == 0) continue;
    if (Persist)
      tc_gemm_persist_kernel<BN, P><<<std::min(tiles, device_sm_count()), kPersistThreads, CF::SMEM, s>>>(g, errflag);
    else
      tc_gemm_grouped_ps_kernel<BN, P><<<tiles, kPsThreads, CF::SMEM, s>>>(g, errflag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <int P>
cudaError_t launch_pair(const TcGemmArgs& a, int* errflag, cudaStream_t s, std::string* why) {
  using CF = CfgPair<P>;
  CUtensorMap tmA, tmB;
  if (!make_map(&tmA, a.A, a.Kp, a.M, a.a_planes, CF::ROWS, why, BKE2)) return cudaErrorInvalidValue;
  if (!make_map(&tmB, a.B, a.Kp, 2 * a.N, a.b_planes, CF::ROWS, why, BKE2)) return cudaErrorInvalidValue;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_pair_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         CF::SMEM);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  ProdList pl;
  pl.n = a.nprod;
  for (int i = 0; i < 9; ++i) {
    pl.a[i] = i < a.nprod ? a.prod_a[i] : 0;
    pl.b[i] = i < a.nprod ? a.prod_b[i] : 0;
  }
  const int nkb = (int)((2 * a.Kp + BKE2 - 1) / BKE2);
  const int64_t pairs_m = (a.M + 255) / 256;
  const int64_t tiles_n = (2 * a.N + CF::TILE_N - 1) / CF::TILE_N;
  if (2 * pairs_m * tiles_n > 2147483647LL) return cudaErrorInvalidConfiguration;
  const PlaneScales sc{a.a_max, a.b_max, a.fp16};
  tc_gemm_pair_kernel<P><<<(unsigned)(2 * pairs_m * tiles_n), 128, CF::SMEM, s>>>(tmA, tmB, a.C, a.M, a.N, nkb, pl,
                                                                                  errflag, sc, (int)tiles_n);
  return cudaGetLastError();
}

// Long-K steps with wide N tiles run on SM pairs (GTN_TC_PAIR=0 keeps them on one SM).
bool tc_use_pair() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("GTN_TC_PAIR");
    v = (e && e[0] == '0') ? 0 : 1;
  }
  return v == 1;
}

// Short-K steps (at most 16 k-blocks of 32) run 128-wide tiles two CTAs per SM.
int tc_short_k_blocks() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("GTN_TC_SHORTK");
    v = e ? atoi(e) : 16;
  }
  return v;
}

// ---- tile shape selection: fixed ladder or measured choice --------------------------
// Variants of the slice-plane kernel (all compute the same products in the same order per
// output element, so they agree bitwise):
enum TcVariant : int {
  TCV_PS32 = 0,     // one CTA per 128 x 32 tile
  TCV_PS64 = 1,     // 128 x 64
  TCV_PS128 = 2,    // 128 x 128
  TCV_PS128X2 = 3,  // 128 x 128, two CTAs per SM (one's epilogue overlaps the other's mainloop)
  TCV_PS256 = 4,    // 128 x 256, one CTA per SM
  TCV_PAIR256 = 5,  // 256 x 256 on an SM pair (cta_group::2)
  TCV_PERSIST128 = 6,  // 128 x 128, persistent (one CTA per SM, epilogue overlapping the next tile)
  TCV_PERSIST256 = 7,  // 128 x 256, persistent (one accumulator set; the operand ring runs on
                       // across tiles, so the next tile's copies land during the epilogue)
  TCV_COUNT = 8
};
const char* const kTcVariantNames[TCV_COUNT] = {"ps32",   "ps64",    "ps128",      "ps128x2",
                                                "ps256",  "pair256", "persist128", "persist256"};

template <int P>
cudaError_t launch_variant(int v, const TcGemmArgs& a, int* errflag, cudaStream_t s, std::string* why) {
  switch (v) {
    case TCV_PS32: return launch_ps<32, P>(a, errflag, s, why);
    case TCV_PS64: return launch_ps<64, P>(a, errflag, s, why);
    case TCV_PS128: return launch_ps<128, P>(a, errflag, s, why);
    case TCV_PS128X2: return launch_ps<128, P, 2>(a, errflag, s, why);
    case TCV_PS256: return launch_ps<256, P>(a, errflag, s, why);
    case TCV_PERSIST128: return launch_grouped_ps<128, P, true>(&a, 1, errflag, s, why);
    case TCV_PERSIST256: return launch_grouped_ps<256, P, true>(&a, 1, errflag, s, why);
    default: return launch_pair<P>(a, errflag, s, why);
  }
}

// The fixed ladder: short-K steps (at most 16 k-blocks of 32) two CTAs per SM, wide
// long-K steps on SM pairs, otherwise the narrowest tile that covers 2N.
int ladder_variant(int64_t n2, int nkb) {
  if (n2 > 64 && nkb <= tc_short_k_blocks()) return TCV_PS128X2;
  if (n2 > 128) return tc_use_pair() ? TCV_PAIR256 : TCV_PS256;
  if (n2 <= 32) return TCV_PS32;
  if (n2 <= 64) return TCV_PS64;
  return TCV_PS128;
}

// Candidates the tuner times for a problem: every variant whose tile is not wider than
// needed by more than one step of the ladder.
int tc_candidates(int64_t n2, int* out) {
  int n = 0;
  if (n2 <= 32) out[n++] = TCV_PS32;
  else if (n2 <= 64) out[n++] = TCV_PS64;
  else if (n2 <= 128) { out[n++] = TCV_PS128; out[n++] = TCV_PS128X2; out[n++] = TCV_PERSIST128; }
  else {
    out[n++] = TCV_PS256;
    out[n++] = TCV_PAIR256;
    out[n++] = TCV_PS128X2;
    out[n++] = TCV_PERSIST128;
    out[n++] = TCV_PERSIST256;
  }
  return n;
}

int ilog2_ceil(int64_t x) {
  int r = 0;
  while ((int64_t(1) << r) < x && r < 62) ++r;
  return r;
}

// Problem class of the tuner's cache: plane count, fp16 planes, product count, ceil(log2 M),
// 2N in steps of 64, ceil(log2 k-blocks).
struct TuneKey {
  int P, fp16, nprod, lm, n64, lk;
  bool operator<(const TuneKey& o) const {
    return std::tie(P, fp16, nprod, lm, n64, lk) < std::tie(o.P, o.fp16, o.nprod, o.lm, o.n64, o.lk);
  }
};
struct TuneRec {
  int chosen = -1;
  float ms[TCV_COUNT];
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneRec> g_tune;
std::atomic<int> g_tune_mode{1};  // 0 ladder, 1 measured (default), 2 + v: variant v forced

template <int P>
cudaError_t launch_ps_tuned(const TcGemmArgs& a, int64_t n2, int* errflag, cudaStream_t s, std::string* why) {
  const int nkb = (int)((2 * a.Kp + BKE2 - 1) / BKE2);
  const int mode = g_tune_mode.load();
  int cand[TCV_COUNT];
  const int nc = tc_candidates(n2, cand);
  if (mode >= 2) {  // a forced variant, where it is a candidate for this problem
    for (int i = 0; i < nc; ++i)
      if (cand[i] == mode - 2) return launch_variant<P>(mode - 2, a, errflag, s, why);
    return launch_variant<P>(ladder_variant(n2, nkb), a, errflag, s, why);
  }
  if (mode == 0 || nc == 1) return launch_variant<P>(ladder_variant(n2, nkb), a, errflag, s, why);
  const TuneKey key{P, a.fp16, a.nprod, ilog2_ceil(a.M), (int)((n2 + 63) / 64), ilog2_ceil(nkb)};
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return launch_variant<P>(it->second.chosen, a, errflag, s, why);
  }
  // Not measured yet.  Under stream capture nothing can be timed: take the ladder's choice
  // without caching it.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return launch_variant<P>(ladder_variant(n2, nkb), a, errflag, s, why);
  // Time every candidate on this problem (one warm-up launch, then two timed launches on
  // the caller's stream); the output is rewritten by each, and the final launch below
  // leaves the chosen variant's result.
  TuneRec rec;
  for (int v = 0; v < TCV_COUNT; ++v) rec.ms[v] = -1.0f;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return cudaGetLastError();
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return cudaGetLastError();
  }
  float best = 0.0f;
  int bestv = ladder_variant(n2, nkb);
  cudaError_t err = cudaSuccess;
  for (int i = 0; i < nc && err == cudaSuccess; ++i) {
    err = launch_variant<P>(cand[i], a, errflag, s, why);
    if (err != cudaSuccess) break;
    cudaEventRecord(e0, s);
    for (int r = 0; r < 2 && err == cudaSuccess; ++r) err = launch_variant<P>(cand[i], a, errflag, s, why);
    cudaEventRecord(e1, s);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    rec.ms[cand[i]] = ms / 2.0f;
    if (err == cudaSuccess && (i == 0 || ms / 2.0f < best)) {
      best = ms / 2.0f;
      bestv = cand[i];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return err;
  rec.chosen = bestv;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune.emplace(key, rec);  // a concurrent tuner of the same class may have won: keep the first
  }
  return launch_variant<P>(bestv, a, errflag, s, why);
}

// Grouped launches (block-sparse steps, batched maps): the persistent kernel with the tile
// width chosen like the dense steps' (measured per problem list unless the tuner is in
// ladder or forced mode): the ladder's width for the widest problem, and half of it.
template <int P>
cudaError_t launch_grouped_persist_bn(int bn, const TcGemmArgs* probs, int nprob, int* errflag, cudaStream_t s,
                              std::string* why) {
  switch (bn) {
    case 32: return launch_grouped_ps<32, P, true>(probs, nprob, errflag, s, why);
    case 64: return launch_grouped_ps<64, P, true>(probs, nprob, errflag, s, why);
    case 128: return launch_grouped_ps<128, P, true>(probs, nprob, errflag, s, why);
    default: return launch_grouped_ps<256, P, true>(probs, nprob, errflag, s, why);
  }
}

struct GroupKey {
  uint64_t h;
  bool operator<(const GroupKey& o) const { return h < o.h; }
};
std::map<GroupKey, int> g_group_tune;

template <int P>
cudaError_t launch_grouped_ps_bn(const TcGemmArgs* probs, int nprob, int64_t n2, int* errflag, cudaStream_t s,
                                 std::string* why) {
  const int ladder = n2 <= 32 ? 32 : n2 <= 64 ? 64 : n2 <= 128 ? 128 : 256;
  const int mode = g_tune_mode.load();
  if (mode != 1 || ladder == 32) return launch_grouped_persist_bn<P>(ladder, probs, nprob, errflag, s, why);
  // FNV-1a over the problem list's shapes and the plane format
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](int64_t v) {
    for (int b = 0; b < 8; ++b) {
      h ^= (uint64_t)((v >> (8 * b)) & 0xff);
      h *= 1099511628211ull;
    }
  };
  mix(P);
  mix(probs[0].fp16);
  mix(probs[0].nprod);
  for (int q = 0; q < nprob; ++q) {
    mix(probs[q].M);
    mix(probs[q].N);
    mix(probs[q].Kp);
  }
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_group_tune.find(GroupKey{h});
    if (it != g_group_tune.end()) return launch_grouped_persist_bn<P>(it->second, probs, nprob, errflag, s, why);
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return launch_grouped_persist_bn<P>(ladder, probs, nprob, errflag, s, why);
  const int cand[2] = {ladder, ladder / 2};
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return cudaGetLastError();
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return cudaGetLastError();
  }
  float best = 0.0f;
  int bestbn = ladder;
  cudaError_t err = cudaSuccess;
  for (int i = 0; i < 2 && err == cudaSuccess; ++i) {
    err = launch_grouped_persist_bn<P>(cand[i], probs, nprob, errflag, s, why);
    if (err != cudaSuccess) break;
    cudaEventRecord(e0, s);
    for (int r = 0; r < 2 && err == cudaSuccess; ++r) err = launch_grouped_persist_bn<P>(cand[i], probs, nprob, errflag, s, why);
    cudaEventRecord(e1, s);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (err == cudaSuccess && (i == 0 || ms < best)) {
      best = ms;
      bestbn = cand[i];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return err;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_group_tune.emplace(GroupKey{h}, bestbn);
  }
  return launch_grouped_persist_bn<P>(bestbn, probs, nprob, errflag, s, why);
}

template <int BN>
cudaError_t launch_bn(const TcGemmArgs& a, int* errflag, cudaStream_t s, std::string* why) {
  using CF = Cfg<BN>;
  CUtensorMap tmA, tmB;
  if (!make_map(&tmA, a.A, a.Kp, a.M, a.a_planes, BM, why)) return cudaErrorInvalidValue;
  if (!make_map(&tmB, a.B, a.Kp, 2 * a.N, a.b_planes, BN, why)) return cudaErrorInvalidValue;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         CF::SMEM);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  ProdList pl;
  pl.n = a.nprod;
  for (int i = 0; i < 9; ++i) {
    pl.a[i] = i < a.nprod ? a.prod_a[i] : 0;
    pl.b[i] = i < a.nprod ? a.prod_b[i] : 0;
  }
  const int nkb = (int)((2 * a.Kp + BKE - 1) / BKE);
  const int64_t gx = (a.M + BM - 1) / BM;
  const int64_t gy = (2 * a.N + BN - 1) / BN;
  if (gx * gy > 2147483647LL) return cudaErrorInvalidConfiguration;
  tc_gemm_kernel<BN><<<(unsigned)(gx * gy), 128, CF::SMEM, s>>>(tmA, tmB, a.C, a.M, a.N, nkb, pl, errflag, (int)gy);
  return cudaGetLastError();
}

template <int BN>
cudaError_t launch_grouped_bn(const TcGemmArgs* probs, int nprob, int* errflag, cudaStream_t s, std::string* why) {
  using CF = Cfg<BN>;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_grouped_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         CF::SMEM);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  for (int base = 0; base < nprob; base += kTcGroupMax) {
    const int cnt = std::min(kTcGroupMax, nprob - base);
    GroupedTc g;
    std::memset(&g, 0, sizeof(g));
    int tiles = 0;
    for (int q = 0; q < cnt; ++q) {
      const TcGemmArgs& a = probs[base + q];
      if (!make_map(&g.tmA[q], a.A, a.Kp, a.M, a.a_planes, BM, why)) return cudaErrorInvalidValue;
      if (!make_map(&g.tmB[q], a.B, a.Kp, 2 * a.N, a.b_planes, BN, why)) return cudaErrorInvalidValue;
      g.C[q] = a.C;
      g.M[q] = a.M;
      g.N[q] = a.N;
      g.nkb[q] = (int)((2 * a.Kp + BKE - 1) / BKE);
      g.tiles_n[q] = (int)((2 * a.N + BN - 1) / BN);
      g.tile_start[q] = tiles;
      tiles += (int)((a.M + BM - 1) / BM) * g.tiles_n[q];
    }
    g.tile_start[cnt] = tiles;
    g.nprob = cnt;
    g.prods.n = probs[base].nprod;
    for (int i = 0; i < 9; ++i) {
      g.prods.a[i] = i < probs[base].nprod ? probs[base].prod_a[i] : 0;
      g.prods.b[i] = i < probs[base].nprod ? probs[base].prod_b[i] : 0;
    }
    if (tiles == 0) continue;
    tc_gemm_grouped_kernel<BN><<<tiles, 128, CF::SMEM, s>>>(g, errflag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_tc_gemm_grouped(const TcGemmArgs* probs, int nprob, int* errflag, cudaStream_t s,
                                   std::string* why) {
  int64_t maxn2 = 0;
  for (int q = 0; q < nprob; ++q) {
    const TcGemmArgs& a = probs[q];
    if (a.Kp % 32 != 0 || a.nprod != probs[0].nprod || a.M <= 0 || a.N <= 0) {
      if (why) *why = "tc_gemm_grouped: Kp multiple of 32, same product list, non-empty problems";
      return cudaErrorInvalidValue;
    }
    if (reinterpret_cast<uintptr_t>(a.A) % 16 || reinterpret_cast<uintptr_t>(a.B) % 16) {
      if (why) *why = "tc_gemm_grouped: operand planes must be 16-byte aligned";
      return cudaErrorInvalidValue;
    }
    maxn2 = std::max(maxn2, 2 * a.N);
  }
  if (nprob == 0) return cudaSuccess;
  const int P = probs[0].a_planes;
  bool planes_ok = P == 2 || P == 3;
  for (int q = 0; q < nprob; ++q) planes_ok = planes_ok && probs[q].a_planes == P && probs[q].b_planes == P;
  for (int q = 0; q < nprob; ++q)
    if (probs[q].fp16 != probs[0].fp16 || (probs[q].fp16 && !planes_ok)) {
      if (why) *why = "tc_gemm_grouped: fp16 planes need one format and 2 or 3 planes per problem";
      return cudaErrorInvalidValue;
    }
  if ((tc_variant() == 1 || probs[0].fp16) && planes_ok)
    return P == 3 ? launch_grouped_ps_bn<3>(probs, nprob, maxn2, errflag, s, why)
                  : launch_grouped_ps_bn<2>(probs, nprob, maxn2, errflag, s, why);
  if (maxn2 <= 32) return launch_grouped_bn<32>(probs, nprob, errflag, s, why);
  if (maxn2 <= 64) return launch_grouped_bn<64>(probs, nprob, errflag, s, why);
  if (maxn2 <= 128) return launch_grouped_bn<128>(probs, nprob, errflag, s, why);
  return launch_grouped_bn<256>(probs, nprob, errflag, s, why);
}

bool tc_gemm_supported(int cc_major, int cc_minor) {
  (void)cc_minor;
  return cc_major == 10 && get_encode() != nullptr;
}

cudaError_t launch_tc_gemm(const TcGemmArgs& a, int* errflag, cudaStream_t s, std::string* why) {
  if (a.M <= 0 || a.N <= 0) return cudaSuccess;
  if (a.Kp % 32 != 0 || a.nprod < 1 || a.nprod > 9) {
    if (why) *why = "tc_gemm: Kp must be a multiple of 32 and 1..9 products";
    return cudaErrorInvalidValue;
  }
  if (reinterpret_cast<uintptr_t>(a.A) % 16 || reinterpret_cast<uintptr_t>(a.B) % 16) {
    if (why) *why = "tc_gemm: operand planes must be 16-byte aligned";
    return cudaErrorInvalidValue;
  }
  const int64_t n2 = 2 * a.N;
  const bool planes_ok = a.a_planes == a.b_planes && (a.a_planes == 2 || a.a_planes == 3);
  if (a.fp16 && !planes_ok) {
    if (why) *why = "tc_gemm: fp16 planes need 2 or 3 planes";
    return cudaErrorInvalidValue;
  }
  if ((tc_variant() == 1 || a.fp16) && planes_ok)
    return a.a_planes == 3 ? launch_ps_tuned<3>(a, n2, errflag, s, why) : launch_ps_tuned<2>(a, n2, errflag, s, why);
  if (n2 <= 32) return launch_bn<32>(a, errflag, s, why);
  if (n2 <= 64) return launch_bn<64>(a, errflag, s, why);
  if (n2 <= 128) return launch_bn<128>(a, errflag, s, why);
  return launch_bn<256>(a, errflag, s, why);
}

cudaError_t launch_wait_selftest(int* errflag, uint64_t timeout_ns, cudaStream_t s) {
  wait_selftest_kernel<<<1, 1, 0, s>>>(errflag, timeout_ns);
  return cudaGetLastError();
}

// Measured tile-shape selection of the dense tcgen05 steps (see launch_ps_tuned).
extern "C" int gtn_tc_tuning(int mode, int clear) {
  if (mode < -1 || mode >= 2 + TCV_COUNT) return -1;
  const int old = g_tune_mode.load();
  if (mode >= 0) g_tune_mode.store(mode);
  if (clear) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune.clear();
    g_group_tune.clear();
  }
  return old;
}

extern "C" int gtn_tc_tune_report(char* buf, int64_t cap, int64_t* needed) {
  std::string out;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    char line[512];
    for (const auto& kv : g_tune) {
      const TuneKey& k = kv.first;
      int n = snprintf(line, sizeof(line), "planes=%d fp16=%d products=%d log2M=%d n2_64=%d log2kb=%d chosen=%s", k.P,
                       k.fp16, k.nprod, k.lm, k.n64, k.lk, kTcVariantNames[kv.second.chosen]);
      for (int v = 0; v < TCV_COUNT && n > 0 && n < (int)sizeof(line); ++v)
        if (kv.second.ms[v] >= 0.0f)
          n += snprintf(line + n, sizeof(line) - n, " %s=%.4fms", kTcVariantNames[v], kv.second.ms[v]);
      out += line;
      out += '\n';
    }
  }
  if (needed) *needed = (int64_t)out.size() + 1;
  if (!buf || cap <= 0) return GTN_OK;
  const size_t n = std::min<size_t>(out.size(), (size_t)cap - 1);
  memcpy(buf, out.data(), n);
  buf[n] = '\0';
  return n == out.size() ? GTN_OK : GTN_ERR_INVALID;
}
