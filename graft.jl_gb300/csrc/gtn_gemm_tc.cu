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
//   warp 0 lane 0 : TMA producer (cp.async.bulk.tensor.3d, SWIZZLE_128B, no multicast)
//   warp 1 lane 0 : tcgen05.mma issuer (kind::f16, bf16 x bf16 -> f32)
//   warp 2        : TMEM allocator
//   warps 0-3     : epilogue (tcgen05.ld 32x32b -> complex FP32 stores, m-fastest)
// Every mbarrier wait is bounded (globaltimer, 4 s); on timeout the CTA records an error
// code in the context's device flag, drains its own copies and MMAs, frees TMEM, returns.
#include "gtn_internal.h"
#include <cuda.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>

namespace {

constexpr int BM = 128;
constexpr int BKE = 64;  // bf16 elements per k-block = 128 bytes = one SW128 row
constexpr int A_BYTES = BM * BKE * 2;
constexpr uint64_t kTimeoutNs = 4000000000ull;

constexpr int kTcGroupMax = 56;

struct ProdList {
  int n;
  int a[9];
  int b[9];
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait on a phase parity.  Returns false on timeout or when another role of the
// CTA has already aborted.
__device__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                          uint64_t timeout_ns = kTimeoutNs) {
  uint64_t t0 = 0;
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u) {
      if (*abort_flag) return false;
      const uint64_t now = globaltimer();
      if (t0 == 0) t0 = now;
      else if (now - t0 > timeout_ns) return false;
    }
  }
}

// A wait that runs out: an mbarrier expecting one arrival that never comes.
__global__ void wait_selftest_kernel(int* __restrict__ errflag, uint64_t timeout_ns) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ volatile int no_abort;
  mbar_init(&bar, 1);
  no_abort = 0;
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  if (!mbar_wait(&bar, 0u, &no_abort, timeout_ns)) atomicCAS(errflag, 0, DEVERR_SELFTEST_TIMEOUT);
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* tm, uint64_t* bar, int x,
                                            int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4, %5}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

// The same load delivered to the shared memory (and mbarrier) at the same offset in every
// CTA of the cluster named by cta_mask (TMA multicast within this GPU's memory).
__device__ __forceinline__ void tma_load_3d_mc(uint32_t dst, const CUtensorMap* tm, uint64_t* bar, int x, int y,
                                               int z, uint16_t cta_mask) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.multicast::cluster "
      "[%0], [%1, {%3, %4, %5}], [%2], %6;" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z), "h"(cta_mask)
      : "memory");
}
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major, SWIZZLE_128B, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024u >> 4) << 32;  // stride byte offset
  d |= (uint64_t)1u << 46;            // descriptor version
  d |= (uint64_t)2u << 61;            // SWIZZLE_128B
  return d;
}

// Shared-memory matrix descriptor: K-major, SWIZZLE_64B, 8-row groups 512 B apart.
__device__ __forceinline__ uint64_t sdesc64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512u >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1u << 46;            // descriptor version
  d |= (uint64_t)4u << 61;            // SWIZZLE_64B
  return d;
}

// Instruction descriptor, kind::f16: D=f32, A=B=bf16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
// The same with A=B=f16 (format code 0 in both operand fields).
__host__ __device__ constexpr uint32_t idesc_f16(int m, int n) {
  return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}
// Arrive on the mbarrier at the same offset in every CTA of cta_mask when the MMAs issued
// so far complete.
__device__ __forceinline__ void umma_commit_mc(uint64_t* bar, uint16_t cta_mask) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"(cta_mask)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
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

// MC: the CTA is one of a cluster pair with the same N tile and adjacent M tiles; each
// CTA loads half of the B' tile and multicasts it to both, and both MMA threads release a
// stage to both producers (empty barriers count two arrivals).
template <int BN, int P, int CPS, bool MC = false>
__device__ __forceinline__ void tc_tile_ps(const CUtensorMap* tmA, const CUtensorMap* tmB, float2* __restrict__ C,
                                           int64_t M, int64_t N, int nkb, const ProdList& prods, int m0, int r0,
                                           int* __restrict__ errflag, const PlaneScales& sc) {
  using CF = Cfg2<BN, P, CPS>;
  const uint32_t crank = MC ? cluster_ctarank() : 0u;
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
      mbar_init(&empty_bar[s], MC ? 2 : 1);
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
  // the peer's multicast loads and commits target this CTA's barriers: both CTAs finish
  // initialising them before either producer starts
  if (MC) cluster_sync_all();
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
        if (MC)
          tma_load_3d_mc(sb + p * CF::B_PLANE + crank * (CF::B_PLANE / 2), tmB, &full_bar[s], it * BKE2,
                         r0 + (int)crank * (BN / 2), p, (uint16_t)3);
        else
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
      if (MC)
        umma_commit_mc(&empty_bar[s], (uint16_t)3);
      else
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
    const int row = warp * 32 + lane;
    const int64_t m = (int64_t)m0 + row;
    const uint32_t taddr = tmem_d + ((uint32_t)(warp * 32) << 16);
    bool has_corr = false;
    for (int q = 0; q < prods.n; ++q) has_corr |= !(prods.a[q] == 0 && prods.b[q] == 0);
    const float ainv = (sc.amax && m < M) ? 1.0f / fp16_row_scale(sc.amax[m]) : 1.0f;
#pragma unroll 1
    for (int c = 0; c < BN; c += 16) {
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
            const float f = sc.bmax ? ainv / fp16_row_scale(sc.bmax[n]) : ainv;
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
  // neither CTA of a pair leaves while the other may still deliver into its shared memory
  if (MC) cluster_sync_all();
  if (warp == 2) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d),
                 "r"(CF::TMEM_COLS)
                 : "memory");
  }
}

// Cluster pairs: CTAs 2p and 2p+1 share N tile p % tiles_n and take M tiles 2 (p / tiles_n)
// and 2 (p / tiles_n) + 1 (the second may lie past M: its loads read the fill value and its
// epilogue stores nothing).
template <int BN, int P>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(128, 1)
    tc_gemm_mc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      float2* __restrict__ C, int64_t M, int64_t N, int nkb, ProdList prods,
                      int* __restrict__ errflag, PlaneScales sc, int tiles_n) {
  const int pair = (int)(blockIdx.x >> 1);
  const int tm = 2 * (pair / tiles_n) + (int)cluster_ctarank();
  tc_tile_ps<BN, P, 1, true>(&tmA, &tmB, C, M, N, nkb, prods, tm * BM, (pair % tiles_n) * BN, errflag, sc);
}

template <int BN, int P, int CPS>
__global__ void __launch_bounds__(128, CPS)
    tc_gemm_ps_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      float2* __restrict__ C, int64_t M, int64_t N, int nkb, ProdList prods,
                      int* __restrict__ errflag, PlaneScales sc, int tiles_n) {
  // N tile fastest: the CTAs that run together share their A tiles through L2
  tc_tile_ps<BN, P, CPS>(&tmA, &tmB, C, M, N, nkb, prods, (int)(blockIdx.x / tiles_n) * BM, (int)(blockIdx.x % tiles_n) * BN,
                    errflag, sc);
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
__global__ void __launch_bounds__(128, 1) tc_gemm_grouped_ps_kernel(const __grid_constant__ GroupedTc g,
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

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn get_encode() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
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
  tc_gemm_ps_kernel<BN, P, CPS><<<(unsigned)(gx * gy), 128, CF::SMEM, s>>>(tmA, tmB, a.C, a.M, a.N, nkb, pl, errflag, sc,
                                                                     (int)gy);
  return cudaGetLastError();
}

template <int BN, int P>
cudaError_t launch_grouped_ps(const TcGemmArgs* probs, int nprob, int* errflag, cudaStream_t s, std::string* why) {
  using CF = Cfg2<BN, P>;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_grouped_ps_kernel<BN, P>,
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
    tc_gemm_grouped_ps_kernel<BN, P><<<tiles, 128, CF::SMEM, s>>>(g, errflag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <int BN, int P>
cudaError_t launch_mc(const TcGemmArgs& a, int* errflag, cudaStream_t s, std::string* why) {
  using CF = Cfg2<BN, P, 1>;
  CUtensorMap tmA, tmB;
  if (!make_map(&tmA, a.A, a.Kp, a.M, a.a_planes, BM, why, BKE2)) return cudaErrorInvalidValue;
  if (!make_map(&tmB, a.B, a.Kp, 2 * a.N, a.b_planes, BN / 2, why, BKE2)) return cudaErrorInvalidValue;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_mc_kernel<BN, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
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
  const int64_t pairs_m = ((a.M + BM - 1) / BM + 1) / 2;
  const int64_t gy = (2 * a.N + BN - 1) / BN;
  if (2 * pairs_m * gy > 2147483647LL) return cudaErrorInvalidConfiguration;
  const PlaneScales sc{a.a_max, a.b_max, a.fp16};
  tc_gemm_mc_kernel<BN, P><<<(unsigned)(2 * pairs_m * gy), 128, CF::SMEM, s>>>(tmA, tmB, a.C, a.M, a.N, nkb, pl,
                                                                               errflag, sc, (int)gy);
  return cudaGetLastError();
}

// Cluster-pair B multicast for long-K steps with 256-wide tiles (GTN_TC_MC=1 selects it).
bool tc_use_mc() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("GTN_TC_MC");
    v = (e && e[0] == '1') ? 1 : 0;
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

template <int P>
cudaError_t launch_ps_bn(const TcGemmArgs& a, int64_t n2, int* errflag, cudaStream_t s, std::string* why) {
  const int nkb = (int)((2 * a.Kp + BKE2 - 1) / BKE2);
  if (n2 > 64 && nkb <= tc_short_k_blocks()) return launch_ps<128, P, 2>(a, errflag, s, why);
  if (n2 > 128 && tc_use_mc()) return launch_mc<256, P>(a, errflag, s, why);
  if (n2 <= 32) return launch_ps<32, P>(a, errflag, s, why);
  if (n2 <= 64) return launch_ps<64, P>(a, errflag, s, why);
  if (n2 <= 128) return launch_ps<128, P>(a, errflag, s, why);
  return launch_ps<256, P>(a, errflag, s, why);
}

template <int P>
cudaError_t launch_grouped_ps_bn(const TcGemmArgs* probs, int nprob, int64_t n2, int* errflag, cudaStream_t s,
                                 std::string* why) {
  if (n2 <= 32) return launch_grouped_ps<32, P>(probs, nprob, errflag, s, why);
  if (n2 <= 64) return launch_grouped_ps<64, P>(probs, nprob, errflag, s, why);
  if (n2 <= 128) return launch_grouped_ps<128, P>(probs, nprob, errflag, s, why);
  return launch_grouped_ps<256, P>(probs, nprob, errflag, s, why);
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
    return a.a_planes == 3 ? launch_ps_bn<3>(a, n2, errflag, s, why) : launch_ps_bn<2>(a, n2, errflag, s, why);
  if (n2 <= 32) return launch_bn<32>(a, errflag, s, why);
  if (n2 <= 64) return launch_bn<64>(a, errflag, s, why);
  if (n2 <= 128) return launch_bn<128>(a, errflag, s, why);
  return launch_bn<256>(a, errflag, s, why);
}

cudaError_t launch_wait_selftest(int* errflag, uint64_t timeout_ns, cudaStream_t s) {
  wait_selftest_kernel<<<1, 1, 0, s>>>(errflag, timeout_ns);
  return cudaGetLastError();
}
