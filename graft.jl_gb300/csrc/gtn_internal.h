// Internal declarations shared by the libgrafttn translation units.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <map>
#include <memory>
#include <mutex>

#include "../../include/grafttn.h"

#define GTN_MAXG 12   // index groups per gather (a two-site tensor of a 4-ary tree has 10 legs)
#define GTN_BLOCK_MAXG 8  // index groups of a gtn_block_gather (the ABI struct's arrays)

// A multi-index group: index i in [0, prod(dim)) decomposes into digits (outer..inner)
// whose strides (in elements) give the offset into a row-major tensor.
struct GroupSpec {
  int n;
  int64_t dim[GTN_MAXG];
  int64_t str[GTN_MAXG];
};

// Device error codes written to the context's error flag by bounded waits.
enum : int { DEVERR_NONE = 0, DEVERR_TMA_TIMEOUT = 1, DEVERR_MMA_TIMEOUT = 2, DEVERR_EPI_TIMEOUT = 3,
             DEVERR_SELFTEST_TIMEOUT = 4 };
cudaError_t launch_wait_selftest(int* errflag, uint64_t timeout_ns, cudaStream_t s);

struct gtn_ctx_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;          // last failure message (any thread), guarded by err_mu
  std::mutex err_mu;
  int64_t launches = 0;
  int* d_errflag = nullptr;
  int sm_count = 0;
  int cc_major = 0, cc_minor = 0;
  // reduction scratch (device + pinned host)
  double2* d_red = nullptr;
  size_t red_cap = 0;
  double2* h_red = nullptr;
  size_t hred_cap = 0;
  // transient workspace for one-shot contractions / factorisations
  void* ws = nullptr;
  size_t ws_bytes = 0;
  // bump arena of one-shot contractions (stream-ordered reuse, grown to the largest need)
  char* carena = nullptr;
  size_t carena_cap = 0, carena_need = 0;
  void* cusolver = nullptr;
  // precision of the GEMMs inside the factorisations (Gram SVD route): GTN_PREC_FP64 or
  // GTN_PREC_FP64E (gtn_ctx_set_linalg_precision)
  int linalg_prec = 0;
  // freed map workspace blocks by size, reused in stream order by later maps on this
  // context (maps are built and dropped at every node visit of a sweep; cudaMalloc and the
  // device-synchronising cudaFree made a small map's creation cost about a millisecond)
  std::multimap<size_t, void*> blk_free;
  size_t blk_cached = 0;
};

// ---- status helpers -------------------------------------------------------------
int set_err(gtn_ctx ctx, int code, const std::string& msg);
#define GTN_CUDA_TRY(ctx, expr)                                                       \
  do {                                                                                \
    cudaError_t e__ = (expr);                                                         \
    if (e__ != cudaSuccess)                                                           \
      return set_err((ctx), GTN_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e__)); \
  } while (0)

cudaError_t ctx_workspace(gtn_ctx ctx, size_t bytes, void** out);
// Map workspace blocks through the context's cache: *got is the block's size, to be handed
// back with the block; release returns it to the cache (or frees it past the cache's bound),
// flush frees every cached block.
cudaError_t ctx_blk_alloc(gtn_ctx ctx, size_t bytes, void** out, size_t* got);
void ctx_blk_release(gtn_ctx ctx, void* p, size_t bytes);
void ctx_blk_flush(gtn_ctx ctx);
// Thin QR of a tall-skinny row-major matrix by shifted Cholesky QR with two refinement
// passes (gtn_tsqr.cu); GTN_ERR_UNSUPPORTED when it does not apply or the matrix is too
// ill-conditioned for it (the Householder QR then runs).
bool tsqr_applies(int64_t m, int64_t n);
// Householder QR of a small matrix (m n and m min(m, n) <= 4096) in one CTA, no host sync.
bool small_qr_applies(int64_t m, int64_t n);
// One-sided Jacobi SVD of a small matrix (min(m, n) <= 64, m n <= 4096) in one CTA:
// S (k, descending), U (m x k row-major), Vh (k x n row-major), k = min(m, n), on the device.
bool small_svd_applies(int64_t m, int64_t n);
int svd_small_launch(gtn_ctx ctx, int64_t m, int64_t n, const double2* A, double* S, double2* U, double2* Vh);
int qr_small(gtn_ctx ctx, int64_t m, int64_t n, const double2* A, double2* Q, double2* R);
int qr_tall_cholesky(gtn_ctx ctx, int64_t m, int64_t n, const double2* A, double2* Q, double2* R);
cudaError_t ctx_red(gtn_ctx ctx, size_t n2);   // ensure d_red/h_red hold n2 double2
void linalg_release(gtn_ctx ctx);               // drop the cuSOLVER handle (gtn_linalg.cu)

// ---- layout kernels (gtn_layout.cu) ----------------------------------------------
// out[m, k] = T[offM(m) + offK(k)] for m < M, k < Kw (zero where k >= K).
cudaError_t launch_gather_c128_to_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg,
                                       int64_t M, int64_t K, int64_t ldo, double2* out, cudaStream_t s);
cudaError_t launch_gather_c128_to_c64(const double2* T, const GroupSpec& mg, const GroupSpec& kg,
                                      int64_t M, int64_t K, int64_t ldo, float2* out, cudaStream_t s);
cudaError_t launch_gather_c64_to_c64(const float2* T, const GroupSpec& mg, const GroupSpec& kg,
                                     int64_t M, int64_t K, int64_t ldo, float2* out, cudaStream_t s);
cudaError_t launch_gather_c64_to_c128(const float2* T, const GroupSpec& mg, const GroupSpec& kg,
                                      int64_t M, int64_t K, int64_t ldo, double2* out, cudaStream_t s);
// Split into bf16 planes: plane p at out + p*pstride, row m at m*ld2, complex k at 2k.
// Columns K <= k < Kp are written as zero (TMA reads the padded extent).
cudaError_t launch_split_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M,
                              int64_t K, int64_t Kp, int nplanes, int64_t pstride,
                              __nv_bfloat16* out, cudaStream_t s);
cudaError_t launch_split_c64(const float2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M,
                             int64_t K, int64_t Kp, int nplanes, int64_t pstride,
                             __nv_bfloat16* out, cudaStream_t s);
// Expanded real operand of a static B [N][K] (complex, row-major) for the tcgen05 path:
// rows (n, c_out), columns (k, c_in): [[Br, -Bi], [Bi, Br]], split into bf16 planes.
// Precomputed element offsets of a gather's rows and columns (device tables) and the
// lane mapping of its load phase.
struct GatherTab {
  const int64_t* om = nullptr;
  const int64_t* ok = nullptr;
  int m_fast = 0;
};
bool gather_m_fast(const GroupSpec& mg, const GroupSpec& kg);
cudaError_t launch_rowmax_tab(const void* T, int is64, const GatherTab& t, int64_t M, int64_t K, float* amax,
                              cudaStream_t s);
cudaError_t launch_split_tab(const void* T, int is64, const GatherTab& t, int64_t M, int64_t K, int64_t Kp,
                             int nplanes, int64_t pstride, __nv_bfloat16* out, cudaStream_t s);
cudaError_t launch_split16_tab(const void* T, int is64, const GatherTab& t, int64_t M, int64_t K, int64_t Kp,
                               int64_t pstride, const float* amax, __nv_bfloat16* out, cudaStream_t s);
// One pass: row maxima (written to amax) and the slice planes together, a cluster of CTAs
// per block of rows; *done = false when a row does not fit the clusters' shared memory.
cudaError_t launch_split16_rows_tab(const void* T, int is64, const GatherTab& t, int64_t M, int64_t K, int64_t Kp,
                                    int64_t pstride, float* amax, __nv_bfloat16* out, cudaStream_t s, bool* done);
cudaError_t launch_split16_rows_grp(const void* T, int is64, const GroupSpec& mg, const GroupSpec& kg, int64_t M,
                                    int64_t K, int64_t Kp, int64_t pstride, float* amax, __nv_bfloat16* out,
                                    cudaStream_t s, bool* done);
cudaError_t launch_split_i7_rows_tab(const double2* T, const GatherTab& t, int64_t M, int64_t K, int64_t Kp,
                                     int64_t pstride, float* amax, __nv_bfloat16* out, cudaStream_t s, bool* done);
cudaError_t launch_split_i7_rows_grp(const double2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                                     int64_t Kp, int64_t pstride, float* amax, __nv_bfloat16* out, cudaStream_t s,
                                     bool* done);
cudaError_t launch_gather_tab_to_c128(const void* T, int is64, const GatherTab& t, int64_t M, int64_t K, int64_t ldo,
                                      double2* out, cudaStream_t s);
// fp16 slice planes (2 planes, hi + lo) of a K-major gather, rows scaled by
// fp16_row_scale(amax[m]); launch_rowmax_* first fills amax[m] = max_k max(|re|, |im|).
cudaError_t launch_rowmax_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                               float* amax, cudaStream_t s);
cudaError_t launch_rowmax_c64(const float2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                              float* amax, cudaStream_t s);
cudaError_t launch_split16_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                                int64_t Kp, int64_t pstride, const float* amax, __nv_bfloat16* out, cudaStream_t s);
cudaError_t launch_split16_c64(const float2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                               int64_t Kp, int64_t pstride, const float* amax, __nv_bfloat16* out, cudaStream_t s);
// Static operand as fp16 planes of B' with per-complex-row maxima written to bmax[N].
cudaError_t launch_pack_b_planes_f16(const double2* B, int64_t N, int64_t K, int64_t Kp, int64_t pstride,
                                     __nv_bfloat16* out, float* bmax, cudaStream_t s);
cudaError_t launch_pack_b_planes(const double2* B, int64_t N, int64_t K, int64_t Kp, int nplanes,
                                 int64_t pstride, __nv_bfloat16* out, cudaStream_t s);

// Grouped variants: independent jobs in one launch (per 48 jobs).
constexpr int kGatherJobMax = 48;
struct GatherJob {
  const void* T;
  GroupSpec mg, kg;
  int64_t M, K, Kw;
  void* out;
  int64_t ld;        // complex output: row pitch
  int64_t pstride;   // split output: plane pitch (bf16 elements)
  int nplanes;       // 0: complex output, 2 or 3: bf16 slice planes (row pitch 2*Kw)
  const float* amax = nullptr;  // with nplanes == 2: fp16 planes scaled by these row maxima
};
struct SmallJob {
  const void* A;
  GroupSpec mg, kg;
  int64_t M;
  int K, N;
  const void* B;
  void* C;
};
cudaError_t launch_gather_grouped(const GatherJob* jobs, int njobs, int in_is64, int out_is64, cudaStream_t s);
// out[i] = offset of index i of the group (i < n), computed on the device.
cudaError_t launch_offsets_table(const GroupSpec& g, int64_t n, int64_t* out, cudaStream_t s);
// Row maxima of the jobs that carry amax (zeroed first), for their fp16 splits.
cudaError_t launch_rowmax_grouped(const GatherJob* jobs, int njobs, int in_is64, cudaStream_t s);
// Device-resident gather jobs (block-sparse maps): buffers resolved per launch.
struct BlockBases {
  void* buf[6];  // 0 x, 1 y, 2/3 running buffers, 4 staging, 5 fp16 row maxima
};
struct DevGatherJob {
  GroupSpec mg, kg;
  int64_t src_off, dst_off;
  int64_t M, K, Kw, ld, pstride;
  int src_buf, dst_buf;
  int nplanes;   // > 0: bf16 slice planes (row pitch 2*ld), else complex
  int dst_is64;  // complex output element type
  int tiles_m, m_fast;
  int mode;                      // 0 copy / bf16 split, 2 fp16 split (row maxima: launch_block_rowmax)
  int64_t amax_off;              // row maxima of this job's rows: (float*)bases.buf[5] + amax_off
  int tks;                       // log2 of the tile width in K (tile = (1024 >> tks) x (1 << tks))
  int fast_m;                    // M digits by 32-bit multiply-shift division (M < 2^31)
  uint32_t m_mag[GTN_MAXG];      // round-up multipliers of mg.dim (Granlund-Montgomery)
  uint32_t m_sh[GTN_MAXG];
};
void finish_dev_gather_job(DevGatherJob* J);
// tile_map[b] = (job, tile within the job) of CTA b: one load instead of a search.
cudaError_t launch_block_rowmax(const DevGatherJob* jobs, const int2* tile_map, int ntiles, const BlockBases& bases,
                                int src_is64, cudaStream_t s);
cudaError_t launch_block_gather(const DevGatherJob* jobs, const int2* tile_map, int ntiles, const BlockBases& bases,
                                int src_is64, cudaStream_t s);
// Fused gather + product for coupled-charge problems with few output columns (block maps):
// a band is the rows [row_off, row_off + M) of A_q, read straight from the running tensor,
// C_q[n][row_off + m] = sum_j A_q[row_off + m][bcol_j] * B_q[n][bcol_j] over the band's
// present columns j, with no staged copy of A_q.  Column j lives at
// src_j + sum_t digit_t(m) * rstr[rect_j][t]: the digits of m in the band's common row
// groups (the refinement of every rectangle's row groups) and the strides of column j's
// rectangle (source block) in those groups.
struct DevBandCol {
  int64_t src;   // element offset of the column in bases.buf[src_buf] (block offset + column offset)
  int32_t rect;  // its rectangle within the band
  int32_t bcol;  // its column of B_q
};
constexpr int kBandMaxRects = 24, kBandMaxGroups = 6;
struct DevBand {
  int64_t M;       // rows of the band
  int64_t row_off; // its first row in A_q
  int64_t c_off;   // product bands: element offset of C_q[0][row_off] in bases.buf[c_buf]
  int64_t ldc;     // product bands: M_q, the pitch between output columns n
  const void* B;   // product bands: B_q [N][Kq] in the compute type
  int64_t a_off;   // split bands: element offset (halves) of A_q's plane 0 in bases.buf[4]
  int64_t pstride; // split bands: plane pitch (halves)
  int64_t amax_off;  // split bands, fp16: row maxima of A_q at (float*)bases.buf[5] + amax_off
  int N, Kq, Kp, nplanes, c_buf, src_buf;
  int col0, ncol;  // present columns: cols[col0, col0 + ncol)
  int rs0, nrect;  // row strides: rstr[rs0 + rect * ng + t]
  int ng, m_fast;  // common row groups (slowest first); loads run along rows when m_fast
  uint32_t dim[kBandMaxGroups], mag[kBandMaxGroups], sh[kBandMaxGroups];  // group sizes, division magic
};
// A CTA's share of a band: the rows [m0, m0 + nrows).
struct DevBandWork {
  int band, nrows;
  int64_t m0;
};
bool block_band_fits(int64_t N, int64_t Kq, int fp64);
int block_band_rows_per_pass(int maxn);  // rows a CTA covers per pass (one thread per row)
size_t block_band_smem(int maxn, int Kq, int nrect, int ng, int fp64);
// Split bands: the slice planes of a tensor-core problem's A_q built band by band (rows of
// up to 1024 columns staged whole, row maxima reduced in the CTA for fp16), replacing the
// row-maxima pass, the block moves and the K padding of that problem.
constexpr int kSplitBandMaxKp = 1024;
int block_split_band_rows(int Kp, int src_is64);  // rows per pass
size_t block_split_band_smem(int Kp, int nrect, int ng, int ncol, int src_is64);
cudaError_t launch_block_split_band(const DevBand* bands, const DevBandWork* work, int nwork, const DevBandCol* cols,
                                    const int64_t* rstr, const BlockBases& bases, int src_is64, int fp16,
                                    size_t smem, cudaStream_t s);
cudaError_t launch_block_band(const DevBand* bands, const DevBandWork* work, int nwork, const DevBandCol* cols,
                              const int64_t* rstr, const BlockBases& bases, int src_is64, int fp64, int maxn,
                              size_t smem, cudaStream_t s);
cudaError_t launch_small_grouped(const SmallJob* jobs, int njobs, int is64, cudaStream_t s);

// C[n][m] = sum_k T[offM(m) + offK(k)] * B[n][k]   (small K; B in shared memory)
cudaError_t launch_small_contract_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg,
                                       int64_t M, int K, int N, const double2* B, double2* C,
                                       cudaStream_t s);
cudaError_t launch_small_contract_c64(const float2* T, const GroupSpec& mg, const GroupSpec& kg,
                                      int64_t M, int K, int N, const float2* B, float2* C,
                                      cudaStream_t s);
bool small_contract_fits(int K, int N, size_t elem_bytes);

// ---- SIMT GEMMs (gtn_gemm_simt.cu): C[n][m] = sum_k A[m][k] B[n][k] -----------------
cudaError_t launch_zgemm_simt(const double2* A, const double2* B, double2* C, int64_t M, int64_t N,
                              int64_t K, cudaStream_t s);
cudaError_t launch_cgemm_simt(const float2* A, const float2* B, float2* C, int64_t M, int64_t N,
                              int64_t K, cudaStream_t s);

constexpr int kGemmJobMax = 64;
struct GemmJob {
  const void* A;
  const void* B;
  void* C;
  int64_t M, N, K;
};
cudaError_t launch_gemm_simt_grouped(const GemmJob* jobs, int njobs, int is64, cudaStream_t s);
// Split-K for GEMMs with few output tiles and a long K: the number of K slices (1 = no
// split), and the launchers with a partial-sum workspace P of slices * M * N elements.
int gemm_splitk_slices(int64_t M, int64_t N, int64_t K);
cudaError_t launch_zgemm_simt_splitk(const double2* A, const double2* B, double2* C, int64_t M, int64_t N, int64_t K,
                                     int S, double2* P, cudaStream_t s);
cudaError_t launch_cgemm_simt_splitk(const float2* A, const float2* B, float2* C, int64_t M, int64_t N, int64_t K,
                                     int S, float2* P, cudaStream_t s);
// Skinny grouped GEMM (same contraction) for N <= 32; every job must pass gemm_skinny_fits.
constexpr int kSkinnyMaxSmem = 96 * 1024;
cudaError_t launch_gemm_skinny_grouped(const GemmJob* jobs, int njobs, int is64, cudaStream_t s);
bool gemm_skinny_fits(int64_t N, int64_t K, int is64);

// ---- tcgen05 GEMM (gtn_gemm_tc.cu) ---------------------------------------------------
// Real GEMM on bf16 slice planes: C (complex fp32, [N][M]) from A planes [P][M][2Kp] and
// B planes [P][2N][2Kp].  prods lists (a_plane, b_plane) pairs accumulated in order.
struct TcGemmArgs {
  const __nv_bfloat16* A;  // planes, pitch 2Kp elements per row
  const __nv_bfloat16* B;
  float2* C;
  int64_t M, N, Kp;        // complex dims; Kp = padded K (multiple of 32)
  int a_planes, b_planes;  // number of planes stored (for the tensor-map extents)
  int nprod;
  int prod_a[9], prod_b[9];
  // fp16 slice planes (the planes hold IEEE half bits): row m of A was scaled by
  // fp16_row_scale(a_max[m]) and complex row n of B by fp16_row_scale(b_max[n]); the
  // epilogue divides both out.  Null maxima and fp16 = 0 for bf16 planes.
  int fp16 = 0;
  const float* a_max = nullptr;
  const float* b_max = nullptr;
};

// Power-of-two scale taking a row maximum mx into [2^14, 2^15) (fp16 holds up to 65504):
// 2^(14 - floor(log2 mx)); 1 for a zero or subnormal maximum.
__host__ __device__ inline float fp16_row_scale(float mx) {
  uint32_t b;
  memcpy(&b, &mx, 4);
  const int e = (int)((b >> 23) & 0xffu);
  if (e == 0) return 1.0f;
  int te = 268 - e;  // biased exponent of 2^(14 - (e - 127))
  te = te < 1 ? 1 : (te > 254 ? 254 : te);
  const uint32_t o = (uint32_t)te << 23;
  float r;
  memcpy(&r, &o, 4);
  return r;
}
// 1 / fp16_row_scale(mx) exactly (a power of two, 2^-127 at the smallest), without a division.
__host__ __device__ inline float fp16_row_scale_inv(float mx) {
  uint32_t b;
  memcpy(&b, &mx, 4);
  const int e = (int)((b >> 23) & 0xffu);
  if (e == 0) return 1.0f;
  int te = 268 - e;
  te = te < 1 ? 1 : (te > 254 ? 254 : te);
  const int ie = 254 - te;  // biased exponent of 2^(127 - te)
  const uint32_t o = ie > 0 ? (uint32_t)ie << 23 : 0x00400000u;
  float r;
  memcpy(&r, &o, 4);
  return r;
}
cudaError_t launch_tc_gemm(const TcGemmArgs& a, int* errflag, cudaStream_t s, std::string* why);

// ---- FP64-grade GEMM on the tensor cores (gtn_gemm_f64e.cu) ------------------------------
// C (complex FP64, [N][M]) = A B^T from integer digit planes: A [S][M][2Kp] (rows scaled by
// 2^k(a_max[m])), B' [S][2N][2Kp] (complex rows scaled by 2^k(b_max[n])), S = kF64eSlices.
constexpr int kF64eSlices = 7;
struct F64eGemmArgs {
  const __nv_bfloat16* A = nullptr;
  const __nv_bfloat16* B = nullptr;
  double2* C = nullptr;
  int64_t M = 0, N = 0, Kp = 0;
  const float* a_max = nullptr;
  const float* b_max = nullptr;
};
cudaError_t launch_f64e_gemm(const F64eGemmArgs& a, int* errflag, cudaStream_t s, std::string* why);
// digit planes of the running tensor's K-major view (c128), rows scaled by amax (from
// launch_rowmax_*), and of a static B [N][K] (bmax written here)
cudaError_t launch_split_i7_tab(const double2* T, const GatherTab& t, int64_t M, int64_t K, int64_t Kp,
                               int64_t pstride, const float* amax, __nv_bfloat16* out, cudaStream_t s);
cudaError_t launch_split_i7_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                                 int64_t Kp, int64_t pstride, const float* amax, __nv_bfloat16* out, cudaStream_t s);
cudaError_t launch_pack_b_planes_i7(const double2* B, int64_t N, int64_t K, int64_t Kp, int64_t pstride,
                                    __nv_bfloat16* out, float* bmax, cudaStream_t s);
bool tc_gemm_supported(int cc_major, int cc_minor);
// Independent problems in one launch per 56 problems (same product list for all).
cudaError_t launch_tc_gemm_grouped(const TcGemmArgs* probs, int nprob, int* errflag, cudaStream_t s,
                                   std::string* why);

// ---- vector kernels (gtn_blas.cu) --------------------------------------------------
// scratch holds nblk * J partials; with scratch_cap > 0 (its capacity in entries) the grid
// may widen up to 4 * nblk CTAs where that helps.
cudaError_t launch_multidot(const double2* V, int64_t ldv, int J, const double2* w, int64_t n,
                            double2* out /*[J]*/, double2* scratch, int nblk, cudaStream_t s,
                            int64_t scratch_cap = 0);
cudaError_t launch_lincomb(double2* w, double2 beta, const double2* V, int64_t ldv, int J,
                           const double2* coef /*device [J]*/, double2 cscale, int64_t n,
                           cudaStream_t s);
cudaError_t launch_axpby(int64_t n, double2 a, const double2* x, double2 b, double2* y,
                         cudaStream_t s);
int multidot_launch_count(int J);  // kernels one launch_multidot[_f32] of J vectors issues
// FP32-product variants for reorthogonalisation passes of mixed-precision bases.
cudaError_t launch_multidot_f32(const double2* V, int64_t ldv, int J, const double2* w, int64_t n,
                                double2* out /*[J]*/, double2* scratch, int nblk, cudaStream_t s,
                                int64_t scratch_cap = 0);
cudaError_t launch_reorth_update_f32(double2* w, const double2* V, int64_t ldv, int J,
                                     const double2* coef /*device [J]*/, int64_t n, cudaStream_t s);
// In place: V_j <- sum_{i<m} Q[i * k + j] V_i for j < k (k <= m <= 64, Q real, device).
cudaError_t launch_basis_rotate(double2* V, int64_t ldv, int m, int k, const double* Q, int64_t n,
                                cudaStream_t s);
cudaError_t launch_c64_to_c128(const float2* x, double2* y, int64_t n, cudaStream_t s);
cudaError_t launch_fill_c128(double2* x, double2 v, int64_t n, cudaStream_t s);
// x[i] = (u, v), u and v uniform in [-1, 1), a fixed function of (seed, i).
cudaError_t launch_fill_uniform_c128(double2* x, int64_t n, uint64_t seed, cudaStream_t s);
cudaError_t launch_conj_inplace(double2* x, int64_t n, cudaStream_t s);
// out[a][j][b] = in[a][idx[j]][b] for j < nsel (idx: device int64, entries < Lin)
cudaError_t launch_restrict_leg(const double2* in, double2* out, int64_t A, int64_t Lin, int64_t nsel, int64_t B,
                                const int64_t* idx, cudaStream_t s);
cudaError_t launch_transpose_c128(const double2* in, int64_t rows, int64_t cols, double2* out,
                                  cudaStream_t s);  // out[c][r] = in[r][c]
cudaError_t launch_zero_lower(double2* R, int64_t rows, int64_t cols, cudaStream_t s);
cudaError_t launch_row_norms(const double2* A, int64_t rows, int64_t cols, double* out, cudaStream_t s);
cudaError_t launch_row_phase_conj(double2* A, int64_t rows, int64_t cols, const double2* ph, cudaStream_t s);
cudaError_t launch_diag_scale(double2* A, int64_t rows, int64_t cols, const double* d, int side,
                              cudaStream_t s);
int multidot_blocks(gtn_ctx ctx);

// ---- plans (gtn_plan.cpp) ----------------------------------------------------------
struct PlanStep {
  int operand;             // static operand absorbed
  bool small;              // strided SIMT path (no permute)
  bool tc;                 // tcgen05 path (mixed precisions only)
  int64_t M, K, N, Kp;
  GroupSpec mg, kg;        // access of the running tensor as [M, K]
  std::vector<int> out_labels;       // labels of C = [N legs..., M legs...]
  std::vector<int64_t> out_dims;
  int64_t out_elems;
  // packed static operand (owned by the map)
  double2* b64 = nullptr;          // [N][K] c128 (conj applied)
  float2* b32 = nullptr;           // [N][K] c64
  __nv_bfloat16* bpl = nullptr;    // [P][2N][2Kp] slice planes
  int bplanes = 0;
  int bfp16 = 0;                   // planes hold fp16 slices scaled per complex row by bmax
  float* bmax = nullptr;           // [N] row maxima of the static (fp16 planes)
  GatherTab tab;                   // offset tables of the running tensor's [M, K] view (tc steps)
  int splitk = 1;                  // K slices of the SIMT GEMM (few output tiles, long K)
  double macs = 0;
};

// Entry guard of the public calls that run a map: a map owns its workspace and Krylov
// basis, so like the reference's WorkspaceMap (lib/GraftPlanning/src/Planning/
// types.jl:503-552) it is task-local and non-reentrant; a second concurrent call is refused.
struct MapUse {
  gtn_map_s* m;
  bool ok;
  explicit MapUse(gtn_map_s* map);
  ~MapUse();
};
int map_busy_error(gtn_map_s* map);

struct gtn_map_s {
  gtn_ctx ctx = nullptr;
  std::atomic<int> busy{0};  // set while a public call runs on this map (maps are not reentrant)
  int precision = 0;
  std::vector<int64_t> x_dims, y_dims;
  int64_t x_elems = 0, y_elems = 0;
  std::vector<PlanStep> steps;
  GroupSpec fin_mg, fin_kg;  // final permute of the last C into y order
  GatherTab fin_tab;         // its offset tables
  int64_t fin_M = 0, fin_K = 0;
  bool fin_identity = false;
  double flops = 0;        // algorithmic FLOPs of the reference's env-first chain
  double exec_flops = 0;   // FLOPs of the executed (possibly grouped) chain
  int n_groups = 0;
  gtn_map fp64_alt = nullptr;  // FP64-optimal plan sharing this map's workspace
  gtn_map fp64_map = nullptr;  // caller-set map serving this map's FP64 applications (not owned)
  int64_t max_t = 0;       // largest running tensor (elements)
  int64_t max_a = 0;       // largest A operand (elements, for permuted / split staging)
  int64_t max_apl = 0;     // largest split-plane staging (bf16 elements per plane * planes)
  int64_t max_mtc = 0;     // largest M of a tensor-core step (fp16 row maxima)
  int64_t max_splitk = 0;  // largest split-K partial-sum workspace (complex elements)
  bool oneshot = false;    // a one-shot contraction (gtn_contract): arena allocations, no tables
  char* arena = nullptr;   // allocations come from here first (one-shot contractions)
  size_t arena_cap = 0, arena_off = 0, arena_spill = 0;
  void* skbuf = nullptr;   // that workspace
  float* amax = nullptr;   // [max_mtc] row maxima of the running operand (fp16 planes)
  // device workspace owned by the map
  void* buf0 = nullptr; void* buf1 = nullptr; void* abuf = nullptr;
  void* dx = nullptr; void* dy = nullptr;     // staging for the host-buffer entry point
  int64_t bytes = 0;
  std::vector<void*> owned;
  std::vector<std::pair<void*, size_t>> blocks;  // workspace from the context's block cache
  struct PendingTab {  // offset tables filled on the device once the plan is admitted
    GroupSpec g;
    int64_t n;
    int64_t* d;
  };
  std::vector<PendingTab> pending_tabs;
  // a Krylov operator backed by block-sparse maps instead of a plan (gtn_blockmap_lanczos_*):
  // applications go to bm (its own precision) or, in FP64, to bm64
  struct gtn_blockmap_s* bm = nullptr;
  struct gtn_blockmap_s* bm64 = nullptr;
  // Krylov scratch
  double2* kv = nullptr; int kv_cap = 0;     // (krylovdim+1) vectors
  double2* kcoef = nullptr; double2* kscratch = nullptr; int kscratch_cap = 0;
};

int plan_build(gtn_ctx ctx, int n_operands, const int* ranks, const int64_t* dims,
               const int* labels, const int* conj, const int* order, const void* const* statics,
               int precision, gtn_map map, bool allow_group = true, bool alloc_ws = true);
int map_run(gtn_map map, int precision, const double2* x, double2* y);
// One eager application of a block-sparse map (no graph), in its own precision.
int blockmap_run(struct gtn_blockmap_s* bm, const double2* x, double2* y);
int blockmap_precision(struct gtn_blockmap_s* bm);
int map_run_profiled(gtn_map map, int precision, const double2* x, double2* y, int cap, double* ms,
                     int* kind, double* flops, int* count);
void map_free(gtn_map map);
int map_run_batched(gtn_map* maps, int n, int precision, const double2* const* xs, double2* const* ys);
