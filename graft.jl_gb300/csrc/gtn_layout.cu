// Layout kernels: strided gathers (permutations), bf16 slice splitting for the tcgen05
// operands, and the strided small-K contraction used for TTNO (W) steps.  All are
// HBM-bound; tiles are 32x32 through shared memory so that both the read and the write
// side are coalesced.
#include "gtn_internal.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

namespace {

__device__ __forceinline__ int64_t decompose(int64_t i, const GroupSpec& g) {
  int64_t off = 0;
#pragma unroll 1
  for (int j = g.n - 1; j >= 0; --j) {
    const int64_t d = g.dim[j];
    const int64_t q = i / d;
    off += (i - q * d) * g.str[j];
    i = q;
  }
  return off;
}

template <typename T> struct Zero;
template <> struct Zero<double2> { __device__ static double2 v() { return make_double2(0.0, 0.0); } };
template <> struct Zero<float2> { __device__ static float2 v() { return make_float2(0.f, 0.f); } };

// Complex FP64 inputs of FP32 copies and of the fp16 and bf16 slice planes are converted with
// integer operations on the doubles' bits: on this part FP64 arithmetic and the F64->F32
// conversion run far below the integer rate and bounded the c128 splits (a multiply,
// conversions and subtractions per value).
// x * 2^shift rounded to float (nearest, ties to even); magnitudes below FLT_MIN become a
// signed zero (far below the fp16 planes' resolution after the row scaling, and 2^-126 of any
// FP32 or bf16 operand of practical size), NaN stays NaN.
__device__ __forceinline__ float d2f_scaled_rn(double x, int shift) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned long long mag = b & 0x7fffffffffffffffull;
  const uint32_t sgn = static_cast<uint32_t>(b >> 32) & 0x80000000u;
  const int E = static_cast<int>(mag >> 52);
  const unsigned long long m52 = mag & 0xfffffffffffffull;
  if (E == 0x7ff) return __uint_as_float(sgn | (m52 ? 0x7fc00000u : 0x7f800000u));
  if (E == 0) return __uint_as_float(sgn);
  const int fe = E - 1023 + shift + 127;  // biased float exponent before rounding
  if (fe < 1) return __uint_as_float(sgn);
  if (fe > 254) return __uint_as_float(sgn | 0x7f800000u);
  unsigned long long r = (static_cast<unsigned long long>(fe) << 52) | m52;
  r += 0x0fffffffull + ((r >> 29) & 1ull);  // round half to even at the 29 dropped bits
  return __uint_as_float(sgn | static_cast<uint32_t>(r >> 29));  // a carry moves into the exponent
}
__device__ __forceinline__ double2 cvt(double2 a, double2*) { return a; }
__device__ __forceinline__ float2 cvt(double2 a, float2*) {
  return make_float2(d2f_scaled_rn(a.x, 0), d2f_scaled_rn(a.y, 0));
}
__device__ __forceinline__ float2 cvt(float2 a, float2*) { return a; }
__device__ __forceinline__ double2 cvt(float2 a, double2*) { return make_double2(a.x, a.y); }

// Writer for complex outputs: out[m*ldo + k].
template <typename Tout> struct ComplexWriter {
  Tout* out;
  int64_t ldo;
  template <typename Tin> __device__ void operator()(int64_t m, int64_t k, Tin v) const {
    out[m * ldo + k] = cvt(v, (Tout*)nullptr);
  }
};

// Splits x into 3 bf16 slices x = s0 + s1 + s2 (round-to-nearest each step; exact for a float,
// whose 24 significant bits the three 8-bit slices hold).
__device__ __forceinline__ void split3(float x, __nv_bfloat16* s) {
  __nv_bfloat16 a = __float2bfloat16_rn(x);
  float r = x - __bfloat162float(a);
  __nv_bfloat16 b = __float2bfloat16_rn(r);
  r -= __bfloat162float(b);
  s[0] = a; s[1] = b; s[2] = __float2bfloat16_rn(r);
}
// A double is first rounded to float (nearest, from its bits): the slices then hold x to a
// relative 2^-25, below the dropped products of the six-product bf16 GEMM.
__device__ __forceinline__ void split3(double x, __nv_bfloat16* s) { split3(d2f_scaled_rn(x, 0), s); }

// Writer for bf16 slice planes.
struct SplitWriter {
  __nv_bfloat16* out;
  int64_t ld2;      // row pitch in bf16 elements (= 2*Kp)
  int64_t pstride;  // plane pitch in bf16 elements
  int nplanes;
  template <typename Tin> __device__ void operator()(int64_t m, int64_t k, Tin v) const {
    __nv_bfloat16 sr[3], si[3];
    split3(v.x, sr);
    split3(v.y, si);
    __nv_bfloat162* row = reinterpret_cast<__nv_bfloat162*>(out + m * ld2 + 2 * k);
    for (int p = 0; p < nplanes; ++p) {
      __nv_bfloat162 pr;
      pr.x = sr[p];
      pr.y = si[p];
      *reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<__nv_bfloat16*>(row) + p * pstride) = pr;
    }
  }
};

// Element offsets of the rows m and columns k of a gather: decomposed through index groups,
// or read from precomputed tables (dense maps, built once per plan step).
// GrpOff refers to groups that already live in device-visible kernel parameters; it is built
// inside a kernel and never passed to one (a host reference would make the device read host
// memory, which Grace's coherent link allows silently, after the host may have freed it).
struct GrpOff {
  const GroupSpec& mg;
  const GroupSpec& kg;
  __device__ int64_t m(int64_t i) const { return decompose(i, mg); }
  __device__ int64_t k(int64_t i) const { return decompose(i, kg); }
};
// The same with the groups held by value: the form a launch passes as a kernel parameter.
struct GrpOffV {
  GroupSpec mg;
  GroupSpec kg;
  __device__ int64_t m(int64_t i) const { return decompose(i, mg); }
  __device__ int64_t k(int64_t i) const { return decompose(i, kg); }
};
struct TabOff {
  const int64_t* __restrict__ om;
  const int64_t* __restrict__ ok;
  __device__ int64_t m(int64_t i) const { return om[i]; }
  __device__ int64_t k(int64_t i) const { return ok[i]; }
};

// Shared-memory staging of a 32 x 32 tile.  Kernels declare it once and pass it to every
// writer variant they instantiate (a static array inside a templated device function would
// be allocated once per instantiation).
template <typename Tin> struct Smem32 {
  int64_t offM[32];
  int64_t offK[32];
  Tin tile[32][33];
};

// Tile gather: rows m (M), columns k (K valid, Kw written).  m_fast selects whether the
// load phase maps lanes to m (the running tensor's unit-stride leg is in M) or to k.
template <typename Tin, class Writer, class Off>
__device__ __forceinline__ void gather_tile_o(const Tin* __restrict__ T, const Off& off, int64_t M, int64_t K,
                                              int64_t Kw, int m_fast, const Writer& w, int64_t m0, int64_t k0,
                                              Smem32<Tin>& sm) {
  int64_t* offM = sm.offM;
  int64_t* offK = sm.offK;
  auto& tile = sm.tile;
  const int tx = threadIdx.x, ty = threadIdx.y;
  if (ty == 0) {
    const int64_t m = m0 + tx;
    offM[tx] = m < M ? off.m(m) : 0;
  } else if (ty == 1) {
    const int64_t k = k0 + tx;
    offK[tx] = k < K ? off.k(k) : 0;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int im = m_fast ? tx : r;
    const int ik = m_fast ? r : tx;
    const int64_t m = m0 + im, k = k0 + ik;
    tile[im][ik] = (m < M && k < K) ? T[offM[im] + offK[ik]] : Zero<Tin>::v();
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int64_t m = m0 + r, k = k0 + tx;
    if (m < M && k < Kw) w(m, k, tile[r][tx]);
  }
}

template <typename Tin, class Writer>
__device__ __forceinline__ void gather_tile(const Tin* __restrict__ T, const GroupSpec& mg, const GroupSpec& kg,
                                            int64_t M, int64_t K, int64_t Kw, int m_fast, const Writer& w,
                                            int64_t m0, int64_t k0, Smem32<Tin>& sm) {
  gather_tile_o<Tin, Writer, GrpOff>(T, GrpOff{mg, kg}, M, K, Kw, m_fast, w, m0, k0, sm);
}

// Table-driven tile of kTabRows x 32: every thread keeps kTabRows / 8 loads in flight
// before the transpose (the gathers are latency-bound at 32 x 32).
constexpr int kTabRows = 64;

// TM x TK tile of 2048 elements (8 loads in flight per thread).  64 x 32 in general; 256 x 8
// when the rows are the unit-stride index, so that every k reads a 4 KB contiguous run
// (a 32-wide tile over far-apart k legs touches 32 pages per tile).
template <typename Tin, class Writer, int TM, int TK>
__global__ void __launch_bounds__(256) gather_tab_kernel(const Tin* __restrict__ T, TabOff off, int64_t M,
                                                         int64_t K, int64_t Kw, int m_fast, Writer w) {
  static_assert(TM * TK == 2048, "2048 elements per tile");
  __shared__ int64_t offM[TM];
  __shared__ int64_t offK[TK];
  __shared__ Tin tile[TM][TK + 1];
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const int64_t m0 = (int64_t)blockIdx.x * TM, k0 = (int64_t)blockIdx.y * TK;
  for (int i = tid; i < TM + TK; i += 256) {
    if (i < TM)
      offM[i] = m0 + i < M ? off.m(m0 + i) : 0;
    else
      offK[i - TM] = k0 + (i - TM) < K ? off.k(k0 + (i - TM)) : 0;
  }
  __syncthreads();
  Tin v[8];
#pragma unroll
  for (int it = 0; it < 8; ++it) {
    const int e = it * 256 + tid;
    const int im = m_fast ? (e % TM) : (e / TK);
    const int ik = m_fast ? (e / TM) : (e % TK);
    v[it] = (m0 + im < M && k0 + ik < K) ? T[offM[im] + offK[ik]] : Zero<Tin>::v();
  }
#pragma unroll
  for (int it = 0; it < 8; ++it) {
    const int e = it * 256 + tid;
    const int im = m_fast ? (e % TM) : (e / TK);
    const int ik = m_fast ? (e / TM) : (e % TK);
    tile[im][ik] = v[it];
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < 8; ++it) {
    const int e = it * 256 + tid;
    const int r = e / TK, c = e % TK;
    if (m0 + r < M && k0 + c < Kw) w(m0 + r, k0 + c, tile[r][c]);
  }
}

template <typename Tin, class Writer>
cudaError_t launch_gather_tab(const Tin* T, const int64_t* om, const int64_t* ok, int64_t M, int64_t K, int64_t Kw,
                              int m_fast, const Writer& w, cudaStream_t s) {
  if (M <= 0 || Kw <= 0) return cudaSuccess;
  if (m_fast) {
    const int64_t gy = (Kw + 7) / 8, gx = (M + 255) / 256;
    if (gy > 65535 || gx > 2147483647LL) return cudaErrorInvalidConfiguration;
    gather_tab_kernel<Tin, Writer, 256, 8><<<dim3((unsigned)gx, (unsigned)gy), dim3(32, 8), 0, s>>>(
        T, TabOff{om, ok}, M, K, Kw, m_fast, w);
  } else {
    const int64_t gy = (Kw + 31) / 32, gx = (M + 63) / 64;
    if (gy > 65535 || gx > 2147483647LL) return cudaErrorInvalidConfiguration;
    gather_tab_kernel<Tin, Writer, 64, 32><<<dim3((unsigned)gx, (unsigned)gy), dim3(32, 8), 0, s>>>(
        T, TabOff{om, ok}, M, K, Kw, m_fast, w);
  }
  return cudaGetLastError();
}

template <typename Tin, class Writer>
__global__ void __launch_bounds__(256) gather_tile_kernel(const Tin* __restrict__ T, GroupSpec mg,
                                                          GroupSpec kg, int64_t M, int64_t K,
                                                          int64_t Kw, int m_fast, Writer w) {
  __shared__ Smem32<Tin> sm;
  gather_tile<Tin, Writer>(T, mg, kg, M, K, Kw, m_fast, w, (int64_t)blockIdx.x * 32, (int64_t)blockIdx.y * 32, sm);
}

inline bool choose_m_fast(const GroupSpec& mg, const GroupSpec& kg) {
  const int64_t sm = mg.n > 0 ? mg.str[mg.n - 1] : INT64_MAX;
  const int64_t sk = kg.n > 0 ? kg.str[kg.n - 1] : INT64_MAX;
  return sm < sk;
}

template <typename Tin, class Writer>
cudaError_t launch_gather(const Tin* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M,
                          int64_t K, int64_t Kw, const Writer& w, cudaStream_t s) {
  if (M <= 0 || Kw <= 0) return cudaSuccess;
  const int64_t gy = (Kw + 31) / 32;
  const int64_t gx = (M + 31) / 32;
  if (gy > 65535 || gx > 2147483647LL) return cudaErrorInvalidConfiguration;
  dim3 grid((unsigned)gx, (unsigned)gy), block(32, 8);
  gather_tile_kernel<Tin, Writer><<<grid, block, 0, s>>>(T, mg, kg, M, K, Kw,
                                                         choose_m_fast(mg, kg) ? 1 : 0, w);
  return cudaGetLastError();
}

// Expanded static operand for the tcgen05 path.
__global__ void pack_b_planes_kernel(const double2* __restrict__ B, int64_t N, int64_t K, int64_t Kp,
                                     int nplanes, int64_t pstride, __nv_bfloat16* __restrict__ out) {
  const int64_t total = 2 * N * Kp;  // (row = (n, c_out)) x (complex column k)
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = idx / Kp;
    const int64_t k = idx - row * Kp;
    const int64_t n = row >> 1;
    const int c_out = (int)(row & 1);
    double v0 = 0.0, v1 = 0.0;  // columns (k, re) and (k, im)
    if (k < K) {
      const double2 b = B[n * K + k];
      if (c_out == 0) { v0 = b.x; v1 = -b.y; } else { v0 = b.y; v1 = b.x; }
    }
    __nv_bfloat16 s0[3], s1[3];
    split3(v0, s0);
    split3(v1, s1);
    for (int p = 0; p < nplanes; ++p) {
      __nv_bfloat162 pr;
      pr.x = s0[p];
      pr.y = s1[p];
      *reinterpret_cast<__nv_bfloat162*>(out + p * pstride + row * (2 * Kp) + 2 * k) = pr;
    }
  }
}

// ---- fp16 slice planes: x * s = hi + lo, s a power-of-two row scale ---------------------
__device__ __forceinline__ void split16(float x, __half* h, __half* l) {
  *h = __float2half_rn(x);
  *l = __float2half_rn(x - __half2float(*h));
}
// The same scaled split as the float overload, for a double and a power-of-two scale s.
__device__ __forceinline__ void split16_scaled(double x, float s, __half* h, __half* l) {
  const float xf = d2f_scaled_rn(x, (int)((__float_as_uint(s) >> 23) & 0xffu) - 127);
  *h = __float2half_rn(xf);
  *l = __float2half_rn(xf - __half2float(*h));
}
__device__ __forceinline__ void split16_scaled(float x, float s, __half* h, __half* l) { split16(x * s, h, l); }
__device__ __forceinline__ float absmax2(float2 v) { return fmaxf(fabsf(v.x), fabsf(v.y)); }
// max(|re|, |im|) of a complex double as a float upper bound with the same binary exponent
// (truncated mantissa), from the bits: NaN entries are ignored like fmax does, a magnitude
// below FLT_MIN gives FLT_MIN (so the row still gets a scale that resolves it).
__device__ __forceinline__ float absmax2(double2 v) {
  constexpr unsigned long long kAbs = 0x7fffffffffffffffull, kInf = 0x7ff0000000000000ull;
  unsigned long long a = static_cast<unsigned long long>(__double_as_longlong(v.x)) & kAbs;
  unsigned long long c = static_cast<unsigned long long>(__double_as_longlong(v.y)) & kAbs;
  if (a > kInf) a = 0;
  if (c > kInf) c = 0;
  const unsigned long long m = a > c ? a : c;
  if (m == 0) return 0.f;
  const int fe = static_cast<int>(m >> 52) - 1023 + 127;
  if (fe < 1) return __uint_as_float(0x00800000u);
  if (fe > 254) return __uint_as_float(0x7f800000u);
  return __uint_as_float((static_cast<uint32_t>(fe) << 23) | static_cast<uint32_t>((m >> 29) & 0x7fffffu));
}

// Element (m, k) as two fp16 planes, the row scaled by fp16_row_scale of its maximum.
template <typename Tin>
__device__ __forceinline__ void put16(__half* out, int64_t ld2, int64_t pstride, int64_t m, int64_t k, Tin v,
                                      float rowmax) {
  const float s = fp16_row_scale(rowmax);
  __half2 hi, lo;
  split16_scaled(v.x, s, &hi.x, &lo.x);
  split16_scaled(v.y, s, &hi.y, &lo.y);
  __half2* row = reinterpret_cast<__half2*>(out + m * ld2 + 2 * k);
  row[0] = hi;
  *reinterpret_cast<__half2*>(reinterpret_cast<__half*>(row) + pstride) = lo;
}

struct Split16Writer {
  __half* out;
  int64_t ld2;      // row pitch in halves (= 2*Kp)
  int64_t pstride;  // plane pitch in halves
  const float* amax;
  template <typename Tin> __device__ void operator()(int64_t m, int64_t k, Tin v) const {
    put16(out, ld2, pstride, m, k, v, amax[m]);
  }
};
// The same, handed the row maximum (the fused split computes it in shared memory), for two
// adjacent columns k, k + 1 (k even): one 8-byte store per plane.
struct Split16RowWriter {
  __half* out;
  int64_t ld2;
  int64_t pstride;
  template <typename Tin> __device__ void operator()(int64_t m, int64_t k, Tin v0, Tin v1, float rowmax) const {
    const float s = fp16_row_scale(rowmax);
    __half2 h0, l0, h1, l1;
    split16_scaled(v0.x, s, &h0.x, &l0.x);
    split16_scaled(v0.y, s, &h0.y, &l0.y);
    split16_scaled(v1.x, s, &h1.x, &l1.x);
    split16_scaled(v1.y, s, &h1.y, &l1.y);
    __half* row = out + m * ld2 + 2 * k;
    uint2 hv, lv;
    hv.x = *reinterpret_cast<uint32_t*>(&h0);
    hv.y = *reinterpret_cast<uint32_t*>(&h1);
    lv.x = *reinterpret_cast<uint32_t*>(&l0);
    lv.y = *reinterpret_cast<uint32_t*>(&l1);
    *reinterpret_cast<uint2*>(row) = hv;
    *reinterpret_cast<uint2*>(row + pstride) = lv;
  }
};

// ---- integer digit planes of the FP64-grade tensor-core GEMM (gtn_gemm_f64e.cu) ---------
// x 2^k (|x| 2^k < 1, k from the row maximum) as kF64eSlices signed base-128 digits,
// x 2^k = sum_i d_i 2^{-7(i+1)}: the fixed-point value N = round(x 2^{k + 7 S}) is formed
// from the double's bits with integer operations (no FP64 arithmetic), then peeled from the
// top digit down with round-half-up shifts; |d_0| <= 128, |d_i| <= 64, all exact in bf16.
__device__ __forceinline__ int f64e_row_exp(float mx) {
  const uint32_t b = __float_as_uint(mx);
  const int e = (int)((b >> 23) & 0xffu);
  return mx > 0.f ? 126 - e : 0;
}
__device__ __forceinline__ void i7_digits(double x, int k, __nv_bfloat16* d) {
  constexpr int NB = 7 * kF64eSlices;
  const long long bits = __double_as_longlong(x);
  const int E = (int)((bits >> 52) & 0x7ff);
  long long N = 0;
  if (E != 0 && E != 0x7ff) {
    const long long mant = (bits & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
    const int r = 1075 - E - k - NB;  // >= 4 whenever |x| 2^k < 1
    if (r <= 0) N = mant << (r < -10 ? 10 : -r);
    else if (r < 63) N = (mant + (1LL << (r - 1))) >> r;
    if (bits < 0) N = -N;
  }
#pragma unroll
  for (int i = 0; i < kF64eSlices; ++i) {
    const int w = 7 * (kF64eSlices - 1 - i);
    long long di;
    if (w > 0) {
      di = (N + (1LL << (w - 1))) >> w;
      N -= di << w;
    } else {
      di = N;
    }
    d[i] = __float2bfloat16_rn((float)di);
  }
}
__device__ __forceinline__ void i7_digits(float x, int k, __nv_bfloat16* d) { i7_digits((double)x, k, d); }

// Element (m, k) as kF64eSlices digit planes, the row scaled by 2^k of its maximum.
template <typename Tin>
__device__ __forceinline__ void put_i7(__nv_bfloat16* out, int64_t ld2, int64_t pstride, int64_t m, int64_t k,
                                       Tin v, float rowmax) {
  const int e = f64e_row_exp(rowmax);
  __nv_bfloat16 dr[kF64eSlices], di[kF64eSlices];
  i7_digits(v.x, e, dr);
  i7_digits(v.y, e, di);
  __nv_bfloat16* row = out + m * ld2 + 2 * k;
#pragma unroll
  for (int p = 0; p < kF64eSlices; ++p) {
    __nv_bfloat162 pr;
    pr.x = dr[p];
    pr.y = di[p];
    *reinterpret_cast<__nv_bfloat162*>(row + p * pstride) = pr;
  }
}

struct Int7Writer {
  __nv_bfloat16* out;
  int64_t ld2;      // row pitch (= 2 Kp)
  int64_t pstride;  // plane pitch
  const float* amax;
  template <typename Tin> __device__ void operator()(int64_t m, int64_t k, Tin v) const {
    put_i7(out, ld2, pstride, m, k, v, amax[m]);
  }
};
struct Int7RowWriter {
  __nv_bfloat16* out;
  int64_t ld2;
  int64_t pstride;
  template <typename Tin> __device__ void operator()(int64_t m, int64_t k, Tin v0, Tin v1, float rowmax) const {
    put_i7(out, ld2, pstride, m, k, v0, rowmax);
    put_i7(out, ld2, pstride, m, k + 1, v1, rowmax);
  }
};

__global__ void pack_b_planes_i7_kernel(const double2* __restrict__ B, int64_t N, int64_t K, int64_t Kp,
                                        int64_t pstride, const float* __restrict__ bmax,
                                        __nv_bfloat16* __restrict__ out) {
  const int64_t total = 2 * N * Kp;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = idx / Kp;
    const int64_t k = idx - row * Kp;
    const int64_t n = row >> 1;
    const int e = f64e_row_exp(bmax[n]);
    double v0 = 0.0, v1 = 0.0;
    if (k < K) {
      const double2 b = B[n * K + k];
      if ((row & 1) == 0) { v0 = b.x; v1 = -b.y; } else { v0 = b.y; v1 = b.x; }
    }
    __nv_bfloat16 d0[kF64eSlices], d1[kF64eSlices];
    i7_digits(v0, e, d0);
    i7_digits(v1, e, d1);
    for (int p = 0; p < kF64eSlices; ++p) {
      __nv_bfloat162 pr;
      pr.x = d0[p];
      pr.y = d1[p];
      *reinterpret_cast<__nv_bfloat162*>(out + p * pstride + row * (2 * Kp) + 2 * k) = pr;
    }
  }
}

// amax[m] = max over k of max(|re|, |im|) of the K-major gather (atomic max of the
// non-negative float bits; amax zeroed before the launch).
template <typename Tin, class Off, int TM, int TK>
__device__ __forceinline__ void rowmax_tile(const Tin* __restrict__ T, const Off& off, int64_t M, int64_t K, int m_fast,
                                            float* __restrict__ amax, int64_t m0, int64_t k0) {
  // TM x TK = 2048 elements per tile (8 loads in flight per thread); 256 x 8 when the rows
  // are the unit-stride index (long contiguous runs per k), else 64 x 32
  static_assert(TM * TK == 2048 && TK <= 32, "tile shape");
  __shared__ int64_t offM[TM];
  __shared__ int64_t offK[TK];
  __shared__ float tile[TM][TK + 1];
  const int tid = threadIdx.x + 32 * threadIdx.y;
  for (int i = tid; i < TM + TK; i += 256) {
    if (i < TM)
      offM[i] = m0 + i < M ? off.m(m0 + i) : 0;
    else
      offK[i - TM] = k0 + (i - TM) < K ? off.k(k0 + (i - TM)) : 0;
  }
  __syncthreads();
  float v[8];
#pragma unroll
  for (int it = 0; it < 8; ++it) {
    const int e = it * 256 + tid;
    const int im = m_fast ? (e % TM) : (e / TK);
    const int ik = m_fast ? (e / TM) : (e % TK);
    v[it] = (m0 + im < M && k0 + ik < K) ? absmax2(T[offM[im] + offK[ik]]) : 0.f;
  }
#pragma unroll
  for (int it = 0; it < 8; ++it) {
    const int e = it * 256 + tid;
    const int im = m_fast ? (e % TM) : (e / TK);
    const int ik = m_fast ? (e / TM) : (e % TK);
    tile[im][ik] = v[it];
  }
  __syncthreads();
  // row r's TK values sit on TK consecutive lanes: segmented max, one atomic per row
#pragma unroll
  for (int it = 0; it < 8; ++it) {
    const int e = it * 256 + tid;
    const int r = e / TK, c = e % TK;
    float x = tile[r][c];
#pragma unroll
    for (int o = TK / 2; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
    if (c == 0 && m0 + r < M && x > 0.f) atomicMax(reinterpret_cast<unsigned int*>(amax) + m0 + r, __float_as_uint(x));
  }
}

template <typename Tin, class Off, int TM, int TK>
__global__ void __launch_bounds__(256) rowmax_kernel(const Tin* __restrict__ T, Off off, int64_t M, int64_t K,
                                                     int m_fast, float* __restrict__ amax) {
  rowmax_tile<Tin, Off, TM, TK>(T, off, M, K, m_fast, amax, (int64_t)blockIdx.x * TM, (int64_t)blockIdx.y * TK);
}

// bmax[n] = max over k of max(|re|, |im|) of B[n][:], one CTA per row
__global__ void __launch_bounds__(256) bmax_kernel(const double2* __restrict__ B, int64_t K, float* __restrict__ bmax) {
  __shared__ float red[256];
  const double2* b = B + (int64_t)blockIdx.x * K;
  float v = 0.f;
  for (int64_t k = threadIdx.x; k < K; k += 256) v = fmaxf(v, absmax2(b[k]));
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) bmax[blockIdx.x] = red[0];
}

// B' = [[Br, -Bi], [Bi, Br]] as 2 fp16 planes, complex row n scaled by fp16_row_scale(bmax[n])
__global__ void pack_b_planes_f16_kernel(const double2* __restrict__ B, int64_t N, int64_t K, int64_t Kp,
                                         int64_t pstride, const float* __restrict__ bmax, __half* __restrict__ out) {
  const int64_t total = 2 * N * Kp;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = idx / Kp;
    const int64_t k = idx - row * Kp;
    const int64_t n = row >> 1;
    const float s = fp16_row_scale(bmax[n]);
    double v0 = 0.0, v1 = 0.0;
    if (k < K) {
      const double2 b = B[n * K + k];
      if ((row & 1) == 0) { v0 = b.x; v1 = -b.y; } else { v0 = b.y; v1 = b.x; }
    }
    __half2 hi, lo;
    split16_scaled(v0, s, &hi.x, &lo.x);
    split16_scaled(v1, s, &hi.y, &lo.y);
    *reinterpret_cast<__half2*>(out + row * (2 * Kp) + 2 * k) = hi;
    *reinterpret_cast<__half2*>(out + pstride + row * (2 * Kp) + 2 * k) = lo;
  }
}

__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}

constexpr int kSmallSmemBytes = 48 * 1024;

// C[n][m] = sum_k T[offM(m) + offK(k)] * B[n][k]; B and the K offsets live in shared memory.
template <typename T, int NB>
__device__ __forceinline__ void small_contract_body(const T* __restrict__ A, const GroupSpec& mg,
                                                    const GroupSpec& kg, int64_t M, int K, int N,
                                                    const T* __restrict__ B, T* __restrict__ C, int64_t blk,
                                                    int64_t nblk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int64_t* offK = reinterpret_cast<int64_t*>(smem_raw);
  T* Bs = reinterpret_cast<T*>(smem_raw + ((K * sizeof(int64_t) + 15) / 16) * 16);
  for (int i = threadIdx.x; i < K; i += blockDim.x) offK[i] = decompose(i, kg);
  for (int i = threadIdx.x; i < N * K; i += blockDim.x) Bs[i] = B[i];
  __syncthreads();
  for (int64_t m = blk * blockDim.x + threadIdx.x; m < M; m += nblk * blockDim.x) {
    const int64_t om = decompose(m, mg);
    for (int n0 = 0; n0 < N; n0 += NB) {
      T acc[NB];
#pragma unroll
      for (int j = 0; j < NB; ++j) acc[j] = Zero<T>::v();
      for (int k = 0; k < K; ++k) {
        const T t = A[om + offK[k]];
#pragma unroll
        for (int j = 0; j < NB; ++j)
          if (n0 + j < N) cfma(acc[j], t, Bs[(n0 + j) * K + k]);
      }
#pragma unroll
      for (int j = 0; j < NB; ++j)
        if (n0 + j < N) C[(int64_t)(n0 + j) * M + m] = acc[j];
    }
  }
}

template <typename T, int NB>
__global__ void __launch_bounds__(256) small_contract_kernel(const T* __restrict__ A, GroupSpec mg,
                                                             GroupSpec kg, int64_t M, int K, int N,
                                                             const T* __restrict__ B,
                                                             T* __restrict__ C) {
  small_contract_body<T, NB>(A, mg, kg, M, K, N, B, C, blockIdx.x, gridDim.x);
}

template <typename T>
cudaError_t launch_small(const T* A, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int K,
                         int N, const T* B, T* C, cudaStream_t s) {
  if (M <= 0) return cudaSuccess;
  const size_t smem = ((K * sizeof(int64_t) + 15) / 16) * 16 + (size_t)N * K * sizeof(T);
  if (smem > (size_t)kSmallSmemBytes) return cudaErrorInvalidValue;
  int64_t blocks = (M + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  small_contract_kernel<T, 8><<<(unsigned)blocks, 256, smem, s>>>(A, mg, kg, M, K, N, B, C);
  return cudaGetLastError();
}

// ---- grouped (multi-problem) variants: one launch for many independent jobs -------------

struct GatherJobsP {
  GatherJob j[kGatherJobMax];
  int tile_start[kGatherJobMax + 1];
  int tiles_m[kGatherJobMax];
  int m_fast[kGatherJobMax];
  int n;
};

__device__ __forceinline__ int find_job(const int* start, int n, int b) {
  int p = 0;
  while (p + 1 < n && start[p + 1] <= b) ++p;
  return p;
}

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(256) gather_grouped_kernel(const __grid_constant__ GatherJobsP g) {
  const int b = blockIdx.x;
  const int p = find_job(g.tile_start, g.n, b);
  const GatherJob& J = g.j[p];
  const int t = b - g.tile_start[p];
  const int64_t m0 = (int64_t)(t % g.tiles_m[p]) * 32, k0 = (int64_t)(t / g.tiles_m[p]) * 32;
  __shared__ Smem32<Tin> sm;
  if (J.nplanes > 0 && J.amax) {
    Split16Writer w{static_cast<__half*>(J.out), 2 * (J.ld > 0 ? J.ld : J.Kw), J.pstride, J.amax};
    gather_tile<Tin, Split16Writer>(static_cast<const Tin*>(J.T), J.mg, J.kg, J.M, J.K, J.Kw, g.m_fast[p], w, m0, k0,
                                    sm);
  } else if (J.nplanes > 0) {
    SplitWriter w{static_cast<__nv_bfloat16*>(J.out), 2 * (J.ld > 0 ? J.ld : J.Kw), J.pstride, J.nplanes};
    gather_tile<Tin, SplitWriter>(static_cast<const Tin*>(J.T), J.mg, J.kg, J.M, J.K, J.Kw, g.m_fast[p], w, m0, k0,
                                  sm);
  } else {
    ComplexWriter<Tout> w{static_cast<Tout*>(J.out), J.ld};
    gather_tile<Tin, ComplexWriter<Tout>>(static_cast<const Tin*>(J.T), J.mg, J.kg, J.M, J.K, J.Kw, g.m_fast[p], w,
                                          m0, k0, sm);
  }
}

struct SmallJobsP {
  SmallJob j[kGatherJobMax];
  int blk_start[kGatherJobMax + 1];
  int n;
};

template <typename T>
__global__ void __launch_bounds__(256) small_grouped_kernel(const __grid_constant__ SmallJobsP g) {
  const int b = blockIdx.x;
  const int p = find_job(g.blk_start, g.n, b);
  const SmallJob& J = g.j[p];
  small_contract_body<T, 8>(static_cast<const T*>(J.A), J.mg, J.kg, J.M, J.K, J.N, static_cast<const T*>(J.B),
                            static_cast<T*>(J.C), b - g.blk_start[p], g.blk_start[p + 1] - g.blk_start[p]);
}

// Row offset by 32-bit multiply-shift division: q = floor(i / d) = umulhi(i, mag) >> sh
// for i < 2^31, with mag = floor(2^(31+l) / d) + 1, l = ceil(log2 d), sh = l - 1 (the
// round-up method of Granlund and Montgomery, PLDI 1994, exact since mag*d - 2^(31+l) <= 2^l).
__device__ __forceinline__ int64_t decompose_fast(int64_t m, const DevGatherJob& J) {
  uint32_t i = (uint32_t)m;
  int64_t off = 0;
#pragma unroll 1
  for (int j = J.mg.n - 1; j >= 0; --j) {
    const uint32_t d = (uint32_t)J.mg.dim[j];
    const uint32_t q = d == 1u ? i : (__umulhi(i, J.m_mag[j]) >> J.m_sh[j]);
    off += (int64_t)(i - q * d) * J.mg.str[j];
    i = q;
  }
  return off;
}

// Adaptive block-move tile: (1024 >> tks) rows x (1 << tks) columns, so that narrow
// coupled-charge blocks (K of a few elements) still move 1024 elements per CTA.  The
// shared tile is skewed by one element every 32 to spread the transposed accesses.
template <typename Tin> struct SmemA {
  int64_t offM[1024];
  int64_t offK[32];
  Tin tile[1024 + 32];
};

template <typename Tin, class Writer>
__device__ __forceinline__ void gather_tile_adaptive(const Tin* __restrict__ T, const DevGatherJob& J,
                                                     const Writer& w, int64_t m0, int64_t k0, SmemA<Tin>& sm) {
  int64_t* offM = sm.offM;
  int64_t* offK = sm.offK;
  Tin* tile = sm.tile;
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const int tks = J.tks, TK = 1 << tks, TM = 1024 >> tks;
  for (int i = tid; i < TM; i += 256) {
    const int64_t m = m0 + i;
    offM[i] = m < J.M ? (J.fast_m ? decompose_fast(m, J) : decompose(m, J.mg)) : 0;
  }
  if (tid < TK) {
    const int64_t k = k0 + tid;
    offK[tid] = k < J.K ? decompose(k, J.kg) : 0;
  }
  __syncthreads();
  for (int e = tid; e < 1024; e += 256) {
    int im, ik;
    if (J.m_fast) {
      im = e & (TM - 1);
      ik = e >> (10 - tks);
    } else {
      ik = e & (TK - 1);
      im = e >> tks;
    }
    const int64_t m = m0 + im, k = k0 + ik;
    const int sidx = im * TK + ik;
    tile[sidx + (sidx >> 5)] = (m < J.M && k < J.K) ? T[offM[im] + offK[ik]] : Zero<Tin>::v();
  }
  __syncthreads();
  for (int e = tid; e < 1024; e += 256) {
    const int ik = e & (TK - 1), im = e >> tks;
    const int64_t m = m0 + im, k = k0 + ik;
    if (m < J.M && k < J.Kw) w(m, k, tile[e + (e >> 5)]);
  }
}

// Row maxima of an adaptive tile (fp16 split of block maps): segmented max over the TK
// lanes of a row, one atomic max per row and tile.
template <typename Tin>
__device__ __forceinline__ void rowmax_tile_adaptive(const Tin* __restrict__ T, const DevGatherJob& J,
                                                     float* __restrict__ amax, int64_t m0, int64_t k0) {
  __shared__ int64_t offM[1024];
  __shared__ int64_t offK[32];
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const int tks = J.tks, TK = 1 << tks, TM = 1024 >> tks;
  for (int i = tid; i < TM; i += 256) {
    const int64_t m = m0 + i;
    offM[i] = m < J.M ? (J.fast_m ? decompose_fast(m, J) : decompose(m, J.mg)) : 0;
  }
  if (tid < TK) {
    const int64_t k = k0 + tid;
    offK[tid] = k < J.K ? decompose(k, J.kg) : 0;
  }
  __syncthreads();
  for (int e = tid; e < 1024; e += 256) {
    const int ik = e & (TK - 1), im = e >> tks;
    const int64_t m = m0 + im, k = k0 + ik;
    float v = (m < J.M && k < J.K) ? absmax2(T[offM[im] + offK[ik]]) : 0.f;
    for (int o = TK >> 1; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (ik == 0 && m < J.M && v > 0.f) atomicMax(reinterpret_cast<unsigned int*>(amax) + m, __float_as_uint(v));
  }
}

// Device-resident job table (block-sparse maps): any number of jobs in one launch; sources
// and destinations are (buffer id, element offset) resolved against the launch's bases.
template <typename Tin>
__global__ void __launch_bounds__(256) block_gather_kernel(const DevGatherJob* __restrict__ jobs,
                                                           const int2* __restrict__ tile_map, BlockBases bases) {
  const int2 jt = tile_map[blockIdx.x];
  const DevGatherJob& J = jobs[jt.x];
  const int t = jt.y;
  const int64_t m0 = (int64_t)(t % J.tiles_m) * (1024 >> J.tks), k0 = (int64_t)(t / J.tiles_m) << J.tks;
  const Tin* src = static_cast<const Tin*>(bases.buf[J.src_buf]) + J.src_off;
  __shared__ SmemA<Tin> sm;
  if (J.mode == 2) {
    Split16Writer w{reinterpret_cast<__half*>(static_cast<__nv_bfloat16*>(bases.buf[J.dst_buf]) + J.dst_off), 2 * J.ld,
                    J.pstride, static_cast<const float*>(bases.buf[5]) + J.amax_off};
    gather_tile_adaptive<Tin, Split16Writer>(src, J, w, m0, k0, sm);
  } else if (J.nplanes > 0) {
    SplitWriter w{static_cast<__nv_bfloat16*>(bases.buf[J.dst_buf]) + J.dst_off, 2 * J.ld, J.pstride, J.nplanes};
    gather_tile_adaptive<Tin, SplitWriter>(src, J, w, m0, k0, sm);
  } else if (J.dst_is64) {
    ComplexWriter<double2> w{static_cast<double2*>(bases.buf[J.dst_buf]) + J.dst_off, J.ld};
    gather_tile_adaptive<Tin, ComplexWriter<double2>>(src, J, w, m0, k0, sm);
  } else {
    ComplexWriter<float2> w{static_cast<float2*>(bases.buf[J.dst_buf]) + J.dst_off, J.ld};
    gather_tile_adaptive<Tin, ComplexWriter<float2>>(src, J, w, m0, k0, sm);
  }
}

// Fused gather + product of a block map's few-column problems.  A CTA takes a range of rows
// of one band, one thread per row.  Per pass each thread computes its row's base offset in
// every rectangle once (digits of the row in the band's common groups times the
// rectangle's strides, kept in shared memory for its own row only), then, for each chunk of
// NPT output columns, reads the row's present columns straight from the running tensor,
// eight (c64) or four (c128) loads in flight before they are used (chunks after the first
// find the row in L1).  B_q is held transposed and zero-padded to a multiple of NPT columns
// so that the products need no predicates.
constexpr int kBandMaxN64 = 32, kBandMaxN32 = 64, kBandMaxSmem = 96 * 1024, kBandRows = 256;
__host__ __device__ constexpr int band_npt(int maxn) { return maxn <= 1 ? 1 : maxn <= 2 ? 2 : maxn <= 4 ? 4 : 8; }
__host__ __device__ constexpr int band_npad(int n, int npt) { return (n + npt - 1) / npt * npt; }

template <typename Tin, typename T, int NPT>
__global__ void __launch_bounds__(256, 4) block_band_kernel(const DevBand* __restrict__ bands,
                                                            const DevBandWork* __restrict__ work,
                                                            const DevBandCol* __restrict__ cols,
                                                            const int64_t* __restrict__ rstr, BlockBases bases) {
  constexpr int LB = sizeof(Tin) == 16 ? 4 : 8;  // loads in flight
  extern __shared__ __align__(16) unsigned char band_smem[];
  const DevBandWork W = work[blockIdx.x];
  const DevBand& D = bands[W.band];
  const int N = D.N, Kq = D.Kq, ng = D.ng, nrect = D.nrect, ncol = D.ncol, NPAD = band_npad(N, NPT);
  T* Bt = reinterpret_cast<T*>(band_smem);                                // [Kq][NPAD]
  int64_t* rs = reinterpret_cast<int64_t*>(Bt + (size_t)Kq * NPAD);      // [nrect][ng]
  int64_t* base = rs + nrect * ng;                                        // [nrect][kBandRows]
  DevBandCol* cc = reinterpret_cast<DevBandCol*>(base + nrect * kBandRows);  // [ncol]
  __shared__ uint32_t sdim[kBandMaxGroups], smag[kBandMaxGroups], ssh[kBandMaxGroups];
  const int r = threadIdx.x;
  const T* __restrict__ B = static_cast<const T*>(D.B);
  for (int i = r; i < Kq * NPAD; i += 256) {
    const int k = i / NPAD, n = i - k * NPAD;
    Bt[i] = n < N ? B[(size_t)n * Kq + k] : Zero<T>::v();
  }
  for (int i = r; i < nrect * ng; i += 256) rs[i] = rstr[D.rs0 + i];
  for (int i = r; i < ncol; i += 256) cc[i] = cols[D.col0 + i];
  if (r < ng) {
    sdim[r] = D.dim[r];
    smag[r] = D.mag[r];
    ssh[r] = D.sh[r];
  }
  __syncthreads();
  const Tin* __restrict__ src = static_cast<const Tin*>(bases.buf[D.src_buf]);
  T* __restrict__ C = static_cast<T*>(bases.buf[D.c_buf]) + D.c_off;
  for (int64_t mr = r; mr < W.nrows; mr += kBandRows) {
    const int64_t m = W.m0 + mr;
    {
      int dig[kBandMaxGroups];
      uint32_t i = (uint32_t)m;
#pragma unroll
      for (int t = kBandMaxGroups - 1; t >= 0; --t) {
        dig[t] = 0;
        if (t < ng) {
          const uint32_t q = sdim[t] == 1u ? i : (__umulhi(i, smag[t]) >> ssh[t]);
          dig[t] = (int)(i - q * sdim[t]);
          i = q;
        }
      }
      for (int q = 0; q < nrect; ++q) {
        const int64_t* st = rs + q * ng;
        int64_t o = 0;
#pragma unroll
        for (int t = 0; t < kBandMaxGroups; ++t)
          if (t < ng) o += (int64_t)dig[t] * st[t];
        base[q * kBandRows + r] = o;
      }
    }
    for (int n0 = 0; n0 < N; n0 += NPT) {
      T acc[NPT];
#pragma unroll
      for (int j = 0; j < NPT; ++j) acc[j] = Zero<T>::v();
      for (int j0 = 0; j0 < ncol; j0 += LB) {
        Tin v[LB];
        int bc[LB];
#pragma unroll
        for (int u = 0; u < LB; ++u) {
          v[u] = Zero<Tin>::v();
          bc[u] = 0;
          if (j0 + u < ncol) {
            const DevBandCol c = cc[j0 + u];
            bc[u] = c.bcol;
            v[u] = src[c.src + base[c.rect * kBandRows + r]];
          }
        }
#pragma unroll
        for (int u = 0; u < LB; ++u) {
          const T a = cvt(v[u], (T*)nullptr);
          const T* bp = Bt + (size_t)bc[u] * NPAD + n0;
#pragma unroll
          for (int j = 0; j < NPT; ++j) cfma(acc[j], a, bp[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < NPT; ++j)
        if (n0 + j < N) C[(int64_t)(n0 + j) * D.ldc + m] = acc[j];
    }
  }
}

// bf16 slice planes of two adjacent columns k, k + 1 (k even): one 8-byte store per plane.
struct SplitRowWriter {
  __nv_bfloat16* out;
  int64_t ld2;
  int64_t pstride;
  int nplanes;
  template <typename Tin> __device__ void operator()(int64_t m, int64_t k, Tin v0, Tin v1, float) const {
    __nv_bfloat16 r0[3], i0[3], r1[3], i1[3];
    split3(v0.x, r0);
    split3(v0.y, i0);
    split3(v1.x, r1);
    split3(v1.y, i1);
    __nv_bfloat16* row = out + m * ld2 + 2 * k;
    for (int p = 0; p < nplanes; ++p) {
      __nv_bfloat162 a, b;
      a.x = r0[p];
      a.y = i0[p];
      b.x = r1[p];
      b.y = i1[p];
      uint2 w;
      w.x = *reinterpret_cast<uint32_t*>(&a);
      w.y = *reinterpret_cast<uint32_t*>(&b);
      *reinterpret_cast<uint2*>(row + p * pstride) = w;
    }
  }
};

// Split bands of the tensor-core problems (Kp <= 1024): a CTA stages TR whole rows of A_q
// (every present column read straight from the running tensor, absent blocks and the K
// padding zero), reduces the fp16 row maxima over the staged rows, and writes the rows'
// slice planes with one 8-byte store per plane and column pair.  The values and the split
// functions are those of the block moves, so the planes equal the staged path's.
// Rows staged per pass: as many as fit 33 KB of the tile, at most 32.
__host__ __device__ inline int split_band_tr(int Kp, int elem) {
  int tr = 32;
  while (tr > 1 && (size_t)tr * (Kp + 1) * elem > 33 * 1024) tr >>= 1;
  return tr;
}

template <typename Tin, bool F16>
__global__ void __launch_bounds__(256) block_split_band_kernel(const DevBand* __restrict__ bands,
                                                               const DevBandWork* __restrict__ work,
                                                               const DevBandCol* __restrict__ cols,
                                                               const int64_t* __restrict__ rstr, BlockBases bases) {
  extern __shared__ __align__(16) unsigned char band_smem[];
  const DevBandWork W = work[blockIdx.x];
  const DevBand& D = bands[W.band];
  const int Kp = D.Kp, P = Kp + 1, ng = D.ng, nrect = D.nrect, ncol = D.ncol;
  const int TR = split_band_tr(Kp, (int)sizeof(Tin));
  Tin* tile = reinterpret_cast<Tin*>(band_smem);                           // [TR][Kp + 1]
  int64_t* rs = reinterpret_cast<int64_t*>(tile + TR * P);                // [nrect][ng]
  int64_t* base = rs + nrect * ng;                                        // [nrect][TR]
  DevBandCol* cc = reinterpret_cast<DevBandCol*>(base + nrect * TR);     // [ncol]
  __shared__ float rmax[32];
  __shared__ uint32_t sdim[kBandMaxGroups], smag[kBandMaxGroups], ssh[kBandMaxGroups];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < nrect * ng; i += 256) rs[i] = rstr[D.rs0 + i];
  for (int i = tid; i < ncol; i += 256) cc[i] = cols[D.col0 + i];
  if (tid < ng) {
    sdim[tid] = D.dim[tid];
    smag[tid] = D.mag[tid];
    ssh[tid] = D.sh[tid];
  }
  const Tin* __restrict__ src = static_cast<const Tin*>(bases.buf[D.src_buf]);
  __half* out = reinterpret_cast<__half*>(bases.buf[4]) + D.a_off;
  const int64_t ld2 = 2 * (int64_t)Kp;
  for (int p0 = 0; p0 < W.nrows; p0 += TR) {
    const int rows = W.nrows - p0 < TR ? W.nrows - p0 : TR;
    const int64_t m0 = W.m0 + p0;
    __syncthreads();  // (first pass: strides, columns, groups; then the previous pass's tile)
    for (int e = tid; e < TR * P; e += 256) tile[e] = Zero<Tin>::v();
    for (int e = tid; e < TR * nrect; e += 256) {  // row i's base offset in rectangle q
      const int i = e % TR, q = e / TR;
      uint32_t x = (uint32_t)(m0 + (i < rows ? i : 0));
      int64_t o = 0;
      for (int t = ng - 1; t >= 0; --t) {
        const uint32_t qq = sdim[t] == 1u ? x : (__umulhi(x, smag[t]) >> ssh[t]);
        o += (int64_t)(x - qq * sdim[t]) * rs[q * ng + t];
        x = qq;
      }
      base[q * TR + i] = o;
    }
    __syncthreads();
    // every present column of the staged rows, eight loads in flight per thread
    for (int e0 = 0; e0 < TR * ncol; e0 += 8 * 256) {
      int64_t off[8];
      int slot[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = e0 + u * 256 + tid;
        int i, j;
        if (D.m_fast) {
          i = e % TR;
          j = e / TR;
        } else {
          j = e % ncol;
          i = e / ncol;
        }
        slot[u] = -1;
        off[u] = 0;
        if (e < TR * ncol && i < rows) {
          const DevBandCol c = cc[j];
          slot[u] = i * P + c.bcol;
          off[u] = c.src + base[c.rect * TR + i];
        }
      }
      Tin v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = slot[u] >= 0 ? src[off[u]] : Zero<Tin>::v();
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (slot[u] >= 0) tile[slot[u]] = v[u];
    }
    __syncthreads();
    if (F16) {  // row maxima, one warp per row
      for (int i = warp; i < rows; i += 8) {
        float mx = 0.f;
        for (int k = lane; k < Kp; k += 32) mx = fmaxf(mx, absmax2(tile[i * P + k]));
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) {
          rmax[i] = mx;
          static_cast<float*>(bases.buf[5])[D.amax_off + m0 + i] = mx;
        }
      }
      __syncthreads();
    }
    const int hw = Kp / 2;
    for (int e = tid; e < rows * hw; e += 256) {
      const int i = e / hw, c = 2 * (e - i * hw);
      const int64_t m = D.row_off + m0 + i;
      if (F16) {
        Split16RowWriter w{out, ld2, D.pstride};
        w(m, c, tile[i * P + c], tile[i * P + c + 1], rmax[i]);
      } else {
        SplitRowWriter w{reinterpret_cast<__nv_bfloat16*>(out), ld2, D.pstride, D.nplanes};
        w(m, c, tile[i * P + c], tile[i * P + c + 1], 0.f);
      }
    }
  }
}

// Row maxima of the jobs of a table (fp16 split of block maps), a kernel of its own so
// that the block moves keep their shared-memory footprint.
template <typename Tin>
__global__ void __launch_bounds__(256) block_rowmax_kernel(const DevGatherJob* __restrict__ jobs,
                                                           const int2* __restrict__ tile_map, BlockBases bases) {
  const int2 jt = tile_map[blockIdx.x];
  const DevGatherJob& J = jobs[jt.x];
  const int t = jt.y;
  const int64_t m0 = (int64_t)(t % J.tiles_m) * (1024 >> J.tks), k0 = (int64_t)(t / J.tiles_m) << J.tks;
  rowmax_tile_adaptive<Tin>(static_cast<const Tin*>(bases.buf[J.src_buf]) + J.src_off, J,
                            static_cast<float*>(bases.buf[5]) + J.amax_off, m0, k0);
}


// ---- fused split: row maxima and slice planes in one pass over the running tensor --------
// A cluster of cs CTAs owns TR rows of the K-major view; CTA r of the cluster stages the
// columns [r kc, (r + 1) kc) of those rows in shared memory (cp.async, every element read
// from HBM once), reduces its partial row maxima, and reads its peers' partial maxima
// through distributed shared memory after a cluster barrier.  It then writes its columns
// of the slice planes, scaled by the full row maxima, and the cluster's rank 0 writes them
// to amax[] for the GEMM epilogue.  The second cluster barrier (arrive after the peer
// reads, wait before exit) keeps each CTA's partial maxima alive while peers read them.
// The barriers are hardware cluster barriers: every CTA of a cluster is co-scheduled and
// every thread reaches both, so no wait can be left hanging.
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.aligned;" ::: "memory"); }
__device__ __forceinline__ float ld_peer_f32(const float* p, uint32_t rank) {
  const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(p));
  uint32_t ra;
  float v;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(ra) : "memory");
  return v;
}
__device__ __forceinline__ void cp_async_el(float2* dst, const float2* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_el(double2* dst, const double2* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// q = floor(i / d) for i < 2^31 by a multiply and a shift (Granlund and Montgomery's
// round-up method, as in decompose_fast); the magic number is made once per CTA.
struct FastDiv {
  uint32_t d, mag, sh;
};
__device__ __forceinline__ FastDiv make_fastdiv(uint32_t d) {
  if (d <= 1) return FastDiv{1u, 0u, 0u};
  uint32_t l = 0;
  while ((1u << l) < d) ++l;
  return FastDiv{d, (uint32_t)((1ull << (31 + l)) / d + 1ull), l - 1};
}
__device__ __forceinline__ uint32_t fast_div(uint32_t i, const FastDiv& f) {
  return f.d == 1u ? i : (__umulhi(i, f.mag) >> f.sh);
}

template <typename Tin> __host__ __device__ constexpr int split_rows_pitch(int kc) { return kc | 1; }
template <typename Tin> __host__ __device__ constexpr size_t split_rows_smem(int TR, int kc) {
  return (size_t)TR * split_rows_pitch<Tin>(kc) * sizeof(Tin) + (size_t)kc * 8 + (size_t)TR * 8 + (size_t)TR * 8;
}

template <typename Tin, int TR, class Off, class W>
__global__ void __launch_bounds__(256) split_rows_kernel(const Tin* __restrict__ T, Off off, int64_t M, int64_t K,
                                                         int64_t Kp, int kc, int cs, int m_fast, W w,
                                                         float* __restrict__ amax) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int pitch = split_rows_pitch<Tin>(kc);  // odd: the row-strided staging stores spread over banks
  Tin* tile = reinterpret_cast<Tin*>(smraw);
  int64_t* offK = reinterpret_cast<int64_t*>(tile + TR * pitch);
  int64_t* offM = offK + kc;
  float* pmax = reinterpret_cast<float*>(offM + TR);
  float* rmax = pmax + TR;
  const int tid = threadIdx.x;
  const uint32_t rank = cs > 1 ? cluster_rank() : 0u;
  const int64_t m0 = (int64_t)(blockIdx.x / cs) * TR;
  const int64_t k0 = (int64_t)rank * kc;
  const int kv = (int)max((int64_t)0, min((int64_t)kc, K - k0));   // columns read
  const int kw = (int)max((int64_t)0, min((int64_t)kc, Kp - k0));  // columns written (zero padding to Kp)
  for (int i = tid; i < kv; i += 256) offK[i] = off.k(k0 + i);
  if (tid < TR) offM[tid] = m0 + tid < M ? off.m(m0 + tid) : 0;
  __syncthreads();
  if (m_fast) {  // consecutive threads on consecutive rows (the unit-stride index is in M)
    for (int e = tid; e < TR * kv; e += 256) {
      const int im = e % TR, ik = e / TR;
      Tin* d = tile + im * pitch + ik;
      if (m0 + im < M) cp_async_el(d, T + offM[im] + offK[ik]);
      else *d = Zero<Tin>::v();
    }
  } else {  // consecutive threads along a row, all threads busy however short the rows
    const FastDiv dkv = make_fastdiv((uint32_t)(kv > 0 ? kv : 1));
    for (int e = tid; e < TR * kv; e += 256) {
      const int r = (int)fast_div((uint32_t)e, dkv), c = e - r * kv;
      Tin* d = tile + r * pitch + c;
      if (m0 + r < M) cp_async_el(d, T + offM[r] + offK[c]);
      else *d = Zero<Tin>::v();
    }
  }
  cp_async_wait_all();
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  for (int r = warp; r < TR; r += 8) {
    float x = 0.f;
    for (int c = lane; c < kv; c += 32) x = fmaxf(x, absmax2(tile[r * pitch + c]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
    if (lane == 0) pmax[r] = x;
  }
  if (cs > 1) {
    cluster_sync_all();  // every CTA's partial maxima are in its shared memory
    if (tid < TR) {
      float x = 0.f;
      for (int q = 0; q < cs; ++q) x = fmaxf(x, ld_peer_f32(pmax + tid, (uint32_t)q));
      rmax[tid] = x;
    }
    cluster_arrive_relaxed();  // done reading the peers
    __syncthreads();
  } else {
    __syncthreads();
    if (tid < TR) rmax[tid] = pmax[tid];
    __syncthreads();
  }
  if (rank == 0 && tid < TR && m0 + tid < M) amax[m0 + tid] = rmax[tid];
  // columns in pairs (kc, Kp and k0 are even): 8-byte stores per plane; (row, pair) indices
  // run jointly over the threads, so short rows still keep every thread busy
  const int hw = kw / 2;
  const FastDiv dhw = make_fastdiv((uint32_t)(hw > 0 ? hw : 1));
  const int nrows = (int)min((int64_t)TR, M - m0);
  for (int e = tid; e < nrows * hw; e += 256) {
    const int r = (int)fast_div((uint32_t)e, dhw), c = 2 * (e - r * hw);
    w(m0 + r, k0 + c, c < kv ? tile[r * pitch + c] : Zero<Tin>::v(),
      c + 1 < kv ? tile[r * pitch + c + 1] : Zero<Tin>::v(), rmax[r]);
  }
  if (cs > 1) cluster_wait();  // peers may read this CTA's maxima until they have arrived
}

// Rows per cluster, cluster size and columns per CTA of the fused split, or false when a
// row of the view does not fit in 16 CTAs' shared memory (the two-kernel path runs then).
// Rows: 32, 16 or 8 (at least 16 when the rows are the unit-stride index, for 128-byte
// runs).  CTAs of at most 48 KB come first, so that four share an SM and their load,
// reduce and store phases overlap; the smallest cluster for the most rows within that
// budget wins, then the same with 112 KB (two per SM).  Columns per CTA: a multiple of 8.
constexpr int kSplitMaxCluster = 16;
template <typename Tin>
bool split_rows_shape(int64_t K, int64_t Kp, int m_fast, int* TR, int* cs, int* kc, size_t* smem) {
  const size_t budgets[2] = {48 * 1024, 112 * 1024};
  const int trs[3] = {32, 16, 8};
  for (size_t budget : budgets) {
    for (int t : trs) {
      if (m_fast && t < 16) break;
      for (int c = 1; c <= kSplitMaxCluster; ++c) {
        const int64_t k = ((Kp + c - 1) / c + 7) / 8 * 8;
        if (c > 1 && (c - 1) * k >= Kp) break;  // every rank holds columns
        const size_t b = split_rows_smem<Tin>(t, (int)k);
        if (b <= budget) {
          *TR = t;
          *cs = c;
          *kc = (int)k;
          *smem = b;
          return true;
        }
      }
    }
  }
  return false;
}

template <typename Tin, int TR, class Off, class W>
cudaError_t launch_split_rows_t(const Tin* T, const Off& off, int64_t M, int64_t K, int64_t Kp, int kc, int cs,
                                int m_fast, const W& w, float* amax, size_t smem, cudaStream_t s) {
  auto kern = split_rows_kernel<Tin, TR, Off, W>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 112 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int64_t tiles = (M + TR - 1) / TR;
  if (tiles * cs > 2147483647LL) return cudaErrorInvalidConfiguration;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(tiles * cs), 1, 1);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attrs[1];
  attrs[0].id = cudaLaunchAttributeClusterDimension;
  attrs[0].val.clusterDim.x = (unsigned)cs;
  attrs[0].val.clusterDim.y = 1;
  attrs[0].val.clusterDim.z = 1;
  cfg.attrs = attrs;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, T, off, M, K, Kp, kc, cs, m_fast, w, amax);
}

template <typename Tin, class Off, class W>
cudaError_t launch_split_rows(const Tin* T, const Off& off, int64_t M, int64_t K, int64_t Kp, int m_fast,
                              const W& w, float* amax, cudaStream_t s, bool* done) {
  static_assert(!std::is_same<Off, GrpOff>::value, "kernel parameters hold index groups by value (GrpOffV)");
  *done = false;
  const char* env = std::getenv("GTN_FUSED_SPLIT");
  if ((env && env[0] == '0') || M <= 0 || K <= 0) return cudaSuccess;
  int TR = 0, cs = 0, kc = 0;
  size_t smem = 0;
  if (!split_rows_shape<Tin>(K, Kp, m_fast, &TR, &cs, &kc, &smem)) return cudaSuccess;
  cudaError_t e;
  if (TR == 32) e = launch_split_rows_t<Tin, 32>(T, off, M, K, Kp, kc, cs, m_fast, w, amax, smem, s);
  else if (TR == 16) e = launch_split_rows_t<Tin, 16>(T, off, M, K, Kp, kc, cs, m_fast, w, amax, smem, s);
  else e = launch_split_rows_t<Tin, 8>(T, off, M, K, Kp, kc, cs, m_fast, w, amax, smem, s);
  if (e == cudaSuccess) {
    *done = true;
    return e;
  }
  // a cluster shape the device cannot schedule is a launch-configuration error (nothing ran):
  // clear it and let the caller take the two-kernel path
  if (e == cudaErrorInvalidClusterSize || e == cudaErrorInvalidConfiguration || e == cudaErrorInvalidValue ||
      e == cudaErrorLaunchOutOfResources) {
    cudaGetLastError();
    return cudaSuccess;
  }
  return e;
}

}  // namespace

cudaError_t launch_block_rowmax(const DevGatherJob* jobs, const int2* tile_map, int ntiles, const BlockBases& bases,
                                int src_is64, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  if (src_is64)
    block_rowmax_kernel<double2><<<ntiles, dim3(32, 8), 0, s>>>(jobs, tile_map, bases);
  else
    block_rowmax_kernel<float2><<<ntiles, dim3(32, 8), 0, s>>>(jobs, tile_map, bases);
  return cudaGetLastError();
}

void finish_dev_gather_job(DevGatherJob* J) {
  int tks = 0;
  while (tks < 5 && (int64_t(1) << tks) < J->Kw) ++tks;
  J->tks = tks;
  J->tiles_m = (int)((J->M + (1024 >> tks) - 1) / (1024 >> tks));
  J->m_fast = choose_m_fast(J->mg, J->kg) ? 1 : 0;
  J->fast_m = J->M < (int64_t(1) << 31) ? 1 : 0;
  for (int j = 0; j < J->mg.n; ++j) {
    const int64_t d = J->mg.dim[j];
    if (d < 1 || d >= (int64_t(1) << 31)) {
      J->fast_m = 0;
      continue;
    }
    int l = 0;
    while ((int64_t(1) << l) < d) ++l;
    if (d == 1) {
      J->m_mag[j] = 0;
      J->m_sh[j] = 0;
    } else {
      J->m_mag[j] = (uint32_t)(((uint64_t)1 << (31 + l)) / (uint64_t)d + 1);
      J->m_sh[j] = (uint32_t)(l - 1);
    }
  }
}

cudaError_t launch_block_gather(const DevGatherJob* jobs, const int2* tile_map, int ntiles, const BlockBases& bases,
                                int src_is64, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  if (src_is64)
    block_gather_kernel<double2><<<ntiles, dim3(32, 8), 0, s>>>(jobs, tile_map, bases);
  else
    block_gather_kernel<float2><<<ntiles, dim3(32, 8), 0, s>>>(jobs, tile_map, bases);
  return cudaGetLastError();
}

size_t block_band_smem(int maxn, int Kq, int nrect, int ng, int fp64) {
  const size_t e = fp64 ? sizeof(double2) : sizeof(float2);
  return (size_t)Kq * band_npad(maxn, band_npt(maxn)) * e + (size_t)nrect * ng * sizeof(int64_t) +
         (size_t)nrect * kBandRows * sizeof(int64_t) + (size_t)Kq * sizeof(DevBandCol);
}

int block_band_rows_per_pass(int) { return kBandRows; }

// Whatever the largest N of its launch (which sets the padding of B), the problem's shared
// memory stays within the launch's budget.
bool block_band_fits(int64_t N, int64_t Kq, int fp64) {
  const int nmax = fp64 ? kBandMaxN64 : kBandMaxN32;
  if (N < 1 || Kq < 1 || N > nmax || Kq > 4096) return false;
  return block_band_smem(nmax, (int)Kq, kBandMaxRects, kBandMaxGroups, fp64) <= (size_t)kBandMaxSmem;
}

namespace {
template <typename Tin, typename T, int NPT>
cudaError_t launch_band_t(const DevBand* bands, const DevBandWork* work, int nwork, const DevBandCol* cols,
                          const int64_t* rstr, const BlockBases& bases, size_t smem, cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(block_band_kernel<Tin, T, NPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kBandMaxSmem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  block_band_kernel<Tin, T, NPT><<<nwork, 256, smem, s>>>(bands, work, cols, rstr, bases);
  return cudaGetLastError();
}

template <typename Tin, typename T>
cudaError_t launch_band_n(const DevBand* bands, const DevBandWork* work, int nwork, const DevBandCol* cols,
                          const int64_t* rstr, const BlockBases& bases, int maxn, size_t smem, cudaStream_t s) {
  switch (band_npt(maxn)) {
    case 1: return launch_band_t<Tin, T, 1>(bands, work, nwork, cols, rstr, bases, smem, s);
    case 2: return launch_band_t<Tin, T, 2>(bands, work, nwork, cols, rstr, bases, smem, s);
    case 4: return launch_band_t<Tin, T, 4>(bands, work, nwork, cols, rstr, bases, smem, s);
    default: return launch_band_t<Tin, T, 8>(bands, work, nwork, cols, rstr, bases, smem, s);
  }
}
}  // namespace

cudaError_t launch_block_band(const DevBand* bands, const DevBandWork* work, int nwork, const DevBandCol* cols,
                              const int64_t* rstr, const BlockBases& bases, int src_is64, int fp64, int maxn,
                              size_t smem, cudaStream_t s) {
  if (nwork <= 0) return cudaSuccess;
  if (smem > (size_t)kBandMaxSmem || maxn > (fp64 ? kBandMaxN64 : kBandMaxN32)) return cudaErrorInvalidValue;
  if (fp64) return launch_band_n<double2, double2>(bands, work, nwork, cols, rstr, bases, maxn, smem, s);
  if (src_is64) return launch_band_n<double2, float2>(bands, work, nwork, cols, rstr, bases, maxn, smem, s);
  return launch_band_n<float2, float2>(bands, work, nwork, cols, rstr, bases, maxn, smem, s);
}

int block_split_band_rows(int Kp, int src_is64) { return split_band_tr(Kp, src_is64 ? 16 : 8); }

size_t block_split_band_smem(int Kp, int nrect, int ng, int ncol, int src_is64) {
  const int tr = block_split_band_rows(Kp, src_is64);
  const size_t e = src_is64 ? sizeof(double2) : sizeof(float2);
  return (size_t)tr * (Kp + 1) * e + (size_t)nrect * ng * sizeof(int64_t) + (size_t)nrect * tr * sizeof(int64_t) +
         (size_t)ncol * sizeof(DevBandCol);
}

namespace {
template <typename Tin, bool F16>
cudaError_t launch_split_band_t(const DevBand* bands, const DevBandWork* work, int nwork, const DevBandCol* cols,
                                const int64_t* rstr, const BlockBases& bases, size_t smem, cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(block_split_band_kernel<Tin, F16>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kBandMaxSmem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  block_split_band_kernel<Tin, F16><<<nwork, 256, smem, s>>>(bands, work, cols, rstr, bases);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_block_split_band(const DevBand* bands, const DevBandWork* work, int nwork, const DevBandCol* cols,
                                    const int64_t* rstr, const BlockBases& bases, int src_is64, int fp16,
                                    size_t smem, cudaStream_t s) {
  if (nwork <= 0) return cudaSuccess;
  if (smem > (size_t)kBandMaxSmem) return cudaErrorInvalidValue;
  if (src_is64)
    return fp16 ? launch_split_band_t<double2, true>(bands, work, nwork, cols, rstr, bases, smem, s)
                : launch_split_band_t<double2, false>(bands, work, nwork, cols, rstr, bases, smem, s);
  return fp16 ? launch_split_band_t<float2, true>(bands, work, nwork, cols, rstr, bases, smem, s)
              : launch_split_band_t<float2, false>(bands, work, nwork, cols, rstr, bases, smem, s);
}

namespace {
// out[i] = element offset of index i of an index group (its digits, innermost fastest, times
// the group's strides): the offset tables of the gathers, computed where they are used.
__global__ void offsets_table_kernel(GroupSpec g, int64_t n, int64_t* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = decompose(i, g);
}
}  // namespace

cudaError_t launch_offsets_table(const GroupSpec& g, int64_t n, int64_t* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 8);
  offsets_table_kernel<<<(unsigned)blocks, 256, 0, s>>>(g, n, out);
  return cudaGetLastError();
}

template <typename Tin, typename Tout>
static cudaError_t launch_gather_grouped_t(const GatherJob* jobs, int njobs, cudaStream_t s) {
  for (int base = 0; base < njobs; base += kGatherJobMax) {
    const int cnt = std::min(kGatherJobMax, njobs - base);
    GatherJobsP g;
    std::memset(&g, 0, sizeof(g));
    int tiles = 0;
    for (int q = 0; q < cnt; ++q) {
      const GatherJob& J = jobs[base + q];
      g.j[q] = J;
      g.tiles_m[q] = (int)((J.M + 31) / 32);
      g.m_fast[q] = choose_m_fast(J.mg, J.kg) ? 1 : 0;
      g.tile_start[q] = tiles;
      tiles += (J.M > 0 && J.Kw > 0) ? g.tiles_m[q] * (int)((J.Kw + 31) / 32) : 0;
    }
    g.tile_start[cnt] = tiles;
    g.n = cnt;
    if (tiles == 0) continue;
    gather_grouped_kernel<Tin, Tout><<<tiles, dim3(32, 8), 0, s>>>(g);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_gather_grouped(const GatherJob* jobs, int njobs, int in_is64, int out_is64, cudaStream_t s) {
  if (in_is64 && out_is64) return launch_gather_grouped_t<double2, double2>(jobs, njobs, s);
  if (in_is64) return launch_gather_grouped_t<double2, float2>(jobs, njobs, s);
  if (out_is64) return launch_gather_grouped_t<float2, double2>(jobs, njobs, s);
  return launch_gather_grouped_t<float2, float2>(jobs, njobs, s);
}

// Row maxima of every job's K-major gather (fp16 planes of grouped launches): 64 x 32 tiles,
// amax of each job zeroed first.
template <typename Tin>
__global__ void __launch_bounds__(256) rowmax_grouped_kernel(const __grid_constant__ GatherJobsP g) {
  const int b = blockIdx.x;
  const int p = find_job(g.tile_start, g.n, b);
  const GatherJob& J = g.j[p];
  const int t = b - g.tile_start[p];
  const int64_t m0 = (int64_t)(t % g.tiles_m[p]) * 64, k0 = (int64_t)(t / g.tiles_m[p]) * 32;
  rowmax_tile<Tin, GrpOff, 64, 32>(static_cast<const Tin*>(J.T), GrpOff{J.mg, J.kg}, J.M, J.K, 0,
                                   const_cast<float*>(J.amax), m0, k0);
}

template <typename Tin>
static cudaError_t launch_rowmax_grouped_t(const GatherJob* jobs, int njobs, cudaStream_t s) {
  for (int q = 0; q < njobs; ++q)
    if (jobs[q].amax && jobs[q].M > 0) {
      cudaError_t e = cudaMemsetAsync(const_cast<float*>(jobs[q].amax), 0, (size_t)jobs[q].M * sizeof(float), s);
      if (e != cudaSuccess) return e;
    }
  for (int base = 0; base < njobs; base += kGatherJobMax) {
    const int cnt = std::min(kGatherJobMax, njobs - base);
    GatherJobsP g;
    std::memset(&g, 0, sizeof(g));
    int tiles = 0, n = 0;
    for (int q = 0; q < cnt; ++q) {
      const GatherJob& J = jobs[base + q];
      if (!J.amax || J.M <= 0 || J.K <= 0) continue;
      g.j[n] = J;
      g.tiles_m[n] = (int)((J.M + 63) / 64);
      g.tile_start[n] = tiles;
      tiles += g.tiles_m[n] * (int)((J.K + 31) / 32);
      ++n;
    }
    g.tile_start[n] = tiles;
    g.n = n;
    if (tiles == 0) continue;
    rowmax_grouped_kernel<Tin><<<tiles, dim3(32, 8), 0, s>>>(g);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_rowmax_grouped(const GatherJob* jobs, int njobs, int in_is64, cudaStream_t s) {
  return in_is64 ? launch_rowmax_grouped_t<double2>(jobs, njobs, s) : launch_rowmax_grouped_t<float2>(jobs, njobs, s);
}

template <typename T>
static cudaError_t launch_small_grouped_t(const SmallJob* jobs, int njobs, cudaStream_t s) {
  for (int base = 0; base < njobs; base += kGatherJobMax) {
    const int cnt = std::min(kGatherJobMax, njobs - base);
    SmallJobsP g;
    std::memset(&g, 0, sizeof(g));
    int blocks = 0;
    size_t smem = 0;
    for (int q = 0; q < cnt; ++q) {
      const SmallJob& J = jobs[base + q];
      g.j[q] = J;
      g.blk_start[q] = blocks;
      int64_t nb = (J.M + 255) / 256;
      if (nb > 512) nb = 512;
      blocks += (int)nb;
      smem = std::max(smem, ((J.K * sizeof(int64_t) + 15) / 16) * 16 + (size_t)J.N * J.K * sizeof(T));
    }
    g.blk_start[cnt] = blocks;
    g.n = cnt;
    if (blocks == 0) continue;
    if (smem > (size_t)kSmallSmemBytes) return cudaErrorInvalidValue;
    small_grouped_kernel<T><<<blocks, 256, smem, s>>>(g);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_small_grouped(const SmallJob* jobs, int njobs, int is64, cudaStream_t s) {
  return is64 ? launch_small_grouped_t<double2>(jobs, njobs, s) : launch_small_grouped_t<float2>(jobs, njobs, s);
}

bool small_contract_fits(int K, int N, size_t elem_bytes) {
  return ((K * sizeof(int64_t) + 15) / 16) * 16 + (size_t)N * K * elem_bytes <= (size_t)kSmallSmemBytes;
}

cudaError_t launch_gather_c128_to_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg,
                                       int64_t M, int64_t K, int64_t ldo, double2* out, cudaStream_t s) {
  return launch_gather(T, mg, kg, M, K, K, ComplexWriter<double2>{out, ldo}, s);
}
cudaError_t launch_gather_c128_to_c64(const double2* T, const GroupSpec& mg, const GroupSpec& kg,
                                      int64_t M, int64_t K, int64_t ldo, float2* out, cudaStream_t s) {
  return launch_gather(T, mg, kg, M, K, K, ComplexWriter<float2>{out, ldo}, s);
}
cudaError_t launch_gather_c64_to_c64(const float2* T, const GroupSpec& mg, const GroupSpec& kg,
                                     int64_t M, int64_t K, int64_t ldo, float2* out, cudaStream_t s) {
  return launch_gather(T, mg, kg, M, K, K, ComplexWriter<float2>{out, ldo}, s);
}
cudaError_t launch_gather_c64_to_c128(const float2* T, const GroupSpec& mg, const GroupSpec& kg,
                                      int64_t M, int64_t K, int64_t ldo, double2* out, cudaStream_t s) {
  return launch_gather(T, mg, kg, M, K, K, ComplexWriter<double2>{out, ldo}, s);
}
cudaError_t launch_split_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M,
                              int64_t K, int64_t Kp, int nplanes, int64_t pstride,
                              __nv_bfloat16* out, cudaStream_t s) {
  return launch_gather(T, mg, kg, M, K, Kp, SplitWriter{out, 2 * Kp, pstride, nplanes}, s);
}
cudaError_t launch_split_c64(const float2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M,
                             int64_t K, int64_t Kp, int nplanes, int64_t pstride,
                             __nv_bfloat16* out, cudaStream_t s) {
  return launch_gather(T, mg, kg, M, K, Kp, SplitWriter{out, 2 * Kp, pstride, nplanes}, s);
}
template <typename Tin, class Off>
static cudaError_t launch_rowmax(const Tin* T, const Off& off, int m_fast, int64_t M, int64_t K, float* amax,
                                 cudaStream_t s) {
  static_assert(!std::is_same<Off, GrpOff>::value, "kernel parameters hold index groups by value (GrpOffV)");
  if (M <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(amax, 0, (size_t)M * sizeof(float), s);
  if (e != cudaSuccess || K <= 0) return e;
  if (m_fast) {
    const int64_t gx = (M + 255) / 256, gy = (K + 7) / 8;
    if (gy > 65535 || gx > 2147483647LL) return cudaErrorInvalidConfiguration;
    rowmax_kernel<Tin, Off, 256, 8><<<dim3((unsigned)gx, (unsigned)gy), dim3(32, 8), 0, s>>>(T, off, M, K, m_fast,
                                                                                           amax);
  } else {
    const int64_t gx = (M + 63) / 64, gy = (K + 31) / 32;
    if (gy > 65535 || gx > 2147483647LL) return cudaErrorInvalidConfiguration;
    rowmax_kernel<Tin, Off, 64, 32><<<dim3((unsigned)gx, (unsigned)gy), dim3(32, 8), 0, s>>>(T, off, M, K, m_fast,
                                                                                           amax);
  }
  return cudaGetLastError();
}
cudaError_t launch_rowmax_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                               float* amax, cudaStream_t s) {
  return launch_rowmax(T, GrpOffV{mg, kg}, choose_m_fast(mg, kg) ? 1 : 0, M, K, amax, s);
}
cudaError_t launch_rowmax_c64(const float2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                              float* amax, cudaStream_t s) {
  return launch_rowmax(T, GrpOffV{mg, kg}, choose_m_fast(mg, kg) ? 1 : 0, M, K, amax, s);
}

// ---- table-driven variants (offsets precomputed per plan step) --------------------------
bool gather_m_fast(const GroupSpec& mg, const GroupSpec& kg) { return choose_m_fast(mg, kg); }
cudaError_t launch_rowmax_tab(const void* T, int is64, const GatherTab& t, int64_t M, int64_t K, float* amax,
                              cudaStream_t s) {
  const TabOff off{t.om, t.ok};
  return is64 ? launch_rowmax(static_cast<const double2*>(T), off, t.m_fast, M, K, amax, s)
              : launch_rowmax(static_cast<const float2*>(T), off, t.m_fast, M, K, amax, s);
}
cudaError_t launch_split_tab(const void* T, int is64, const GatherTab& t, int64_t M, int64_t K, int64_t Kp,
                             int nplanes, int64_t pstride, __nv_bfloat16* out, cudaStream_t s) {
  const SplitWriter w{out, 2 * Kp, pstride, nplanes};
  return is64 ? launch_gather_tab(static_cast<const double2*>(T), t.om, t.ok, M, K, Kp, t.m_fast, w, s)
              : launch_gather_tab(static_cast<const float2*>(T), t.om, t.ok, M, K, Kp, t.m_fast, w, s);
}
cudaError_t launch_split16_tab(const void* T, int is64, const GatherTab& t, int64_t M, int64_t K, int64_t Kp,
                               int64_t pstride, const float* amax, __nv_bfloat16* out, cudaStream_t s) {
  const Split16Writer w{reinterpret_cast<__half*>(out), 2 * Kp, pstride, amax};
  return is64 ? launch_gather_tab(static_cast<const double2*>(T), t.om, t.ok, M, K, Kp, t.m_fast, w, s)
              : launch_gather_tab(static_cast<const float2*>(T), t.om, t.ok, M, K, Kp, t.m_fast, w, s);
}
// Fused one-pass split (row maxima through cluster shared memory), table or group offsets;
// *done = false when the view's rows do not fit (the caller runs rowmax + split instead).
cudaError_t launch_split16_rows_tab(const void* T, int is64, const GatherTab& t, int64_t M, int64_t K, int64_t Kp,
                                    int64_t pstride, float* amax, __nv_bfloat16* out, cudaStream_t s, bool* done) {
  const Split16RowWriter w{reinterpret_cast<__half*>(out), 2 * Kp, pstride};
  const TabOff off{t.om, t.ok};
  return is64 ? launch_split_rows(static_cast<const double2*>(T), off, M, K, Kp, t.m_fast, w, amax, s, done)
              : launch_split_rows(static_cast<const float2*>(T), off, M, K, Kp, t.m_fast, w, amax, s, done);
}
cudaError_t launch_split16_rows_grp(const void* T, int is64, const GroupSpec& mg, const GroupSpec& kg, int64_t M,
                                    int64_t K, int64_t Kp, int64_t pstride, float* amax, __nv_bfloat16* out,
                                    cudaStream_t s, bool* done) {
  const Split16RowWriter w{reinterpret_cast<__half*>(out), 2 * Kp, pstride};
  const GrpOffV off{mg, kg};
  const int mf = choose_m_fast(mg, kg) ? 1 : 0;
  return is64 ? launch_split_rows(static_cast<const double2*>(T), off, M, K, Kp, mf, w, amax, s, done)
              : launch_split_rows(static_cast<const float2*>(T), off, M, K, Kp, mf, w, amax, s, done);
}
cudaError_t launch_split_i7_rows_tab(const double2* T, const GatherTab& t, int64_t M, int64_t K, int64_t Kp,
                                     int64_t pstride, float* amax, __nv_bfloat16* out, cudaStream_t s, bool* done) {
  return launch_split_rows(T, TabOff{t.om, t.ok}, M, K, Kp, t.m_fast, Int7RowWriter{out, 2 * Kp, pstride}, amax, s,
                           done);
}
cudaError_t launch_split_i7_rows_grp(const double2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                                     int64_t Kp, int64_t pstride, float* amax, __nv_bfloat16* out, cudaStream_t s,
                                     bool* done) {
  return launch_split_rows(T, GrpOffV{mg, kg}, M, K, Kp, choose_m_fast(mg, kg) ? 1 : 0,
                           Int7RowWriter{out, 2 * Kp, pstride}, amax, s, done);
}
cudaError_t launch_split_i7_tab(const double2* T, const GatherTab& t, int64_t M, int64_t K, int64_t Kp,
                               int64_t pstride, const float* amax, __nv_bfloat16* out, cudaStream_t s) {
  const Int7Writer w{out, 2 * Kp, pstride, amax};
  return launch_gather_tab(T, t.om, t.ok, M, K, Kp, t.m_fast, w, s);
}
cudaError_t launch_split_i7_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                                 int64_t Kp, int64_t pstride, const float* amax, __nv_bfloat16* out, cudaStream_t s) {
  const Int7Writer w{out, 2 * Kp, pstride, amax};
  return launch_gather(T, mg, kg, M, K, Kp, w, s);
}
cudaError_t launch_pack_b_planes_i7(const double2* B, int64_t N, int64_t K, int64_t Kp, int64_t pstride,
                                    __nv_bfloat16* out, float* bmax, cudaStream_t s) {
  if (N <= 0) return cudaSuccess;
  if (N > 2147483647LL) return cudaErrorInvalidConfiguration;
  bmax_kernel<<<(unsigned)N, 256, 0, s>>>(B, K, bmax);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int64_t total = 2 * N * Kp;
  int64_t blocks = std::min<int64_t>(std::max<int64_t>((total + 255) / 256, 1), 152 * 32);
  pack_b_planes_i7_kernel<<<(unsigned)blocks, 256, 0, s>>>(B, N, K, Kp, pstride, bmax, out);
  return cudaGetLastError();
}
cudaError_t launch_gather_tab_to_c128(const void* T, int is64, const GatherTab& t, int64_t M, int64_t K, int64_t ldo,
                                      double2* out, cudaStream_t s) {
  const ComplexWriter<double2> w{out, ldo};
  return is64 ? launch_gather_tab(static_cast<const double2*>(T), t.om, t.ok, M, K, K, t.m_fast, w, s)
              : launch_gather_tab(static_cast<const float2*>(T), t.om, t.ok, M, K, K, t.m_fast, w, s);
}
cudaError_t launch_split16_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                                int64_t Kp, int64_t pstride, const float* amax, __nv_bfloat16* out, cudaStream_t s) {
  return launch_gather(T, mg, kg, M, K, Kp, Split16Writer{reinterpret_cast<__half*>(out), 2 * Kp, pstride, amax}, s);
}
cudaError_t launch_split16_c64(const float2* T, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K,
                               int64_t Kp, int64_t pstride, const float* amax, __nv_bfloat16* out, cudaStream_t s) {
  return launch_gather(T, mg, kg, M, K, Kp, Split16Writer{reinterpret_cast<__half*>(out), 2 * Kp, pstride, amax}, s);
}
cudaError_t launch_pack_b_planes_f16(const double2* B, int64_t N, int64_t K, int64_t Kp, int64_t pstride,
                                     __nv_bfloat16* out, float* bmax, cudaStream_t s) {
  if (N <= 0) return cudaSuccess;
  if (N > 2147483647LL) return cudaErrorInvalidConfiguration;
  bmax_kernel<<<(unsigned)N, 256, 0, s>>>(B, K, bmax);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int64_t total = 2 * N * Kp;
  int64_t blocks = std::min<int64_t>(std::max<int64_t>((total + 255) / 256, 1), 152 * 32);
  pack_b_planes_f16_kernel<<<(unsigned)blocks, 256, 0, s>>>(B, N, K, Kp, pstride, bmax, reinterpret_cast<__half*>(out));
  return cudaGetLastError();
}
cudaError_t launch_pack_b_planes(const double2* B, int64_t N, int64_t K, int64_t Kp, int nplanes,
                                 int64_t pstride, __nv_bfloat16* out, cudaStream_t s) {
  const int64_t total = 2 * N * Kp;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (blocks < 1) blocks = 1;
  pack_b_planes_kernel<<<(unsigned)blocks, 256, 0, s>>>(B, N, K, Kp, nplanes, pstride, out);
  return cudaGetLastError();
}
cudaError_t launch_small_contract_c128(const double2* T, const GroupSpec& mg, const GroupSpec& kg,
                                       int64_t M, int K, int N, const double2* B, double2* C,
                                       cudaStream_t s) {
  return launch_small(T, mg, kg, M, K, N, B, C, s);
}
cudaError_t launch_small_contract_c64(const float2* T, const GroupSpec& mg, const GroupSpec& kg,
                                      int64_t M, int K, int N, const float2* B, float2* C,
                                      cudaStream_t s) {
  return launch_small(T, mg, kg, M, K, N, B, C, s);
}
