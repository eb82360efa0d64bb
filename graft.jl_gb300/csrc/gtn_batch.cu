// Batched application of many independent maps: step s of every map runs in one grouped
// launch per kernel kind (grouped small-K contraction, grouped gather/split, grouped
// tcgen05 or SIMT GEMM, grouped output permutation).  A batch object can capture the
// whole application once into a CUDA graph and replay it (the reference's many small maps
// of a sweep, lib/GraftContractions/src/Contractions/effective.jl:26-30,153-165, become one
// graph launch).
#include "gtn_internal.h"

#include <algorithm>
#include <cstring>
#include <new>

namespace {

bool is_tc_prec(int p) { return p == GTN_PREC_BF16X6 || p == GTN_PREC_BF16X3 || p == GTN_PREC_FP16X3; }
int planes_of(int p) { return p == GTN_PREC_BF16X6 ? 3 : 2; }

void flat_groups(int64_t n, GroupSpec* mg, GroupSpec* kg, int64_t* M, int64_t* K) {
  std::memset(mg, 0, sizeof(*mg));
  std::memset(kg, 0, sizeof(*kg));
  if (n % 32 == 0 && n >= 32) {
    *M = n / 32;
    *K = 32;
    mg->n = 1; mg->dim[0] = *M; mg->str[0] = 32;
    kg->n = 1; kg->dim[0] = 32; kg->str[0] = 1;
  } else {
    *M = n;
    *K = 1;
    mg->n = 1; mg->dim[0] = n; mg->str[0] = 1;
  }
}

}  // namespace

int map_run_batched(gtn_map* maps_in, int n, int precision, const double2* const* xs, double2* const* ys) {
  if (n <= 0) return GTN_OK;
  gtn_ctx ctx = maps_in[0]->ctx;
  cudaStream_t s = ctx->stream;
  std::vector<gtn_map> maps(n);
  for (int i = 0; i < n; ++i) {
    gtn_map m = maps_in[i];
    if (m->ctx != ctx) return set_err(ctx, GTN_ERR_INVALID, "batched maps must share one context");
    maps[i] = (precision == GTN_PREC_FP64 && m->fp64_alt) ? m->fp64_alt : m;
  }
  const bool fp64 = precision == GTN_PREC_FP64;
  const bool f16 = precision == GTN_PREC_FP16X3;
  const bool tc = is_tc_prec(precision);
  const int P = tc ? planes_of(precision) : 0;
  if (tc)
    for (gtn_map m : maps)
      for (auto& st : m->steps)
        if (!st.small && (!st.bpl || st.bplanes != P || st.bfp16 != (f16 ? 1 : 0) || (f16 && !m->amax)))
          return set_err(ctx, GTN_ERR_INVALID, "a batched map was not created for this tcgen05 precision");
  std::vector<const void*> cur(n);
  std::vector<bool> cur64(n, true);
  size_t max_steps = 0;
  for (int i = 0; i < n; ++i) {
    cur[i] = xs[i];
    max_steps = std::max(max_steps, maps[i]->steps.size());
  }
  cudaError_t e = cudaSuccess;
  std::string why;
  // FP32 kernels read complex FP32: convert inputs whose first step needs it (one launch)
  if (!fp64) {
    std::vector<GatherJob> conv;
    for (int i = 0; i < n; ++i) {
      const PlanStep& st0 = maps[i]->steps[0];
      if (st0.small || !tc) {
        GatherJob J;
        std::memset(&J, 0, sizeof(J));
        flat_groups(maps[i]->x_elems, &J.mg, &J.kg, &J.M, &J.K);
        J.T = cur[i];
        J.Kw = J.K;
        J.out = maps[i]->buf1;
        J.ld = J.K;
        conv.push_back(J);
        cur[i] = maps[i]->buf1;
        cur64[i] = false;
      }
    }
    if (!conv.empty()) {
      e = launch_gather_grouped(conv.data(), (int)conv.size(), 1, 0, s);
      ctx->launches += (int64_t)((conv.size() + kGatherJobMax - 1) / kGatherJobMax);
      if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("batched convert: ") + cudaGetErrorString(e));
    }
  }
  for (size_t si = 0; si < max_steps; ++si) {
    std::vector<SmallJob> small;
    std::vector<GatherJob> gath[2];  // by input type (0: c64, 1: c128)
    std::vector<GemmJob> gemm;
    std::vector<TcGemmArgs> tcp;
    std::vector<void*> outs(n, nullptr);
    for (int i = 0; i < n; ++i) {
      gtn_map m = maps[i];
      if (si >= m->steps.size()) continue;
      const PlanStep& st = m->steps[si];
      void* out = (si & 1) ? m->buf1 : m->buf0;
      if (out == cur[i]) out = (out == m->buf0) ? m->buf1 : m->buf0;
      outs[i] = out;
      if (st.small) {
        SmallJob J;
        J.A = cur[i];
        J.mg = st.mg;
        J.kg = st.kg;
        J.M = st.M;
        J.K = (int)st.K;
        J.N = (int)st.N;
        J.B = fp64 ? static_cast<const void*>(st.b64) : static_cast<const void*>(st.b32);
        J.C = out;
        small.push_back(J);
        continue;
      }
      GatherJob G;
      std::memset(&G, 0, sizeof(G));
      G.T = cur[i];
      G.mg = st.mg;
      G.kg = st.kg;
      G.M = st.M;
      G.K = st.K;
      G.out = m->abuf;
      if (tc) {
        G.Kw = st.Kp;
        G.ld = st.Kp;
        G.nplanes = P;
        G.pstride = st.M * 2 * st.Kp;
        TcGemmArgs a;
        a.A = static_cast<const __nv_bfloat16*>(m->abuf);
        a.B = st.bpl;
        a.C = static_cast<float2*>(out);
        a.M = st.M;
        a.N = st.N;
        a.Kp = st.Kp;
        a.a_planes = P;
        a.b_planes = P;
        if (f16) {  // fp16 planes: rows of A scaled by their maxima, complex rows of B by theirs
          G.amax = m->amax;
          a.fp16 = 1;
          a.a_max = m->amax;
          a.b_max = st.bmax;
        }
        if (P == 3) {
          const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
          a.nprod = 6;
          for (int q = 0; q < 6; ++q) { a.prod_a[q] = pa[q]; a.prod_b[q] = pb[q]; }
        } else {
          const int pa[3] = {1, 0, 0}, pb[3] = {0, 1, 0};
          a.nprod = 3;
          for (int q = 0; q < 3; ++q) { a.prod_a[q] = pa[q]; a.prod_b[q] = pb[q]; }
        }
        tcp.push_back(a);
      } else {
        G.Kw = st.K;
        G.ld = st.K;
        GemmJob J;
        J.A = m->abuf;
        J.B = fp64 ? static_cast<const void*>(st.b64) : static_cast<const void*>(st.b32);
        J.C = out;
        J.M = st.M;
        J.N = st.N;
        J.K = st.K;
        gemm.push_back(J);
      }
      gath[cur64[i] ? 1 : 0].push_back(G);
    }
    if (!small.empty()) {
      e = launch_small_grouped(small.data(), (int)small.size(), fp64 ? 1 : 0, s);
      ctx->launches += (int64_t)((small.size() + kGatherJobMax - 1) / kGatherJobMax);
    }
    if (f16)
      for (int t = 0; t < 2 && e == cudaSuccess; ++t)
        if (!gath[t].empty()) {
          e = launch_rowmax_grouped(gath[t].data(), (int)gath[t].size(), t, s);
          ctx->launches += (int64_t)((gath[t].size() + kGatherJobMax - 1) / kGatherJobMax);
        }
    for (int t = 0; t < 2 && e == cudaSuccess; ++t)
      if (!gath[t].empty()) {
        e = launch_gather_grouped(gath[t].data(), (int)gath[t].size(), t, fp64 ? 1 : 0, s);
        ctx->launches += (int64_t)((gath[t].size() + kGatherJobMax - 1) / kGatherJobMax);
      }
    if (e == cudaSuccess && !gemm.empty()) {
      e = launch_gemm_simt_grouped(gemm.data(), (int)gemm.size(), fp64 ? 1 : 0, s);
      ctx->launches += (int64_t)((gemm.size() + kGemmJobMax - 1) / kGemmJobMax);
    }
    if (e == cudaSuccess && !tcp.empty()) {
      std::stable_sort(tcp.begin(), tcp.end(), [](const TcGemmArgs& a, const TcGemmArgs& b) { return a.Kp > b.Kp; });
      e = launch_tc_gemm_grouped(tcp.data(), (int)tcp.size(), ctx->d_errflag, s, &why);
      ctx->launches += (int64_t)((tcp.size() + 55) / 56);
    }
    if (e != cudaSuccess)
      return set_err(ctx, GTN_ERR_CUDA, "batched step " + std::to_string(si) + ": " + why + " " + cudaGetErrorString(e));
    for (int i = 0; i < n; ++i)
      if (outs[i]) {
        cur[i] = outs[i];
        if (!fp64) cur64[i] = false;
      }
  }
  // outputs (one launch per input type)
  std::vector<GatherJob> fin[2];
  for (int i = 0; i < n; ++i) {
    gtn_map m = maps[i];
    GatherJob G;
    std::memset(&G, 0, sizeof(G));
    G.T = cur[i];
    G.mg = m->fin_mg;
    G.kg = m->fin_kg;
    G.M = m->fin_M;
    G.K = m->fin_K;
    G.Kw = m->fin_K;
    G.out = ys[i];
    G.ld = m->fin_K;
    fin[cur64[i] ? 1 : 0].push_back(G);
  }
  for (int t = 0; t < 2 && e == cudaSuccess; ++t)
    if (!fin[t].empty()) {
      e = launch_gather_grouped(fin[t].data(), (int)fin[t].size(), t, 1, s);
      ctx->launches += (int64_t)((fin[t].size() + kGatherJobMax - 1) / kGatherJobMax);
    }
  if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("batched output: ") + cudaGetErrorString(e));
  return GTN_OK;
}

struct gtn_batch_s {
  gtn_ctx ctx = nullptr;
  std::vector<gtn_map> maps;
  std::vector<const double2*> xs;
  std::vector<double2*> ys;
  int precision = 0;
  bool use_graph = false;
  int runs = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t launches_per_run = 0;
};

extern "C" {

int gtn_map_apply_batched(int n, const gtn_map* maps, const void* const* xs, void* const* ys, int precision) {
  if (n <= 0 || !maps || !xs || !ys || !maps[0]) return GTN_ERR_INVALID;
  std::vector<gtn_map> ms(maps, maps + n);
  return map_run_batched(ms.data(), n, precision, reinterpret_cast<const double2* const*>(xs),
                         reinterpret_cast<double2* const*>(ys));
}

int gtn_batch_create(int n, const gtn_map* maps, const void* const* xs, void* const* ys, int precision,
                     int use_graph, gtn_batch* out) {
  if (n <= 0 || !maps || !xs || !ys || !out || !maps[0]) return GTN_ERR_INVALID;
  gtn_batch b = new (std::nothrow) gtn_batch_s();
  if (!b) return GTN_ERR_MEMORY;
  b->ctx = maps[0]->ctx;
  b->maps.assign(maps, maps + n);
  for (int i = 0; i < n; ++i) {
    b->xs.push_back(static_cast<const double2*>(xs[i]));
    b->ys.push_back(static_cast<double2*>(ys[i]));
  }
  b->precision = precision;
  b->use_graph = use_graph != 0;
  *out = b;
  return GTN_OK;
}

int gtn_batch_run(gtn_batch b) {
  if (!b) return GTN_ERR_INVALID;
  gtn_ctx ctx = b->ctx;
  const int n = (int)b->maps.size();
  // first run eager (sets kernel attributes, validates); the second run is captured
  if (!b->use_graph || b->runs == 0) {
    const int64_t l0 = ctx->launches;
    int st = map_run_batched(b->maps.data(), n, b->precision, b->xs.data(), b->ys.data());
    b->launches_per_run = ctx->launches - l0;
    b->runs++;
    return st;
  }
  if (!b->exec) {
    // capture on a private stream (the caller's stream may be the legacy default stream,
    // which cannot be captured), then replay on the context's stream
    cudaStream_t cs = nullptr;
    GTN_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    GTN_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    cudaError_t be = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (be != cudaSuccess) {
      cudaStreamDestroy(cs);
      return set_err(ctx, GTN_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(be));
    }
    cudaStream_t saved = ctx->stream;
    ctx->stream = cs;
    const int64_t l0 = ctx->launches;
    int st = map_run_batched(b->maps.data(), n, b->precision, b->xs.data(), b->ys.data());
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &g);
    ctx->stream = saved;
    cudaStreamDestroy(cs);
    ctx->launches = l0;
    if (st != GTN_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    b->graph = g;
    GTN_CUDA_TRY(ctx, cudaGraphInstantiate(&b->exec, g, 0));
  }
  GTN_CUDA_TRY(ctx, cudaGraphLaunch(b->exec, ctx->stream));
  ctx->launches += b->launches_per_run;
  b->runs++;
  return GTN_OK;
}

int gtn_batch_destroy(gtn_batch b) {
  if (!b) return GTN_ERR_INVALID;
  cudaStreamSynchronize(b->ctx->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  delete b;
  return GTN_OK;
}

}  // extern "C"
