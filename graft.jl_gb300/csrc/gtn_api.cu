// C ABI entry points: contexts, maps, one-shot contractions, permutations and vector helpers.
#include "gtn_internal.h"

#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>

namespace {
// The message of the last failure on each host thread, with the context it belongs to.
// gtn_last_error reads this copy on the thread that made the failing call, so a call
// refused on one thread (a busy map) never races with a message written on another.
thread_local std::string t_err;
thread_local const void* t_err_ctx = nullptr;
}  // namespace

int set_err(gtn_ctx ctx, int code, const std::string& msg) {
  if (ctx) {
    t_err = msg;
    t_err_ctx = ctx;
    std::lock_guard<std::mutex> lock(ctx->err_mu);
    ctx->err = msg;
  }
  return code;
}

cudaError_t ctx_workspace(gtn_ctx ctx, size_t bytes, void** out) {
  if (bytes > ctx->ws_bytes) {
    if (ctx->ws) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(ctx->ws);
      ctx->ws = nullptr;
      ctx->ws_bytes = 0;
    }
    const size_t want = bytes + bytes / 4;
    cudaError_t e = cudaMalloc(&ctx->ws, want);
    if (e != cudaSuccess) return e;
    ctx->ws_bytes = want;
  }
  *out = ctx->ws;
  return cudaSuccess;
}

// Block sizes: 256-byte multiples below 1 MiB, 1 MiB multiples above; a cached block is
// reused for a request of at least half its size; the cache holds at most 4 GiB.
constexpr size_t kBlkCacheMax = size_t(4) << 30;

cudaError_t ctx_blk_alloc(gtn_ctx ctx, size_t bytes, void** out, size_t* got) {
  size_t sz = bytes < 256 ? 256 : bytes;
  sz = sz < (size_t(1) << 20) ? (sz + 255) / 256 * 256 : (sz + (size_t(1) << 20) - 1) >> 20 << 20;
  auto it = ctx->blk_free.lower_bound(sz);
  if (it != ctx->blk_free.end() && it->first <= 2 * sz) {
    *out = it->second;
    *got = it->first;
    ctx->blk_cached -= it->first;
    ctx->blk_free.erase(it);
    return cudaSuccess;
  }
  cudaError_t e = cudaMalloc(out, sz);
  if (e != cudaSuccess && !ctx->blk_free.empty()) {  // memory held by the cache: give it back, retry
    cudaGetLastError();
    ctx_blk_flush(ctx);
    e = cudaMalloc(out, sz);
  }
  *got = e == cudaSuccess ? sz : 0;
  return e;
}

void ctx_blk_release(gtn_ctx ctx, void* p, size_t bytes) {
  if (!p) return;
  if (ctx->blk_cached + bytes > kBlkCacheMax) {
    cudaFree(p);
    return;
  }
  ctx->blk_free.emplace(bytes, p);
  ctx->blk_cached += bytes;
}

void ctx_blk_flush(gtn_ctx ctx) {
  if (ctx->blk_free.empty()) return;
  cudaStreamSynchronize(ctx->stream);
  for (auto& kv : ctx->blk_free) cudaFree(kv.second);
  ctx->blk_free.clear();
  ctx->blk_cached = 0;
}

cudaError_t ctx_red(gtn_ctx ctx, size_t n2) {
  if (n2 > ctx->red_cap) {
    if (ctx->d_red) cudaFree(ctx->d_red);
    ctx->d_red = nullptr;
    cudaError_t e = cudaMalloc(&ctx->d_red, n2 * sizeof(double2));
    if (e != cudaSuccess) return e;
    ctx->red_cap = n2;
  }
  if (!ctx->h_red) {
    cudaError_t e = cudaMallocHost(&ctx->h_red, 256 * sizeof(double2));
    if (e != cudaSuccess) return e;
    ctx->hred_cap = 256;
  }
  return cudaSuccess;
}

MapUse::MapUse(gtn_map_s* map) : m(map), ok(map != nullptr && map->busy.exchange(1) == 0) {}
MapUse::~MapUse() {
  if (ok) m->busy.store(0);
}

int map_busy_error(gtn_map_s* map) {
  return set_err(map->ctx, GTN_ERR_INVALID,
                 "map is in use by another call: a map is not reentrant (one map per host thread)");
}

extern "C" {

int gtn_ctx_create(int device, gtn_ctx* out) {
  if (!out) return GTN_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GTN_ERR_CUDA;
  if (device < 0 || device >= ndev) return GTN_ERR_INVALID;
  gtn_ctx ctx = new (std::nothrow) gtn_ctx_s();
  if (!ctx) return GTN_ERR_MEMORY;
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return GTN_ERR_CUDA; }
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  ctx->sm_count = prop.multiProcessorCount;
  ctx->cc_major = prop.major;
  ctx->cc_minor = prop.minor;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return GTN_ERR_CUDA;
  }
  ctx->own_stream = true;
  if (cudaMalloc(&ctx->d_errflag, sizeof(int)) != cudaSuccess ||
      cudaMemset(ctx->d_errflag, 0, sizeof(int)) != cudaSuccess) {
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GTN_ERR_CUDA;
  }
  if (ctx_red(ctx, 4096) != cudaSuccess) {
    cudaFree(ctx->d_errflag);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GTN_ERR_CUDA;
  }
  *out = ctx;
  return GTN_OK;
}

int gtn_ctx_destroy(gtn_ctx ctx) {
  if (!ctx) return GTN_ERR_INVALID;
  cudaStreamSynchronize(ctx->stream);
  linalg_release(ctx);
  ctx_blk_flush(ctx);
  if (ctx->ws) cudaFree(ctx->ws);
  if (ctx->carena) cudaFree(ctx->carena);
  if (ctx->d_red) cudaFree(ctx->d_red);
  if (ctx->h_red) cudaFreeHost(ctx->h_red);
  if (ctx->d_errflag) cudaFree(ctx->d_errflag);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GTN_OK;
}

int gtn_ctx_set_stream(gtn_ctx ctx, void* stream) {
  if (!ctx) return GTN_ERR_INVALID;
  cudaStreamSynchronize(ctx->stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  ctx->stream = static_cast<cudaStream_t>(stream);
  ctx->own_stream = false;
  return GTN_OK;
}

void* gtn_ctx_stream(gtn_ctx ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

int gtn_ctx_set_linalg_precision(gtn_ctx ctx, int precision) {
  if (!ctx) return GTN_ERR_INVALID;
  if (precision != GTN_PREC_FP64 && precision != GTN_PREC_FP64E)
    return set_err(ctx, GTN_ERR_INVALID, "linalg precision: GTN_PREC_FP64 or GTN_PREC_FP64E");
  if (precision == GTN_PREC_FP64E && !tc_gemm_supported(ctx->cc_major, ctx->cc_minor))
    return set_err(ctx, GTN_ERR_UNSUPPORTED, "GTN_PREC_FP64E needs an sm_10x device");
  ctx->linalg_prec = precision;
  return GTN_OK;
}

int gtn_ctx_linalg_precision(gtn_ctx ctx) { return ctx ? ctx->linalg_prec : -1; }

const char* gtn_last_error(gtn_ctx ctx) {
  if (!ctx) return "null context";
  if (t_err_ctx == ctx) return t_err.c_str();
  std::lock_guard<std::mutex> lock(ctx->err_mu);
  return ctx->err.c_str();
}

int64_t gtn_ctx_launch_count(gtn_ctx ctx) { return ctx ? ctx->launches : -1; }

int gtn_ctx_sync(gtn_ctx ctx) {
  if (!ctx) return GTN_ERR_INVALID;
  GTN_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  int flag = 0;
  GTN_CUDA_TRY(ctx, cudaMemcpy(&flag, ctx->d_errflag, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag != 0) {
    cudaMemset(ctx->d_errflag, 0, sizeof(int));
    return set_err(ctx, GTN_ERR_TIMEOUT, "device wait timed out (code " + std::to_string(flag) + ")");
  }
  return GTN_OK;
}

int gtn_map_create(gtn_ctx ctx, int n_operands, const int* ranks, const int64_t* dims,
                   const int* labels, const int* conj, const int* order,
                   const void* const* statics, int precision, gtn_map* out) {
  if (!ctx || !out || !ranks || !dims || !labels || !order) return set_err(ctx, GTN_ERR_INVALID, "null argument");
  *out = nullptr;
  gtn_map map = new (std::nothrow) gtn_map_s();
  if (!map) return set_err(ctx, GTN_ERR_MEMORY, "host allocation failed");
  const int st = plan_build(ctx, n_operands, ranks, dims, labels, conj, order, statics, precision, map);
  if (st != GTN_OK) {
    cudaStreamSynchronize(ctx->stream);
    map_free(map);
    delete map;
    return st;
  }
  *out = map;
  return GTN_OK;
}

int gtn_map_destroy(gtn_map map) {
  if (!map) return GTN_ERR_INVALID;
  // claim the map so that no call can start on it between this check and the free
  if (map->busy.exchange(1) != 0) return map_busy_error(map);
  if (map->ctx) cudaStreamSynchronize(map->ctx->stream);
  map_free(map);
  delete map;
  return GTN_OK;
}

int gtn_map_set_fp64(gtn_map map, gtn_map fp64_map) {
  if (!map) return GTN_ERR_INVALID;
  if (fp64_map) {
    if (fp64_map == map || fp64_map->ctx != map->ctx || fp64_map->x_elems != map->x_elems ||
        fp64_map->y_elems != map->y_elems || fp64_map->fp64_map)
      return set_err(map->ctx, GTN_ERR_INVALID, "gtn_map_set_fp64: a different map of the same shape and context");
    if (fp64_map->precision != GTN_PREC_FP64 && fp64_map->precision != GTN_PREC_FP64E)
      return set_err(map->ctx, GTN_ERR_INVALID, "gtn_map_set_fp64: the map must be FP64 or FP64-grade");
  }
  map->fp64_map = fp64_map;
  return GTN_OK;
}

int gtn_map_apply_prec(gtn_map map, int precision, const void* x, void* y) {
  if (!map || !x || !y) return GTN_ERR_INVALID;
  MapUse use(map);
  if (!use.ok) return map_busy_error(map);
  return map_run(map, precision, static_cast<const double2*>(x), static_cast<double2*>(y));
}

int gtn_map_apply(gtn_map map, const void* x, void* y) {
  if (!map) return GTN_ERR_INVALID;
  return gtn_map_apply_prec(map, map->precision, x, y);
}

int gtn_map_apply_profiled(gtn_map map, int precision, const void* x, void* y, int cap, double* ms,
                           int* kind, double* flops, int* count) {
  if (!map || !x || !y || !ms || !kind || !flops || !count) return GTN_ERR_INVALID;
  MapUse use(map);
  if (!use.ok) return map_busy_error(map);
  return map_run_profiled(map, precision, static_cast<const double2*>(x), static_cast<double2*>(y), cap, ms,
                          kind, flops, count);
}

int gtn_map_apply_host(gtn_map map, const void* x_host, void* y_host) {
  if (!map || !x_host || !y_host) return GTN_ERR_INVALID;
  MapUse use(map);
  if (!use.ok) return map_busy_error(map);
  gtn_ctx ctx = map->ctx;
  if (!map->dx) {
    if (cudaMalloc(&map->dx, map->x_elems * sizeof(double2)) != cudaSuccess ||
        cudaMalloc(&map->dy, map->y_elems * sizeof(double2)) != cudaSuccess)
      return set_err(ctx, GTN_ERR_MEMORY, "host-apply staging allocation failed");
    map->owned.push_back(map->dx);
    map->owned.push_back(map->dy);
  }
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(map->dx, x_host, map->x_elems * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
  int st = map_run(map, map->precision, static_cast<const double2*>(map->dx), static_cast<double2*>(map->dy));
  if (st != GTN_OK) return st;
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(y_host, map->dy, map->y_elems * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
  return gtn_ctx_sync(ctx);
}

int gtn_map_info(gtn_map map, int64_t* x_elems, int64_t* y_elems, double* flops, int* n_steps,
                 int64_t* bytes) {
  if (!map) return GTN_ERR_INVALID;
  if (x_elems) *x_elems = map->x_elems;
  if (y_elems) *y_elems = map->y_elems;
  if (flops) *flops = map->flops;
  if (n_steps) *n_steps = (int)map->steps.size();
  if (bytes) *bytes = map->bytes;
  return GTN_OK;
}

int gtn_map_out_shape(gtn_map map, int* rank, int64_t* dims) {
  if (!map || !rank) return GTN_ERR_INVALID;
  *rank = (int)map->y_dims.size();
  if (dims)
    for (size_t i = 0; i < map->y_dims.size(); ++i) dims[i] = map->y_dims[i];
  return GTN_OK;
}

int gtn_contract(gtn_ctx ctx, int n_operands, const int* ranks, const int64_t* dims,
                 const int* labels, const int* conj, const int* order,
                 const void* const* operands, void* out, int precision) {
  if (!ctx || !operands || !out) return set_err(ctx, GTN_ERR_INVALID, "null argument");
  // a one-shot contraction: no static grouping (a pre-contracted group only pays off when
  // the map is applied many times); its buffers come from the context's arena, reused in
  // stream order by the next contraction, and the arena grows to the largest need seen
  if (ctx->carena_need > ctx->carena_cap) {
    if (ctx->carena) cudaFree(ctx->carena);
    ctx->carena = nullptr;
    ctx->carena_cap = 0;
    if (cudaMalloc(&ctx->carena, ctx->carena_need) == cudaSuccess) ctx->carena_cap = ctx->carena_need;
    else ctx->carena = nullptr;
  }
  gtn_map map = new (std::nothrow) gtn_map_s();
  if (!map) return set_err(ctx, GTN_ERR_MEMORY, "host allocation failed");
  map->ctx = ctx;
  map->oneshot = true;
  map->arena = ctx->carena;
  map->arena_cap = ctx->carena_cap;
  int st = plan_build(ctx, n_operands, ranks, dims, labels, conj, order, operands, precision, map, false);
  const size_t need = map->arena_off + map->arena_spill;
  if (need > ctx->carena_need && need <= (size_t(8) << 30)) ctx->carena_need = need;
  if (st != GTN_OK) {
    cudaStreamSynchronize(ctx->stream);
    map_free(map);
    delete map;
    return st;
  }
  st = map_run(map, precision, static_cast<const double2*>(operands[0]), static_cast<double2*>(out));
  // arena buffers are reused in stream order: only spilled allocations need the stream to
  // drain before they are freed
  if (!map->owned.empty()) cudaStreamSynchronize(ctx->stream);
  map_free(map);
  delete map;
  return st;
}

// Adjoint of one operand of a contraction (the VJP behind an rrule).  For
// y = contract(operands) and a cotangent ybar shaped like y, out = G with
// <G, d op_slot> = <ybar, dy> for every perturbation of the operand as it enters the
// contraction (after its conj flag), i.e.
//   G = contract(ybar, conj(op_i) for i != slot)   with op_slot's legs as the output.
// The label graph is rewritten: ybar takes the output legs (new positive labels), the legs
// op_slot shared become output legs -1..-r in op_slot's leg order, every other operand's
// conj flag flips.  Without an order the chain starts at ybar and absorbs, greedily, the
// operand sharing the largest contracted extent with the running tensor (ties: the
// smaller result), so that no step is an outer product while a contraction is available.
int gtn_contract_vjp(gtn_ctx ctx, int n_operands, const int* ranks, const int64_t* dims, const int* labels,
                     const int* conj, const int* order, const void* const* operands, int slot, const void* ybar,
                     void* out, int precision) {
  if (!ctx || !ranks || !dims || !labels || !operands || !ybar || !out)
    return set_err(ctx, GTN_ERR_INVALID, "contract_vjp: null argument");
  if (n_operands < 1 || slot < 0 || slot >= n_operands)
    return set_err(ctx, GTN_ERR_INVALID, "contract_vjp: slot outside 0..n_operands-1");
  std::vector<int64_t> off(n_operands + 1, 0);
  for (int i = 0; i < n_operands; ++i) {
    if (ranks[i] < 0 || ranks[i] > 16) return set_err(ctx, GTN_ERR_INVALID, "contract_vjp: rank outside 0..16");
    off[i + 1] = off[i] + ranks[i];
  }
  int maxlab = 0, nout = 0;
  std::vector<int64_t> outdim(64, -1);
  for (int64_t j = 0; j < off[n_operands]; ++j) {
    const int l = labels[j];
    if (l > 0) maxlab = std::max(maxlab, l);
    if (l < 0) {
      if (-l > 63) return set_err(ctx, GTN_ERR_INVALID, "contract_vjp: more than 63 output legs");
      if (outdim[-l] >= 0) return set_err(ctx, GTN_ERR_INVALID, "contract_vjp: output label used twice");
      outdim[-l] = dims[j];
      nout = std::max(nout, -l);
    }
  }
  for (int k = 1; k <= nout; ++k)
    if (outdim[k] < 0) return set_err(ctx, GTN_ERR_INVALID, "contract_vjp: output labels must be -1..-R");
  // new operands: 0 = ybar, then every operand except slot
  std::vector<int> nr, nl, nc;
  std::vector<int64_t> nd;
  std::vector<const void*> np;
  std::vector<int> src;  // original index of each new operand (-1 for ybar)
  nr.push_back(nout);
  for (int k = 1; k <= nout; ++k) {
    nd.push_back(outdim[k]);
    nl.push_back(maxlab + k);
  }
  nc.push_back(0);
  np.push_back(ybar);
  src.push_back(-1);
  for (int i = 0; i < n_operands; ++i) {
    if (i == slot) continue;
    nr.push_back(ranks[i]);
    for (int64_t j = off[i]; j < off[i + 1]; ++j) {
      nd.push_back(dims[j]);
      nl.push_back(labels[j] < 0 ? maxlab - labels[j] : labels[j]);
    }
    nc.push_back(conj && conj[i] ? 0 : 1);
    np.push_back(operands[i]);
    src.push_back(i);
  }
  // the legs op_slot shared become the result's legs -1..-r
  for (int64_t j = off[slot]; j < off[slot + 1]; ++j) {
    const int l = labels[j];
    const int target = l > 0 ? l : maxlab - l;
    int hits = 0;
    for (size_t q = 0; q < nl.size(); ++q)
      if (nl[q] == target) {
        nl[q] = -(int)(j - off[slot] + 1);
        ++hits;
      }
    if (hits != 1) return set_err(ctx, GTN_ERR_INVALID, "contract_vjp: a label of the slot is not shared exactly once");
  }
  const int nn = (int)nr.size();
  std::vector<int64_t> noff(nn + 1, 0);
  for (int i = 0; i < nn; ++i) noff[i + 1] = noff[i] + nr[i];
  std::vector<int> ord;
  if (order) {
    ord.assign(order, order + nn);
  } else {
    std::vector<int> cur(nl.begin() + noff[0], nl.begin() + noff[1]);
    std::vector<int64_t> curd(nd.begin() + noff[0], nd.begin() + noff[1]);
    std::vector<bool> used(nn, false);
    used[0] = true;
    ord.push_back(0);
    for (int step = 1; step < nn; ++step) {
      int best = -1;
      double best_shared = -1, best_size = 0;
      for (int q = 1; q < nn; ++q) {
        if (used[q]) continue;
        double shared = 1, size = 1;
        bool any = false;
        for (int64_t j = noff[q]; j < noff[q + 1]; ++j) {
          bool in_cur = false;
          for (size_t c = 0; c < cur.size(); ++c)
            if (nl[j] > 0 && cur[c] == nl[j]) in_cur = true;
          if (in_cur) { shared *= (double)nd[j]; any = true; }
          else size *= (double)nd[j];
        }
        for (size_t c = 0; c < cur.size(); ++c) {
          bool in_q = false;
          for (int64_t j = noff[q]; j < noff[q + 1]; ++j)
            if (cur[c] > 0 && nl[j] == cur[c]) in_q = true;
          if (!in_q) size *= (double)curd[c];
        }
        if (!any) shared = 0;
        if (shared > best_shared || (shared == best_shared && size < best_size)) {
          best = q;
          best_shared = shared;
          best_size = size;
        }
      }
      used[best] = true;
      ord.push_back(best);
      std::vector<int> nxt;
      std::vector<int64_t> nxtd;
      for (size_t c = 0; c < cur.size(); ++c) {
        bool in_q = false;
        for (int64_t j = noff[best]; j < noff[best + 1]; ++j)
          if (cur[c] > 0 && nl[j] == cur[c]) in_q = true;
        if (!in_q) { nxt.push_back(cur[c]); nxtd.push_back(curd[c]); }
      }
      for (int64_t j = noff[best]; j < noff[best + 1]; ++j) {
        bool in_cur = false;
        for (size_t c = 0; c < cur.size(); ++c)
          if (nl[j] > 0 && cur[c] == nl[j]) in_cur = true;
        if (!in_cur) { nxt.push_back(nl[j]); nxtd.push_back(nd[j]); }
      }
      cur.swap(nxt);
      curd.swap(nxtd);
    }
  }
  return gtn_contract(ctx, nn, nr.data(), nd.data(), nl.data(), nc.data(), ord.data(), np.data(), out, precision);
}

int gtn_permute(gtn_ctx ctx, int rank, const int64_t* dims, const int* perm, const void* in, void* out) {
  if (!ctx || rank < 1 || rank > 16 || !dims || !perm || !in || !out)
    return set_err(ctx, GTN_ERR_INVALID, "gtn_permute: bad argument");
  std::vector<int64_t> strides(rank, 1);
  for (int i = rank - 2; i >= 0; --i) strides[i] = strides[i + 1] * dims[i + 1];
  // out legs perm[0..rank-2] -> M group, perm[rank-1] -> K group (strides of the input)
  std::vector<int64_t> gd, gs;
  int64_t M = 1;
  for (int a = 0; a + 1 < rank; ++a) {
    const int l = perm[a];
    if (l < 0 || l >= rank) return set_err(ctx, GTN_ERR_INVALID, "gtn_permute: bad permutation");
    M *= dims[l];
    if (dims[l] == 1) continue;
    if (!gd.empty() && gs.back() == strides[l] * dims[l]) {
      gd.back() *= dims[l];
      gs.back() = strides[l];
    } else {
      gd.push_back(dims[l]);
      gs.push_back(strides[l]);
    }
  }
  if ((int)gd.size() > GTN_MAXG) return set_err(ctx, GTN_ERR_UNSUPPORTED, "gtn_permute: rank too high");
  GroupSpec mg, kg;
  std::memset(&mg, 0, sizeof(mg));
  std::memset(&kg, 0, sizeof(kg));
  mg.n = (int)gd.size();
  for (int i = 0; i < mg.n; ++i) { mg.dim[i] = gd[i]; mg.str[i] = gs[i]; }
  const int lk = perm[rank - 1];
  const int64_t K = dims[lk];
  kg.n = 1;
  kg.dim[0] = K;
  kg.str[0] = strides[lk];
  cudaError_t e = launch_gather_c128_to_c128(static_cast<const double2*>(in), mg, kg, M, K, K,
                                             static_cast<double2*>(out), ctx->stream);
  ctx->launches++;
  if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("gtn_permute: ") + cudaGetErrorString(e));
  return GTN_OK;
}

int gtn_dot(gtn_ctx ctx, int64_t n, const void* x, const void* y, double* out2) {
  if (!ctx || !x || !y || !out2) return set_err(ctx, GTN_ERR_INVALID, "gtn_dot: null argument");
  const int nblk = multidot_blocks(ctx);
  GTN_CUDA_TRY(ctx, ctx_red(ctx, (size_t)nblk + 8));
  GTN_CUDA_TRY(ctx, launch_multidot(static_cast<const double2*>(x), 0, 1, static_cast<const double2*>(y), n,
                                    ctx->d_red, ctx->d_red + 8, nblk, ctx->stream));
  ctx->launches += 2;
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_red, ctx->d_red, sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
  int st = gtn_ctx_sync(ctx);
  if (st != GTN_OK) return st;
  out2[0] = ctx->h_red[0].x;
  out2[1] = ctx->h_red[0].y;
  return GTN_OK;
}

int gtn_axpby(gtn_ctx ctx, int64_t n, double a_re, double a_im, const void* x, double b_re, double b_im,
              void* y) {
  if (!ctx || !x || !y) return set_err(ctx, GTN_ERR_INVALID, "gtn_axpby: null argument");
  GTN_CUDA_TRY(ctx, launch_axpby(n, make_double2(a_re, a_im), static_cast<const double2*>(x),
                                 make_double2(b_re, b_im), static_cast<double2*>(y), ctx->stream));
  ctx->launches++;
  return GTN_OK;
}

int gtn_copy2d(gtn_ctx ctx, int64_t rows, int64_t cols, const void* src, int64_t src_ld, void* dst,
               int64_t dst_ld) {
  if (!ctx || !src || !dst || rows < 0 || cols < 0 || src_ld < cols || dst_ld < cols)
    return set_err(ctx, GTN_ERR_INVALID, "gtn_copy2d: bad argument");
  if (rows == 0 || cols == 0) return GTN_OK;
  GTN_CUDA_TRY(ctx, cudaMemcpy2DAsync(dst, dst_ld * sizeof(double2), src, src_ld * sizeof(double2),
                                      cols * sizeof(double2), rows, cudaMemcpyDeviceToDevice, ctx->stream));
  return GTN_OK;
}

int gtn_diag_scale(gtn_ctx ctx, int64_t rows, int64_t cols, const double* d_host, int side, void* A) {
  if (!ctx || !d_host || !A || rows < 0 || cols < 0 || (side != 0 && side != 1))
    return set_err(ctx, GTN_ERR_INVALID, "gtn_diag_scale: bad argument");
  const int64_t nd = side == 0 ? cols : rows;
  void* ws = nullptr;
  GTN_CUDA_TRY(ctx, ctx_workspace(ctx, (size_t)nd * sizeof(double) + 256, &ws));
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(ws, d_host, nd * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  GTN_CUDA_TRY(ctx, launch_diag_scale(static_cast<double2*>(A), rows, cols, static_cast<const double*>(ws), side,
                                      ctx->stream));
  ctx->launches++;
  // the host factors are pageable: the copy above is synchronous with respect to the host
  return GTN_OK;
}

int gtn_fill(gtn_ctx ctx, int64_t n, double re, double im, void* x) {
  if (!ctx || !x || n < 0) return set_err(ctx, GTN_ERR_INVALID, "gtn_fill: bad argument");
  if (n == 0) return GTN_OK;
  GTN_CUDA_TRY(ctx, launch_fill_c128(static_cast<double2*>(x), make_double2(re, im), n, ctx->stream));
  ctx->launches++;
  return GTN_OK;
}

int gtn_restrict_leg(gtn_ctx ctx, int rank, const int64_t* dims, int leg, int64_t nsel, const int64_t* idx_host,
                     const void* in, void* out) {
  if (!ctx || !dims || !idx_host || !in || !out || rank < 1 || rank > 16 || leg < 0 || leg >= rank || nsel < 0)
    return set_err(ctx, GTN_ERR_INVALID, "gtn_restrict_leg: bad argument");
  int64_t A = 1, B = 1;
  for (int i = 0; i < leg; ++i) A *= dims[i];
  for (int i = leg + 1; i < rank; ++i) B *= dims[i];
  for (int64_t j = 0; j < nsel; ++j)
    if (idx_host[j] < 0 || idx_host[j] >= dims[leg])
      return set_err(ctx, GTN_ERR_INVALID, "gtn_restrict_leg: index outside the leg");
  if (nsel == 0 || A == 0 || B == 0) return GTN_OK;
  void* ws = nullptr;
  GTN_CUDA_TRY(ctx, ctx_workspace(ctx, (size_t)nsel * sizeof(int64_t) + 256, &ws));
  GTN_CUDA_TRY(ctx, cudaMemcpyAsync(ws, idx_host, nsel * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  GTN_CUDA_TRY(ctx, launch_restrict_leg(static_cast<const double2*>(in), static_cast<double2*>(out), A, dims[leg], nsel,
                                        B, static_cast<const int64_t*>(ws), ctx->stream));
  ctx->launches++;
  // the index list is pageable host memory: the copy above completes before the call returns
  return GTN_OK;
}

}  // extern "C"

extern "C" int gtn_selftest_wait(gtn_ctx ctx, int64_t timeout_us) {
  if (!ctx || timeout_us < 1 || timeout_us > 2000000) return set_err(ctx, GTN_ERR_INVALID, "gtn_selftest_wait: bad argument");
  GTN_CUDA_TRY(ctx, launch_wait_selftest(ctx->d_errflag, (uint64_t)timeout_us * 1000ull, ctx->stream));
  ctx->launches++;
  return GTN_OK;
}
