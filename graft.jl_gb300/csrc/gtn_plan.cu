// Plan compiler and executor for effective maps: an ncon label graph is lowered once
// into a chain of pair steps (the reference's ContractionPlan of PairSteps,
// lib/GraftPlanning/src/Planning/types.jl:54-115, executed like executor.jl:99-144).
//
// Each step absorbs one static S into the running tensor T:
//     C[n][m] = sum_k T[m, k] * S[n, k]
// m runs over T's free legs (in T's order), k over the shared legs (in T's order), n over
// S's free legs (in S's order).  C's legs are (S free..., T free...), row-major.  T is read
// in place through strided index groups, so no permutation kernel runs for small-K steps;
// large-K steps gather T into a K-major operand (c128 for FP64, bf16 slice planes for the
// tcgen05 path).  Statics are permuted/conjugated/packed once when the map is created.
#include "gtn_internal.h"

#include <cstdlib>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <set>

namespace {

constexpr int kSmallK = 64;

// Build an index group over `legs` (positions into a row-major tensor with `dims`),
// merging neighbours that are contiguous in memory.
bool make_group(const std::vector<int64_t>& dims, const std::vector<int>& legs, GroupSpec* g) {
  std::vector<int64_t> strides(dims.size(), 1);
  for (int i = (int)dims.size() - 2; i >= 0; --i) strides[i] = strides[i + 1] * dims[i + 1];
  std::vector<int64_t> gd, gs;
  for (int l : legs) {
    const int64_t d = dims[l], st = strides[l];
    if (d == 1) continue;
    if (!gd.empty() && gs.back() == st * d) {
      gd.back() *= d;
      gs.back() = st;
    } else {
      gd.push_back(d);
      gs.push_back(st);
    }
  }
  if ((int)gd.size() > GTN_MAXG) return false;
  std::memset(g, 0, sizeof(*g));
  g->n = (int)gd.size();
  for (int i = 0; i < g->n; ++i) {
    g->dim[i] = gd[i];
    g->str[i] = gs[i];
  }
  return true;
}

int64_t prod(const std::vector<int64_t>& d, const std::vector<int>& legs) {
  int64_t p = 1;
  for (int l : legs) p *= d[l];
  return p;
}

template <typename T> cudaError_t dalloc(gtn_map map, T** p, size_t bytes) {
  const size_t sz = ((bytes < 256 ? 256 : bytes) + 255) / 256 * 256;
  if (map->oneshot) {
    if (map->arena && map->arena_off + sz <= map->arena_cap) {
      *p = reinterpret_cast<T*>(map->arena + map->arena_off);
      map->arena_off += sz;
      map->bytes += (int64_t)bytes;
      return cudaSuccess;
    }
    map->arena_spill += sz;
  }
  void* q = nullptr;
  size_t got = 0;
  cudaError_t e = ctx_blk_alloc(map->ctx, bytes, &q, &got);
  if (e == cudaSuccess) {
    map->blocks.emplace_back(q, got);
    map->bytes += (int64_t)bytes;
  }
  *p = static_cast<T*>(q);
  return e;
}

bool is_tc(int precision) {
  return precision == GTN_PREC_BF16X6 || precision == GTN_PREC_BF16X3 || precision == GTN_PREC_FP16X3;
}
int nplanes_of(int precision) { return precision == GTN_PREC_BF16X6 ? 3 : 2; }
bool is_fp16(int precision) { return precision == GTN_PREC_FP16X3; }
bool is_f64e(int precision) { return precision == GTN_PREC_FP64E; }

// Device table of the element offsets of indices 0..n-1 of an index group (digits outer..
// inner, the innermost one incremented first), owned by the map.  Computed by a kernel on
// the map's stream: a host table copied from pageable memory would make the copy wait for
// all earlier work on the stream, stalling every map build and one-shot contraction.
// The fill is queued and launched by fill_offset_tables once the plan has passed its memory
// admission, so that a refused plan launches nothing but its statics' packing.
cudaError_t upload_offsets(gtn_map map, const GroupSpec& g, int64_t n, const int64_t** out) {
  int64_t* d = nullptr;
  cudaError_t e = dalloc(map, &d, (size_t)std::max<int64_t>(n, 1) * sizeof(int64_t));
  if (e == cudaSuccess) map->pending_tabs.push_back({g, n, d});
  *out = d;
  return e;
}

int fill_offset_tables(gtn_map map) {
  cudaError_t e = cudaSuccess;
  for (const auto& t : map->pending_tabs) {
    if (t.n > 0) {
      e = launch_offsets_table(t.g, t.n, t.d, map->ctx->stream);
      map->ctx->launches++;
    } else {
      e = cudaMemsetAsync(t.d, 0, sizeof(int64_t), map->ctx->stream);
    }
    if (e != cudaSuccess) break;
  }
  map->pending_tabs.clear();
  return e == cudaSuccess ? GTN_OK : set_err(map->ctx, GTN_ERR_CUDA, std::string("offset tables: ") + cudaGetErrorString(e));
}

// Offset tables of an [M, K] gather, or none (index-group decomposition) when they would
// exceed 256 MiB.
cudaError_t make_tab(gtn_map map, const GroupSpec& mg, const GroupSpec& kg, int64_t M, int64_t K, GatherTab* t) {
  *t = GatherTab();
  if ((M + K) * (int64_t)sizeof(int64_t) > (int64_t(256) << 20)) return cudaSuccess;
  cudaError_t e = upload_offsets(map, mg, M, &t->om);
  if (e == cudaSuccess) e = upload_offsets(map, kg, K, &t->ok);
  t->m_fast = gather_m_fast(mg, kg) ? 1 : 0;
  if (e != cudaSuccess) *t = GatherTab();
  return e;
}

}  // namespace

namespace {

// ---- static grouping: pre-contract consecutive statics when the cost model says so -----
// The chain absorbs statics one at a time; small statics (the child environments of a node
// whose children have small bonds, a TTNO tensor) can be contracted with each other once,
// at map creation, so that the running tensor meets one larger operator in a tensor-core
// GEMM instead of several memory-bound small-K passes.  The reported algorithmic FLOPs stay
// those of the reference's env-first chain.

constexpr int64_t kMaxCombined = int64_t(1) << 22;  // elements of a pre-contracted static

double est_step_time(int prec, double M, double K, double N) {
  const bool fp64 = prec == GTN_PREC_FP64;
  const double e = fp64 ? 16.0 : 8.0;
  const double flops = 8.0 * M * K * N;
  const double hbm = 5e12;
  const bool small = K <= kSmallK && small_contract_fits((int)K, (int)std::min(N, 1048576.0), sizeof(double2));
  double t = 5e-6;  // launch and tail
  if (small) return t + (M * K + M * N) * e / hbm + flops / (fp64 ? 1.1e12 : 15e12);
  if (fp64) return t + flops / 1.1e12 + (2 * M * K + M * N) * e / hbm;
  if (prec == GTN_PREC_FP32) return t + flops / 20e12 + (2 * M * K + M * N) * e / hbm;
  if (prec == GTN_PREC_FP64E) {  // 28 digit products; 7 digit planes of A written and read
    const double Kp = std::ceil(K / 32.0) * 32.0;
    return t + flops / 40e12 + (M * K * 16.0 + M * 2 * Kp * 7 * 2 * 2 + M * N * 16.0) / hbm;
  }
  const double rate = prec == GTN_PREC_BF16X6 ? 200e12 : 300e12;  // bf16x3 and fp16x3: 3 products
  const double P = prec == GTN_PREC_BF16X6 ? 3.0 : 2.0;
  const double Kp = std::ceil(K / 32.0) * 32.0;
  return t + flops / rate + (M * K * e + M * 2 * Kp * P * 2 + M * N * 8) / hbm;
}

struct ChainOp {
  std::vector<int> L;
  std::vector<int64_t> D;
};

// Largest intermediate (elements) of contracting ops[0], ops[1], ... in order.
double group_peak(const std::vector<ChainOp>& ops) {
  std::vector<int> LT = ops[0].L;
  std::vector<int64_t> DT = ops[0].D;
  double peak = 1;
  for (auto d : DT) peak *= (double)d;
  for (size_t j = 1; j < ops.size(); ++j) {
    std::vector<int> nL;
    std::vector<int64_t> nD;
    for (size_t a = 0; a < ops[j].L.size(); ++a) {
      const int l = ops[j].L[a];
      if (!(l > 0 && std::find(LT.begin(), LT.end(), l) != LT.end())) {
        nL.push_back(l);
        nD.push_back(ops[j].D[a]);
      }
    }
    for (size_t a = 0; a < LT.size(); ++a) {
      const int l = LT[a];
      if (!(l > 0 && std::find(ops[j].L.begin(), ops[j].L.end(), l) != ops[j].L.end())) {
        nL.push_back(l);
        nD.push_back(DT[a]);
      }
    }
    LT.swap(nL);
    DT.swap(nD);
    double sz = 1;
    for (auto d : DT) sz *= (double)d;
    peak = std::max(peak, sz);
  }
  return peak;
}

// External legs of a group of operands: labels not paired inside the group, in order.
ChainOp group_external(const std::vector<ChainOp>& ops) {
  std::map<int, int> cnt;
  for (auto& o : ops)
    for (int l : o.L) cnt[l]++;
  ChainOp out;
  for (auto& o : ops)
    for (size_t i = 0; i < o.L.size(); ++i)
      if (!(o.L[i] > 0 && cnt[o.L[i]] == 2)) {
        out.L.push_back(o.L[i]);
        out.D.push_back(o.D[i]);
      }
  return out;
}

// (cost, env-first MACs) of absorbing `chain` into the running tensor `x`.
std::pair<double, double> chain_cost(const ChainOp& x, const std::vector<ChainOp>& chain, int prec) {
  std::vector<int> LT = x.L;
  std::vector<int64_t> DT = x.D;
  double t = 0, macs = 0;
  for (auto& S : chain) {
    double M = 1, K = 1, N = 1;
    std::vector<int> nL;
    std::vector<int64_t> nD;
    std::vector<int> shared;
    for (size_t a = 0; a < LT.size(); ++a) {
      const bool sh = LT[a] > 0 && std::find(S.L.begin(), S.L.end(), LT[a]) != S.L.end();
      if (sh) { K *= (double)DT[a]; shared.push_back(LT[a]); }
      else M *= (double)DT[a];
    }
    for (size_t b = 0; b < S.L.size(); ++b)
      if (std::find(shared.begin(), shared.end(), S.L[b]) == shared.end()) {
        N *= (double)S.D[b];
        nL.push_back(S.L[b]);
        nD.push_back(S.D[b]);
      }
    for (size_t a = 0; a < LT.size(); ++a)
      if (std::find(shared.begin(), shared.end(), LT[a]) == shared.end()) {
        nL.push_back(LT[a]);
        nD.push_back(DT[a]);
      }
    t += est_step_time(prec, M, K, N);
    macs += M * K * N;
    LT.swap(nL);
    DT.swap(nD);
  }
  return {t, macs};
}

}  // namespace

__global__ void c128_to_c64_kernel(const double2* __restrict__ x, float2* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = make_float2((float)x[i].x, (float)x[i].y);
}

int plan_build(gtn_ctx ctx, int n, const int* ranks, const int64_t* dims, const int* labels,
               const int* conj, const int* order, const void* const* statics, int precision,
               gtn_map map, bool allow_group, bool alloc_ws) {
  if (n < 2) return set_err(ctx, GTN_ERR_INVALID, "map needs the input and at least one static");
  if (precision < 0 || precision > GTN_PREC_FP64E) return set_err(ctx, GTN_ERR_INVALID, "unknown precision");
  if ((is_tc(precision) || is_f64e(precision)) && !tc_gemm_supported(ctx->cc_major, ctx->cc_minor))
    return set_err(ctx, GTN_ERR_UNSUPPORTED, "tcgen05 precision modes need an sm_10x device");
  std::vector<std::vector<int64_t>> D(n);
  std::vector<std::vector<int>> L(n);
  int64_t off = 0;
  std::map<int, int> count;
  std::map<int, int64_t> ldim;
  for (int i = 0; i < n; ++i) {
    if (ranks[i] < 0 || ranks[i] > 16) return set_err(ctx, GTN_ERR_INVALID, "bad operand rank");
    for (int r = 0; r < ranks[i]; ++r) {
      D[i].push_back(dims[off + r]);
      L[i].push_back(labels[off + r]);
      if (dims[off + r] <= 0) return set_err(ctx, GTN_ERR_SHAPE, "non-positive leg dimension");
      const int l = labels[off + r];
      if (l == 0) return set_err(ctx, GTN_ERR_INVALID, "label 0 is not allowed");
      count[l]++;
      auto it = ldim.find(l);
      if (it != ldim.end() && it->second != dims[off + r])
        return set_err(ctx, GTN_ERR_SHAPE, "label " + std::to_string(l) + " joins legs of different dimension");
      ldim[l] = dims[off + r];
    }
    off += ranks[i];
  }
  int nout = 0;
  for (auto& kv : count) {
    if (kv.first > 0 && kv.second != 2)
      return set_err(ctx, GTN_ERR_INVALID, "positive label " + std::to_string(kv.first) + " must appear twice");
    if (kv.first < 0) {
      if (kv.second != 1) return set_err(ctx, GTN_ERR_INVALID, "output label repeated");
      nout++;
    }
  }
  for (int k = 1; k <= nout; ++k)
    if (!count.count(-k)) return set_err(ctx, GTN_ERR_INVALID, "output labels must be -1..-R");
  if (conj && conj[0]) return set_err(ctx, GTN_ERR_INVALID, "the input operand cannot be conjugated");
  {
    std::set<int> seen;
    if (order[0] != 0) return set_err(ctx, GTN_ERR_INVALID, "order must start with operand 0");
    for (int i = 0; i < n; ++i) {
      if (order[i] < 0 || order[i] >= n || seen.count(order[i]))
        return set_err(ctx, GTN_ERR_INVALID, "order must be a permutation of the operands");
      seen.insert(order[i]);
    }
  }

  map->ctx = ctx;
  map->precision = precision;
  map->x_dims = D[0];
  map->x_elems = 1;
  for (auto d : D[0]) map->x_elems *= d;
  std::vector<int> LT = L[0];
  std::vector<int64_t> DT = D[0];
  map->max_t = map->x_elems;
  map->max_a = 0;
  map->max_apl = 0;
  const bool tc = is_tc(precision);
  const bool f64e = is_f64e(precision);
  const int P = tc ? nplanes_of(precision) : (f64e ? kF64eSlices : 0);

  // ---- the reference's env-first chain and the grouped chain we execute ------------------
  ChainOp X{L[0], D[0]};
  std::vector<ChainOp> base;
  for (int s = 1; s < n; ++s) base.push_back(ChainOp{L[order[s]], D[order[s]]});
  const auto ref_cost = chain_cost(X, base, precision);
  map->flops = 8.0 * ref_cost.second;
  const int ns = n - 1;
  std::vector<int> best_cut(ns, 1);  // cut[i] = 1: a group ends after static i
  double best_t = ref_cost.first;
  // GTN_STATIC_GROUPING=0 keeps the env-first chain of single statics (no pre-contracted
  // groups): the comparison point of the grouping choice
  const char* genv = std::getenv("GTN_STATIC_GROUPING");
  if (genv && genv[0] == '0') allow_group = false;
  if (allow_group && statics && ns >= 2 && ns <= 12) {
    for (uint32_t mask = 0; mask < (1u << (ns - 1)); ++mask) {
      std::vector<ChainOp> chain;
      std::vector<ChainOp> cur;
      bool ok = true;
      for (int i = 0; i < ns && ok; ++i) {
        cur.push_back(base[i]);
        const bool cut = i == ns - 1 || ((mask >> i) & 1u);
        if (cut) {
          if (cur.size() > 1) {
            if (conj && conj[order[1 + i - (int)cur.size() + 1]]) ok = false;
            ChainOp g = group_external(cur);
            double sz = 1;
            for (auto d : g.D) sz *= (double)d;
            if (sz > (double)kMaxCombined) ok = false;
            // the pre-contraction runs as a chain in member order: every intermediate of it
            // stays within the same bound (members with no shared leg would form outer
            // products far larger than the group)
            if (ok && group_peak(cur) > (double)kMaxCombined) ok = false;
            chain.push_back(g);
          } else {
            chain.push_back(cur[0]);
          }
          cur.clear();
        }
      }
      if (!ok) continue;
      const double t = chain_cost(X, chain, precision).first;
      if (t < 0.9 * best_t) {
        best_t = t;
        for (int i = 0; i < ns; ++i) best_cut[i] = (i == ns - 1 || ((mask >> i) & 1u)) ? 1 : 0;
      }
    }
  }
  // materialise the chain: single statics as given, groups pre-contracted in FP64 on device
  struct Entry {
    std::vector<int> L;
    std::vector<int64_t> D;
    const void* ptr;
    bool conj;
  };
  std::vector<Entry> chain;
  {
    std::vector<int> members;
    for (int i = 0; i < ns; ++i) {
      members.push_back(order[1 + i]);
      if (!best_cut[i]) continue;
      if (members.size() == 1) {
        const int j = members[0];
        chain.push_back(Entry{L[j], D[j], statics ? statics[j] : nullptr, conj && conj[j]});
      } else {
        std::vector<ChainOp> ops;
        for (int j : members) ops.push_back(ChainOp{L[j], D[j]});
        ChainOp g = group_external(ops);
        // sub-network: internal labels kept, external legs renumbered -1..-R
        std::vector<int> sranks, slabels, sconj, sorder;
        std::vector<int64_t> sdims;
        std::vector<const void*> sptrs;
        for (size_t q = 0; q < members.size(); ++q) {
          const int j = members[q];
          sranks.push_back((int)L[j].size());
          for (size_t r = 0; r < L[j].size(); ++r) {
            sdims.push_back(D[j][r]);
            int l = L[j][r];
            auto it = std::find(g.L.begin(), g.L.end(), l);
            if (!(l > 0 && std::count(g.L.begin(), g.L.end(), l) == 0)) l = -(int)(it - g.L.begin()) - 1;
            slabels.push_back(l);
          }
          sconj.push_back(conj && conj[j] ? 1 : 0);
          sorder.push_back((int)q);
          sptrs.push_back(statics[j]);
        }
        int64_t ne = 1;
        for (auto d : g.D) ne *= d;
        double2* buf = nullptr;
        if (dalloc(map, &buf, (size_t)ne * sizeof(double2)) != cudaSuccess)
          return set_err(ctx, GTN_ERR_MEMORY, "pre-contracted static allocation failed");
        gtn_map_s sub;
        int st = plan_build(ctx, (int)members.size(), sranks.data(), sdims.data(), slabels.data(), sconj.data(),
                            sorder.data(), sptrs.data(), GTN_PREC_FP64, &sub, false, true);
        if (st == GTN_OK) st = map_run(&sub, GTN_PREC_FP64, static_cast<const double2*>(sptrs[0]), buf);
        cudaStreamSynchronize(ctx->stream);
        map_free(&sub);
        if (st != GTN_OK) return st;
        chain.push_back(Entry{g.L, g.D, buf, false});
      }
      members.clear();
    }
  }
  map->n_groups = (int)chain.size();

  for (int s = 1; s <= (int)chain.size(); ++s) {
    const int j = s - 1;
    const std::vector<int>& LS = chain[j].L;
    const std::vector<int64_t>& DS = chain[j].D;
    std::vector<int> sh, freeT, freeS;  // positions
    std::vector<int> shS;               // positions in S of the shared labels (T order)
    for (int a = 0; a < (int)LT.size(); ++a) {
      const int l = LT[a];
      auto it = std::find(LS.begin(), LS.end(), l);
      if (l > 0 && it != LS.end()) {
        sh.push_back(a);
        shS.push_back((int)(it - LS.begin()));
      } else {
        freeT.push_back(a);
      }
    }
    for (int b = 0; b < (int)LS.size(); ++b)
      if (std::find(shS.begin(), shS.end(), b) == shS.end()) freeS.push_back(b);
    for (int a : freeT)
      if (LT[a] > 0 && std::count(LT.begin(), LT.end(), LT[a]) > 1)
        return set_err(ctx, GTN_ERR_UNSUPPORTED, "self-contraction inside one operand");

    PlanStep st;
    st.operand = j;
    st.M = prod(DT, freeT);
    st.K = prod(DT, sh);
    st.N = prod(DS, freeS);
    st.macs = (double)st.M * (double)st.N * (double)st.K;
    if (!make_group(DT, freeT, &st.mg) || !make_group(DT, sh, &st.kg))
      return set_err(ctx, GTN_ERR_UNSUPPORTED, "too many non-contiguous leg groups");
    st.small = st.K <= kSmallK && small_contract_fits((int)st.K, (int)std::min<int64_t>(st.N, 1 << 20), sizeof(double2));
    st.tc = (tc || f64e) && !st.small;
    st.Kp = ((st.K + 31) / 32) * 32;
    // C legs: S free (S order), then T free (T order)
    for (int b : freeS) { st.out_labels.push_back(LS[b]); st.out_dims.push_back(DS[b]); }
    for (int a : freeT) { st.out_labels.push_back(LT[a]); st.out_dims.push_back(DT[a]); }
    st.out_elems = st.M * st.N;
    map->max_t = std::max(map->max_t, st.out_elems);
    if (!st.small) {
      map->max_a = std::max(map->max_a, st.M * st.K);
      if (st.tc) map->max_apl = std::max(map->max_apl, (int64_t)P * st.M * 2 * st.Kp);
      if (st.tc) map->max_mtc = std::max(map->max_mtc, st.M);
      st.splitk = gemm_splitk_slices(st.M, st.N, st.K);
      if (st.splitk > 1) map->max_splitk = std::max(map->max_splitk, (int64_t)st.splitk * st.M * st.N);
    }

    // ---- pack the static: B[n][k] = S[freeS(n), shared(k)] (conj applied) -------------
    if (chain[j].ptr) {
      cudaError_t e = dalloc(map, &st.b64, (size_t)st.N * st.K * sizeof(double2));
      if (e != cudaSuccess) return set_err(ctx, GTN_ERR_MEMORY, "static packing allocation failed");
      GroupSpec gn, gk;
      if (!make_group(DS, freeS, &gn) || !make_group(DS, shS, &gk))
        return set_err(ctx, GTN_ERR_UNSUPPORTED, "too many non-contiguous static leg groups");
      e = launch_gather_c128_to_c128(static_cast<const double2*>(chain[j].ptr), gn, gk, st.N, st.K, st.K,
                                     st.b64, ctx->stream);
      ctx->launches++;
      if (e == cudaSuccess && chain[j].conj) {
        e = launch_conj_inplace(st.b64, st.N * st.K, ctx->stream);
        ctx->launches++;
      }
      // (a one-shot FP64 contraction and an FP64-grade plan never read the complex FP32 copy)
      if (e == cudaSuccess && !(map->oneshot && precision == GTN_PREC_FP64) && !f64e) {
        e = dalloc(map, &st.b32, (size_t)st.N * st.K * sizeof(float2));
        if (e == cudaSuccess) {
          const int64_t ne = st.N * st.K;
          int64_t blocks = std::min<int64_t>((ne + 255) / 256, 152 * 8);
          c128_to_c64_kernel<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, ctx->stream>>>(st.b64, st.b32, ne);
          ctx->launches++;
          e = cudaGetLastError();
        }
      }
      if (e == cudaSuccess && st.tc) {
        st.bplanes = P;
        const int64_t pstride = 2 * st.N * 2 * st.Kp;
        e = dalloc(map, &st.bpl, (size_t)P * pstride * sizeof(__nv_bfloat16));
        if (e == cudaSuccess && f64e) {
          st.bfp16 = 2;  // integer digit planes
          e = dalloc(map, &st.bmax, (size_t)st.N * sizeof(float));
          if (e == cudaSuccess) e = launch_pack_b_planes_i7(st.b64, st.N, st.K, st.Kp, pstride, st.bpl, st.bmax,
                                                            ctx->stream);
          ctx->launches += 2;
        } else if (e == cudaSuccess && is_fp16(precision)) {
          st.bfp16 = 1;
          e = dalloc(map, &st.bmax, (size_t)st.N * sizeof(float));
          if (e == cudaSuccess) e = launch_pack_b_planes_f16(st.b64, st.N, st.K, st.Kp, pstride, st.bpl, st.bmax,
                                                             ctx->stream);
          ctx->launches += 2;
        } else if (e == cudaSuccess) {
          e = launch_pack_b_planes(st.b64, st.N, st.K, st.Kp, P, pstride, st.bpl, ctx->stream);
          ctx->launches++;
        }
      }
      if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("static packing: ") + cudaGetErrorString(e));
    }
    if (statics && st.tc && !map->oneshot) {
      cudaError_t e = make_tab(map, st.mg, st.kg, st.M, st.K, &st.tab);
      if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("offset tables: ") + cudaGetErrorString(e));
    }
    map->exec_flops += 8.0 * st.macs;
    map->steps.push_back(st);
    LT = map->steps.back().out_labels;
    DT = map->steps.back().out_dims;
  }
  for (int l : LT)
    if (l > 0) return set_err(ctx, GTN_ERR_INVALID, "unresolved positive label after the last step");
  // final permutation to y order (-1, -2, ...)
  const int R = (int)LT.size();
  std::vector<int> ypos(R);
  map->y_dims.assign(R, 1);
  for (int a = 0; a < R; ++a) {
    const int k = -LT[a] - 1;
    ypos[k] = a;
    map->y_dims[k] = DT[a];
  }
  map->y_elems = 1;
  for (auto d : map->y_dims) map->y_elems *= d;
  std::vector<int> mlegs(ypos.begin(), ypos.end() - (R > 0 ? 1 : 0));
  std::vector<int> klegs;
  if (R > 0) klegs.push_back(ypos[R - 1]);
  if (!make_group(DT, mlegs, &map->fin_mg) || !make_group(DT, klegs, &map->fin_kg))
    return set_err(ctx, GTN_ERR_UNSUPPORTED, "too many non-contiguous output leg groups");
  map->fin_K = R > 0 ? map->y_dims[R - 1] : 1;
  map->fin_M = map->y_elems / map->fin_K;
  bool ident = true;
  for (int a = 0; a < R; ++a) ident = ident && ypos[a] == a;
  map->fin_identity = ident;
  if (statics && !map->oneshot) {  // one-shot contractions skip the tables
    cudaError_t e = make_tab(map, map->fin_mg, map->fin_kg, map->fin_M, map->fin_K, &map->fin_tab);
    if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("offset tables: ") + cudaGetErrorString(e));
  }

  // ---- an FP64 plan of its own when this plan's grouping was chosen for a mixed mode ------
  // (the Rayleigh quotient and FP64 comparisons then run the FP64-optimal chain; both plans
  // share the workspace below, they never run concurrently)
  if (allow_group && precision != GTN_PREC_FP64 && statics && map->n_groups != n - 1) {
    gtn_map alt = new (std::nothrow) gtn_map_s();
    if (!alt) return set_err(ctx, GTN_ERR_MEMORY, "host allocation failed");
    const int st = plan_build(ctx, n, ranks, dims, labels, conj, order, statics, GTN_PREC_FP64, alt, true, false);
    if (st != GTN_OK) {
      map_free(alt);
      delete alt;
      return st;
    }
    map->fp64_alt = alt;
  }
  if (!alloc_ws) return fill_offset_tables(map);

  // ---- workspace admission, then allocation ------------------------------------------
  int64_t max_t = map->max_t, max_a = map->max_a, max_sk = map->max_splitk;
  if (map->fp64_alt) {
    max_t = std::max(max_t, map->fp64_alt->max_t);
    max_a = std::max(max_a, map->fp64_alt->max_a);
    max_sk = std::max(max_sk, map->fp64_alt->max_splitk);
  }
  const size_t tbytes = (size_t)max_t * sizeof(double2);
  const size_t abytes = std::max<size_t>((size_t)max_a * sizeof(double2),
                                         (size_t)map->max_apl * sizeof(__nv_bfloat16));
  size_t freeb = 0, totalb = 0;
  if (map->oneshot) freeb = SIZE_MAX;  // one-shot contraction: the arena or a failing cudaMalloc decides
  else {
    cudaMemGetInfo(&freeb, &totalb);
    freeb += ctx->blk_cached;  // cached blocks are reused or given back on demand
  }
  const size_t need = 2 * tbytes + abytes + (size_t)(1u << 30);
  if (need > freeb)
    return set_err(ctx, GTN_ERR_MEMORY, "memory admission refused: map workspace " +
                                            std::to_string(need >> 20) + " MiB > free " +
                                            std::to_string(freeb >> 20) + " MiB");
  if (dalloc(map, &map->buf0, tbytes) != cudaSuccess || dalloc(map, &map->buf1, tbytes) != cudaSuccess ||
      dalloc(map, &map->abuf, std::max<size_t>(abytes, 256)) != cudaSuccess)
    return set_err(ctx, GTN_ERR_MEMORY, "map workspace allocation failed");
  if ((is_fp16(precision) || f64e) && map->max_mtc > 0 &&
      dalloc(map, &map->amax, (size_t)map->max_mtc * sizeof(float)) != cudaSuccess)
    return set_err(ctx, GTN_ERR_MEMORY, "map workspace allocation failed");
  if (max_sk > 0 && dalloc(map, reinterpret_cast<double2**>(&map->skbuf), (size_t)max_sk * sizeof(double2)) !=
                        cudaSuccess)
    return set_err(ctx, GTN_ERR_MEMORY, "map workspace allocation failed");
  if (map->fp64_alt) {
    map->fp64_alt->buf0 = map->buf0;
    map->fp64_alt->buf1 = map->buf1;
    map->fp64_alt->abuf = map->abuf;
    map->fp64_alt->skbuf = map->skbuf;
  }
  return fill_offset_tables(map);
}

void map_free(gtn_map map) {
  if (map->fp64_alt) {
    map_free(map->fp64_alt);
    delete map->fp64_alt;
    map->fp64_alt = nullptr;
  }
  for (void* p : map->owned) cudaFree(p);
  map->owned.clear();
  for (auto& b : map->blocks) ctx_blk_release(map->ctx, b.first, b.second);
  map->blocks.clear();
  if (map->kv) cudaFree(map->kv);
  map->kv = nullptr;
  if (map->kscratch) cudaFree(map->kscratch);
  map->kscratch = nullptr;
}

// Optional per-launch timing: CUDA events around every kernel of one application.
struct ProfRec {
  cudaEvent_t a, b;
  int kind;
  double flops;
};
static std::vector<ProfRec>* g_prof = nullptr;

static void prof_begin(cudaStream_t s) {
  if (!g_prof) return;
  ProfRec r;
  cudaEventCreate(&r.a);
  cudaEventCreate(&r.b);
  cudaEventRecord(r.a, s);
  r.kind = -1;
  r.flops = 0;
  g_prof->push_back(r);
}
static void prof_end(cudaStream_t s, int kind, double flops) {
  if (!g_prof || g_prof->empty()) return;
  ProfRec& r = g_prof->back();
  cudaEventRecord(r.b, s);
  r.kind = kind;
  r.flops = flops;
}

int map_run(gtn_map map, int precision, const double2* x, double2* y) {
  if (map->bm) {  // a block-sparse Krylov operator
    if (precision == blockmap_precision(map->bm)) return blockmap_run(map->bm, x, y);
    if (precision == GTN_PREC_FP64 && map->bm64) return blockmap_run(map->bm64, x, y);
    return set_err(map->ctx, GTN_ERR_INVALID, "block map: no map of the requested precision (pass an FP64 block map)");
  }
  if (precision == GTN_PREC_FP64 && map->fp64_map) {  // e.g. an FP64-grade tensor-core twin
    gtn_map m2 = map->fp64_map;
    return map_run(m2, m2->precision, x, y);
  }
  if (precision == GTN_PREC_FP64 && map->fp64_alt) return map_run(map->fp64_alt, precision, x, y);
  gtn_ctx ctx = map->ctx;
  cudaStream_t s = ctx->stream;
  const bool tc = is_tc(precision);
  if (tc) {
    for (auto& st : map->steps)
      if (!st.small && (!st.bpl || st.bplanes != nplanes_of(precision) || st.bfp16 != (is_fp16(precision) ? 1 : 0)))
        return set_err(ctx, GTN_ERR_INVALID, "map was not created for this tcgen05 precision");
  }
  const bool f64e = is_f64e(precision);
  if (f64e) {
    for (auto& st : map->steps)
      if (!st.small && (!st.bpl || st.bplanes != kF64eSlices || st.bfp16 != 2 || !map->amax))
        return set_err(ctx, GTN_ERR_INVALID, "map was not created for the FP64-grade tensor-core precision");
  }
  const bool fp64 = precision == GTN_PREC_FP64 || f64e;  // complex FP64 running tensors
  const int P = tc ? nplanes_of(precision) : 0;
  void* bufs[2] = {map->buf0, map->buf1};
  const void* cur = x;
  bool cur64 = true;
  cudaError_t e = cudaSuccess;
  const int nst = (int)map->steps.size();
  for (int i = 0; i < nst && e == cudaSuccess; ++i) {
    const PlanStep& st = map->steps[i];
    void* out = bufs[i & 1];
    if (fp64) {
      if (st.small) {
        prof_begin(s);
        e = launch_small_contract_c128(static_cast<const double2*>(cur), st.mg, st.kg, st.M, (int)st.K,
                                       (int)st.N, st.b64, static_cast<double2*>(out), s);
        prof_end(s, GTN_KERNEL_SMALL, 8.0 * st.macs);
        ctx->launches++;
      } else if (f64e) {
        // integer digit planes of the running tensor (row maxima first), then the exact
        // chunked digit-product GEMM straight into complex FP64
        __nv_bfloat16* Apl = static_cast<__nv_bfloat16*>(map->abuf);
        const int64_t pstride = st.M * 2 * st.Kp;
        prof_begin(s);
        bool fused = false;
        if (st.tab.om)
          e = launch_split_i7_rows_tab(static_cast<const double2*>(cur), st.tab, st.M, st.K, st.Kp, pstride,
                                       map->amax, Apl, s, &fused);
        else
          e = launch_split_i7_rows_grp(static_cast<const double2*>(cur), st.mg, st.kg, st.M, st.K, st.Kp, pstride,
                                       map->amax, Apl, s, &fused);
        if (e == cudaSuccess && !fused) {  // rows too long for the clusters: maxima first, then the split
          if (st.tab.om) {
            e = launch_rowmax_tab(cur, 1, st.tab, st.M, st.K, map->amax, s);
            if (e == cudaSuccess)
              e = launch_split_i7_tab(static_cast<const double2*>(cur), st.tab, st.M, st.K, st.Kp, pstride,
                                      map->amax, Apl, s);
          } else {
            e = launch_rowmax_c128(static_cast<const double2*>(cur), st.mg, st.kg, st.M, st.K, map->amax, s);
            if (e == cudaSuccess)
              e = launch_split_i7_c128(static_cast<const double2*>(cur), st.mg, st.kg, st.M, st.K, st.Kp, pstride,
                                       map->amax, Apl, s);
          }
        }
        prof_end(s, GTN_KERNEL_SPLIT, 0.0);
        ctx->launches += fused ? 1 : 2;
        if (e == cudaSuccess) {
          F64eGemmArgs a;
          a.A = Apl;
          a.B = st.bpl;
          a.C = static_cast<double2*>(out);
          a.M = st.M;
          a.N = st.N;
          a.Kp = st.Kp;
          a.a_max = map->amax;
          a.b_max = st.bmax;
          std::string why;
          prof_begin(s);
          e = launch_f64e_gemm(a, ctx->d_errflag, s, &why);
          prof_end(s, GTN_KERNEL_TC_GEMM, 8.0 * st.macs);
          ctx->launches++;
          if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, "f64e_gemm: " + why + " " + cudaGetErrorString(e));
        }
      } else {
        double2* A = static_cast<double2*>(map->abuf);
        prof_begin(s);
        e = launch_gather_c128_to_c128(static_cast<const double2*>(cur), st.mg, st.kg, st.M, st.K, st.K, A, s);
        prof_end(s, GTN_KERNEL_GATHER, 0.0);
        prof_begin(s);
        if (e == cudaSuccess && st.splitk > 1 && map->skbuf)
          e = launch_zgemm_simt_splitk(A, st.b64, static_cast<double2*>(out), st.M, st.N, st.K, st.splitk,
                                       static_cast<double2*>(map->skbuf), s);
        else if (e == cudaSuccess)
          e = launch_zgemm_simt(A, st.b64, static_cast<double2*>(out), st.M, st.N, st.K, s);
        prof_end(s, GTN_KERNEL_ZGEMM, 8.0 * st.macs);
        ctx->launches += 2;
      }
    } else {
      if (cur64 && (st.small || !tc)) {
        // the FP32 kernels read complex FP32: convert the FP64 input once
        void* conv = bufs[(i + 1) & 1];
        int64_t blocks = std::min<int64_t>((map->x_elems + 255) / 256, 152 * 8);
        prof_begin(s);
        c128_to_c64_kernel<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(
            static_cast<const double2*>(cur), static_cast<float2*>(conv), map->x_elems);
        prof_end(s, GTN_KERNEL_CONVERT, 0.0);
        ctx->launches++;
        e = cudaGetLastError();
        cur = conv;
        cur64 = false;
        if (e != cudaSuccess) break;
      }
      if (st.small) {
        prof_begin(s);
        e = launch_small_contract_c64(static_cast<const float2*>(cur), st.mg, st.kg, st.M, (int)st.K,
                                      (int)st.N, st.b32, static_cast<float2*>(out), s);
        prof_end(s, GTN_KERNEL_SMALL, 8.0 * st.macs);
        ctx->launches++;
      } else if (!tc) {
        float2* A = static_cast<float2*>(map->abuf);
        prof_begin(s);
        e = launch_gather_c64_to_c64(static_cast<const float2*>(cur), st.mg, st.kg, st.M, st.K, st.K, A, s);
        prof_end(s, GTN_KERNEL_GATHER, 0.0);
        prof_begin(s);
        if (e == cudaSuccess && st.splitk > 1 && map->skbuf)
          e = launch_cgemm_simt_splitk(A, st.b32, static_cast<float2*>(out), st.M, st.N, st.K, st.splitk,
                                       static_cast<float2*>(map->skbuf), s);
        else if (e == cudaSuccess)
          e = launch_cgemm_simt(A, st.b32, static_cast<float2*>(out), st.M, st.N, st.K, s);
        prof_end(s, GTN_KERNEL_CGEMM, 8.0 * st.macs);
        ctx->launches += 2;
      } else {
        __nv_bfloat16* Apl = static_cast<__nv_bfloat16*>(map->abuf);
        const int64_t pstride = st.M * 2 * st.Kp;
        const bool f16 = is_fp16(precision);
        prof_begin(s);
        bool fused = false;
        if (f16) {  // one pass: row maxima and fp16 planes together
          if (st.tab.om)
            e = launch_split16_rows_tab(cur, cur64 ? 1 : 0, st.tab, st.M, st.K, st.Kp, pstride, map->amax, Apl, s,
                                        &fused);
          else
            e = launch_split16_rows_grp(cur, cur64 ? 1 : 0, st.mg, st.kg, st.M, st.K, st.Kp, pstride, map->amax, Apl,
                                        s, &fused);
          if (fused) ctx->launches++;
        }
        if (e == cudaSuccess && !fused) {  // two passes: row maxima (fp16 planes only), then the split
          if (st.tab.om) {
            // offsets from the step's tables
            if (f16) {
              e = launch_rowmax_tab(cur, cur64 ? 1 : 0, st.tab, st.M, st.K, map->amax, s);
              if (e == cudaSuccess)
                e = launch_split16_tab(cur, cur64 ? 1 : 0, st.tab, st.M, st.K, st.Kp, pstride, map->amax, Apl, s);
              ctx->launches += 2;
            } else {
              e = launch_split_tab(cur, cur64 ? 1 : 0, st.tab, st.M, st.K, st.Kp, P, pstride, Apl, s);
              ctx->launches++;
            }
          } else if (f16) {
            // fp16 planes: per-row maxima first, then the scaled two-slice split
            if (cur64)
              e = launch_rowmax_c128(static_cast<const double2*>(cur), st.mg, st.kg, st.M, st.K, map->amax, s);
            else
              e = launch_rowmax_c64(static_cast<const float2*>(cur), st.mg, st.kg, st.M, st.K, map->amax, s);
            if (e == cudaSuccess && cur64)
              e = launch_split16_c128(static_cast<const double2*>(cur), st.mg, st.kg, st.M, st.K, st.Kp, pstride,
                                      map->amax, Apl, s);
            else if (e == cudaSuccess)
              e = launch_split16_c64(static_cast<const float2*>(cur), st.mg, st.kg, st.M, st.K, st.Kp, pstride,
                                     map->amax, Apl, s);
            ctx->launches += 2;
          } else if (cur64) {
            e = launch_split_c128(static_cast<const double2*>(cur), st.mg, st.kg, st.M, st.K, st.Kp, P,
                                  pstride, Apl, s);
            ctx->launches++;
          } else {
            e = launch_split_c64(static_cast<const float2*>(cur), st.mg, st.kg, st.M, st.K, st.Kp, P,
                                 pstride, Apl, s);
            ctx->launches++;
          }
        }
        prof_end(s, GTN_KERNEL_SPLIT, 0.0);
        if (e == cudaSuccess) {
          TcGemmArgs a;
          a.A = Apl;
          a.B = st.bpl;
          a.C = static_cast<float2*>(out);
          a.M = st.M;
          a.N = st.N;
          a.Kp = st.Kp;
          a.a_planes = P;
          a.b_planes = P;
          if (f16) {
            a.fp16 = 1;
            a.a_max = map->amax;
            a.b_max = st.bmax;
          }
          // products accumulated small terms first
          if (P == 3) {
            const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
            a.nprod = 6;
            for (int q = 0; q < 6; ++q) { a.prod_a[q] = pa[q]; a.prod_b[q] = pb[q]; }
          } else {
            const int pa[3] = {1, 0, 0}, pb[3] = {0, 1, 0};
            a.nprod = 3;
            for (int q = 0; q < 3; ++q) { a.prod_a[q] = pa[q]; a.prod_b[q] = pb[q]; }
          }
          std::string why;
          prof_begin(s);
          e = launch_tc_gemm(a, ctx->d_errflag, s, &why);
          prof_end(s, GTN_KERNEL_TC_GEMM, 8.0 * st.macs);
          ctx->launches++;
          if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, "tc_gemm: " + why + " " + cudaGetErrorString(e));
        }
      }
      cur64 = false;
    }
    cur = out;
  }
  if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("map step: ") + cudaGetErrorString(e));
  prof_begin(s);
  if (map->fin_tab.om)
    e = launch_gather_tab_to_c128(cur, cur64 ? 1 : 0, map->fin_tab, map->fin_M, map->fin_K, map->fin_K, y, s);
  else if (cur64)
    e = launch_gather_c128_to_c128(static_cast<const double2*>(cur), map->fin_mg, map->fin_kg, map->fin_M,
                                   map->fin_K, map->fin_K, y, s);
  else
    e = launch_gather_c64_to_c128(static_cast<const float2*>(cur), map->fin_mg, map->fin_kg, map->fin_M,
                                  map->fin_K, map->fin_K, y, s);
  prof_end(s, GTN_KERNEL_OUTPUT, 0.0);
  ctx->launches++;
  if (e != cudaSuccess) return set_err(ctx, GTN_ERR_CUDA, std::string("map output: ") + cudaGetErrorString(e));
  return GTN_OK;
}

int map_run_profiled(gtn_map map, int precision, const double2* x, double2* y, int cap, double* ms,
                     int* kind, double* flops, int* count) {
  std::vector<ProfRec> recs;
  g_prof = &recs;
  int st = map_run(map, precision, x, y);
  g_prof = nullptr;
  cudaError_t e = cudaStreamSynchronize(map->ctx->stream);
  int n = 0;
  for (auto& r : recs) {
    float t = 0.f;
    if (st == GTN_OK && e == cudaSuccess) cudaEventElapsedTime(&t, r.a, r.b);
    if (n < cap) {
      ms[n] = t;
      kind[n] = r.kind;
      flops[n] = r.flops;
    }
    ++n;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  *count = n;
  if (st != GTN_OK) return st;
  if (e != cudaSuccess) return set_err(map->ctx, GTN_ERR_CUDA, cudaGetErrorString(e));
  return GTN_OK;
}
