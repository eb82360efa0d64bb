// Tensor objects and kind-based construction of the effective maps and environment updates.
//
// The reference builds its Krylov maps from a node's local structure only
// (lib/GraftContractions/src/Contractions/effective.jl:627-797,878-1034) and its environment
// updates the same way (envcache.jl:919-999): which legs of the node tensor face which
// neighbour, where the TTNO legs sit (children..., P_out, P_in, parent), and whether the node
// is the root (whose unit parent legs are closed by an all-ones cap, Backend.jl:144-150).
// This file writes those label graphs and their env-first absorption orders from a
// gtn_site_desc, so a caller that holds tensors (gtn_tensor handles, or plain device
// buffers) can ask for "the two-site map of edge n -> m" without building an ncon graph.
// The graphs are the same, leg for leg, as the host harness's contractions.h1_spec /
// h2_spec / env_spec (checked label by label by the CPU tests).
#include "gtn_internal.h"

#include <algorithm>
#include <new>

struct gtn_tensor_s {
  gtn_ctx ctx = nullptr;
  int rank = 0;
  int64_t dims[16] = {};
  int64_t elems = 0;
  void* data = nullptr;
  bool owned = false;
};

namespace {

struct Spec {
  std::vector<std::vector<int>> labels;  // per operand
  std::vector<int> order;
  bool cap = false;                      // the last operand is the root cap (synthesised)
  int x_rank = 0;
};

int state_leg(int K, bool parent_side, int slot) { return parent_side ? K + 1 : slot; }
int op_leg(int K, bool parent_side, int slot) { return parent_side ? K + 2 : slot; }

// One-site map at n: operands (x, W, env(w->n) for the children in slot order then the
// parent, cap?); order x, children envs, W, parent env, cap (effective.jl:627-686).
Spec h1_spec(int K, bool root) {
  Spec s;
  int fresh = 0;
  const int xr = K + 2, wr = K + 3;
  std::vector<int> x(xr, 0), w(wr, 0);
  const int pin = ++fresh;
  x[K] = pin;
  w[K + 1] = pin;
  w[K] = -(K + 1);
  std::vector<std::vector<int>> envs;
  std::vector<int> children, parents;
  int idx = 2;
  for (int j = 0; j < K + (root ? 0 : 1); ++j) {
    const bool par = j == K;
    const int lx = state_leg(K, par, j);
    const int kk = ++fresh, oo = ++fresh;
    x[lx] = kk;
    w[op_leg(K, par, j)] = oo;
    envs.push_back({kk, oo, -(lx + 1)});
    (par ? parents : children).push_back(idx++);
  }
  s.labels.push_back(x);
  s.labels.push_back(w);
  for (auto& e : envs) s.labels.push_back(e);
  if (root) {
    const int ka = ++fresh, ko = ++fresh;
    s.labels[0][xr - 1] = ka;
    s.labels[1][wr - 1] = ko;
    s.labels.push_back({ka, ko, -xr});
    s.cap = true;
  }
  s.order.push_back(0);
  for (int c : children) s.order.push_back(c);
  s.order.push_back(1);
  for (int p : parents) s.order.push_back(p);
  if (s.cap) s.order.push_back((int)s.labels.size() - 1);
  s.x_rank = xr;
  return s;
}

// Two-site map of the edge n -> m (m the parent, n its child in slot k): Θ legs
// (n children..., phys_n, m children except n..., phys_m, m parent); operands (Θ, Wn, Wm,
// env(w->n) for n's children, env(w->m) for m's other children then m's parent, cap?);
// order Θ, n's envs, Wn, m's child envs, Wm, m's parent env, cap (effective.jl:878-976).
Spec h2_spec(int Kn, int Km, int k, bool m_root) {
  Spec s;
  int fresh = 0;
  const int pn = Kn + 1;
  const int xr = pn + (Km - 1) + 2;
  const int wnr = Kn + 3, wmr = Km + 3;
  std::vector<int> x(xr, 0), wn(wnr, 0), wm(wmr, 0);
  auto mpos = [&](int j) { return pn + (j < k ? j : j - 1); };
  const int ob = ++fresh;
  wn[wnr - 1] = ob;
  wm[k] = ob;
  int pin = ++fresh;
  x[Kn] = pin;
  wn[Kn + 1] = pin;
  wn[Kn] = -(Kn + 1);
  pin = ++fresh;
  x[mpos(Km)] = pin;
  wm[Km + 1] = pin;
  wm[Km] = -(mpos(Km) + 1);
  std::vector<std::vector<int>> envs;
  std::vector<int> envn, envmc, envmp;
  int idx = 3;
  for (int j = 0; j < Kn; ++j) {
    const int kk = ++fresh, oo = ++fresh;
    x[j] = kk;
    wn[j] = oo;
    envs.push_back({kk, oo, -(j + 1)});
    envn.push_back(idx++);
  }
  for (int j = 0; j < Km + (m_root ? 0 : 1); ++j) {
    if (j == k) continue;
    const bool par = j == Km;
    int lw, lx;
    if (par) {
      lw = wmr - 1;
      lx = xr - 1;
    } else {
      lw = j;
      lx = mpos(j);
    }
    const int kk = ++fresh, oo = ++fresh;
    x[lx] = kk;
    wm[lw] = oo;
    envs.push_back({kk, oo, -(lx + 1)});
    (par ? envmp : envmc).push_back(idx++);
  }
  s.labels.push_back(x);
  s.labels.push_back(wn);
  s.labels.push_back(wm);
  for (auto& e : envs) s.labels.push_back(e);
  if (m_root) {
    const int ka = ++fresh, ko = ++fresh;
    s.labels[0][xr - 1] = ka;
    s.labels[2][wmr - 1] = ko;
    s.labels.push_back({ka, ko, -xr});
    s.cap = true;
  }
  s.order.push_back(0);
  for (int c : envn) s.order.push_back(c);
  s.order.push_back(1);
  for (int c : envmc) s.order.push_back(c);
  s.order.push_back(2);
  for (int c : envmp) s.order.push_back(c);
  if (s.cap) s.order.push_back((int)s.labels.size() - 1);
  s.x_rank = xr;
  return s;
}

// Environment of node u towards neighbour v (v = u's parent when open_slot < 0, else u's
// child in that slot): operands (ket A, env(w->u) for the other neighbours in slot order
// then the parent, cap?, W, conj(bra A)); output (ket, op, bra) (envcache.jl:919-999).
Spec env_spec(int K, bool root, int open_slot) {
  Spec s;
  int fresh = 0;
  const int ar = K + 2, wr = K + 3;
  std::vector<int> a(ar, 0), b(ar, 0), w(wr, 0);
  const int pin = ++fresh, pout = ++fresh;
  a[K] = pin;
  w[K + 1] = pin;
  w[K] = pout;
  b[K] = pout;
  std::vector<std::vector<int>> envs;
  for (int j = 0; j < K + (root ? 0 : 1); ++j) {
    const bool par = j == K;
    const int la = state_leg(K, par, j), lw = op_leg(K, par, j);
    const bool open = par ? open_slot < 0 : open_slot == j;
    if (open) {
      a[la] = -1;
      w[lw] = -2;
      b[la] = -3;
    } else {
      const int e0 = ++fresh, e1 = ++fresh, e2 = ++fresh;
      a[la] = e0;
      w[lw] = e1;
      b[la] = e2;
      envs.push_back({e0, e1, e2});
    }
  }
  std::vector<int> cap;
  if (root) {
    const int ka = ++fresh, ko = ++fresh, kb = ++fresh;
    a[ar - 1] = ka;
    w[wr - 1] = ko;
    b[ar - 1] = kb;
    cap = {kb, ko, ka};
    s.cap = true;
  }
  s.labels.push_back(a);
  for (auto& e : envs) s.labels.push_back(e);
  if (root) s.labels.push_back(cap);
  s.labels.push_back(w);
  s.labels.push_back(b);
  for (int i = 0; i < (int)s.labels.size(); ++i) s.order.push_back(i);
  s.x_rank = ar;
  return s;
}

// Link map y = E(n->m) C E(m->n): labels [[1,2],[1,3,-1],[2,3,-2]] (effective.jl:739-749).
Spec h0_spec() {
  Spec s;
  s.labels = {{1, 2}, {1, 3, -1}, {2, 3, -2}};
  s.order = {0, 1, 2};
  s.x_rank = 2;
  return s;
}

int build_spec(const gtn_site_desc* d, Spec* s) {
  if (!d) return GTN_ERR_INVALID;
  if (d->n_children < 0 || d->n_children > 12 || d->m_children < 0 || d->m_children > 12) return GTN_ERR_INVALID;
  switch (d->kind) {
    case GTN_MAP_H1: *s = h1_spec(d->n_children, d->n_is_root != 0); return GTN_OK;
    case GTN_MAP_H2:
      if (d->m_children < 1 || d->slot < 0 || d->slot >= d->m_children) return GTN_ERR_INVALID;
      *s = h2_spec(d->n_children, d->m_children, d->slot, d->m_is_root != 0);
      return GTN_OK;
    case GTN_MAP_H0: *s = h0_spec(); return GTN_OK;
    case GTN_MAP_ENV:
      if (d->slot >= d->n_children || (d->slot < 0 && d->n_is_root)) return GTN_ERR_INVALID;
      *s = env_spec(d->n_children, d->n_is_root != 0, d->slot);
      return GTN_OK;
    default: return GTN_ERR_INVALID;
  }
}

// Operand dims of a spec from the caller's tensors: every positive label takes its dim from
// the first tensor that carries it; the x operand's (and the cap's) dims follow from there.
// ENV: operand 0 (ket) and the last (bra) are the same tensor A.
int spec_dims(const Spec& s, int kind, const std::vector<const gtn_tensor_s*>& given, std::vector<int64_t>* dims,
              std::string* why) {
  const int nops = (int)s.labels.size();
  std::vector<const gtn_tensor_s*> at(nops, nullptr);
  // the given tensors fill operands 1.. (maps) or every non-cap operand (ENV: ket = bra)
  int gi = 0;
  for (int i = 0; i < nops; ++i) {
    const bool is_cap = s.cap && ((kind == GTN_MAP_ENV && i == nops - 3) || (kind != GTN_MAP_ENV && i == nops - 1));
    if (is_cap) continue;
    if (kind == GTN_MAP_ENV && i == nops - 1) {
      at[i] = at[0];
      continue;
    }
    if (kind != GTN_MAP_ENV && i == 0) continue;  // the map input x
    if (gi >= (int)given.size()) {
      *why = "too few tensors for this kind of map";
      return GTN_ERR_INVALID;
    }
    at[i] = given[gi++];
  }
  if (gi != (int)given.size()) {
    *why = "too many tensors for this kind of map";
    return GTN_ERR_INVALID;
  }
  std::vector<int64_t> labdim(256, -1);
  for (int i = 0; i < nops; ++i) {
    if (!at[i]) continue;
    if (at[i]->rank != (int)s.labels[i].size()) {
      *why = "operand " + std::to_string(i) + " has rank " + std::to_string(at[i]->rank) + ", the map needs " +
             std::to_string(s.labels[i].size());
      return GTN_ERR_SHAPE;
    }
    for (int j = 0; j < at[i]->rank; ++j) {
      const int l = s.labels[i][j];
      if (l <= 0) continue;
      if (labdim[l] >= 0 && labdim[l] != at[i]->dims[j]) {
        *why = "leg dimension mismatch on label " + std::to_string(l);
        return GTN_ERR_SHAPE;
      }
      labdim[l] = at[i]->dims[j];
    }
  }
  dims->clear();
  for (int i = 0; i < nops; ++i) {
    if (at[i]) {
      for (int j = 0; j < at[i]->rank; ++j) dims->push_back(at[i]->dims[j]);
      continue;
    }
    for (int l : s.labels[i]) {
      if (l > 0 && labdim[l] >= 0) dims->push_back(labdim[l]);
      else if (l > 0) dims->push_back(1);  // the root cap's legs and x's unit parent leg
      else {
        // an output leg of x (maps): its dim is the dim of the env/W leg that carries the
        // same output label
        int64_t dd = -1;
        for (int q = 0; q < nops && dd < 0; ++q)
          if (at[q])
            for (int j = 0; j < at[q]->rank; ++j)
              if (s.labels[q][j] == l) dd = at[q]->dims[j];
        dims->push_back(dd < 0 ? 1 : dd);
      }
    }
  }
  return GTN_OK;
}

// Column-major operands (TensorKit/Julia arrays): an array with legs (l1..lN), first leg
// fastest, is the row-major tensor with legs (lN..l1).  Reverse every operand's labels and
// dims, and renumber the output legs -k -> -(R + 1 - k) so that the output comes out
// column-major in the reference's leg order too.
void to_row_major(std::vector<int>& ranks, std::vector<int>& labels, std::vector<int64_t>& dims) {
  int R = 0;
  for (int l : labels) R = std::max(R, -l);
  size_t off = 0;
  for (int r : ranks) {
    std::reverse(labels.begin() + off, labels.begin() + off + r);
    std::reverse(dims.begin() + off, dims.begin() + off + r);
    off += r;
  }
  for (int& l : labels)
    if (l < 0) l = -(R + 1 + l);
}

}  // namespace

extern "C" {

int gtn_tensor_create(gtn_ctx ctx, int rank, const int64_t* dims, gtn_tensor* out) {
  if (!ctx || !out || rank < 0 || rank > 16 || (rank > 0 && !dims)) return set_err(ctx, GTN_ERR_INVALID, "gtn_tensor_create: bad argument");
  *out = nullptr;
  gtn_tensor t = new (std::nothrow) gtn_tensor_s();
  if (!t) return set_err(ctx, GTN_ERR_MEMORY, "host allocation failed");
  t->ctx = ctx;
  t->rank = rank;
  t->elems = 1;
  for (int i = 0; i < rank; ++i) {
    if (dims[i] < 1) {
      delete t;
      return set_err(ctx, GTN_ERR_INVALID, "gtn_tensor_create: leg dims must be >= 1");
    }
    t->dims[i] = dims[i];
    t->elems *= dims[i];
  }
  if (cudaMalloc(&t->data, (size_t)t->elems * sizeof(double2)) != cudaSuccess) {
    delete t;
    return set_err(ctx, GTN_ERR_MEMORY, "gtn_tensor_create: device allocation refused");
  }
  t->owned = true;
  *out = t;
  return GTN_OK;
}

int gtn_tensor_wrap(gtn_ctx ctx, int rank, const int64_t* dims, void* device_data, gtn_tensor* out) {
  if (!ctx || !out || !device_data || rank < 0 || rank > 16 || (rank > 0 && !dims))
    return set_err(ctx, GTN_ERR_INVALID, "gtn_tensor_wrap: bad argument");
  *out = nullptr;
  gtn_tensor t = new (std::nothrow) gtn_tensor_s();
  if (!t) return set_err(ctx, GTN_ERR_MEMORY, "host allocation failed");
  t->ctx = ctx;
  t->rank = rank;
  t->elems = 1;
  for (int i = 0; i < rank; ++i) {
    t->dims[i] = dims[i];
    t->elems *= dims[i];
  }
  t->data = device_data;
  t->owned = false;
  *out = t;
  return GTN_OK;
}

int gtn_tensor_destroy(gtn_tensor t) {
  if (!t) return GTN_ERR_INVALID;
  if (t->owned && t->data) {
    cudaStreamSynchronize(t->ctx->stream);
    cudaFree(t->data);
  }
  delete t;
  return GTN_OK;
}

void* gtn_tensor_data(gtn_tensor t) { return t ? t->data : nullptr; }

int gtn_tensor_shape(gtn_tensor t, int* rank, int64_t* dims) {
  if (!t || !rank) return GTN_ERR_INVALID;
  *rank = t->rank;
  if (dims)
    for (int i = 0; i < t->rank; ++i) dims[i] = t->dims[i];
  return GTN_OK;
}

int gtn_tensor_upload(gtn_tensor t, const void* host, int64_t elems) {
  if (!t || !host || elems != t->elems) return set_err(t ? t->ctx : nullptr, GTN_ERR_INVALID, "gtn_tensor_upload: size");
  GTN_CUDA_TRY(t->ctx, cudaMemcpyAsync(t->data, host, (size_t)elems * sizeof(double2), cudaMemcpyHostToDevice,
                                       t->ctx->stream));
  GTN_CUDA_TRY(t->ctx, cudaStreamSynchronize(t->ctx->stream));
  return GTN_OK;
}

int gtn_tensor_download(gtn_tensor t, void* host, int64_t elems) {
  if (!t || !host || elems != t->elems)
    return set_err(t ? t->ctx : nullptr, GTN_ERR_INVALID, "gtn_tensor_download: size");
  GTN_CUDA_TRY(t->ctx, cudaMemcpyAsync(host, t->data, (size_t)elems * sizeof(double2), cudaMemcpyDeviceToHost,
                                       t->ctx->stream));
  GTN_CUDA_TRY(t->ctx, cudaStreamSynchronize(t->ctx->stream));
  return GTN_OK;
}

int gtn_site_labels(const gtn_site_desc* desc, int cap, int* n_operands, int* ranks, int* labels, int* order) {
  Spec s;
  const int st = build_spec(desc, &s);
  if (st != GTN_OK) return st;
  const int n = (int)s.labels.size();
  if (n_operands) *n_operands = n;
  int tot = 0;
  for (auto& l : s.labels) tot += (int)l.size();
  if (cap < tot || !ranks || !labels || !order) return cap < tot ? GTN_ERR_INVALID : GTN_OK;
  int o = 0;
  for (int i = 0; i < n; ++i) {
    ranks[i] = (int)s.labels[i].size();
    for (int l : s.labels[i]) labels[o++] = l;
    order[i] = s.order[i];
  }
  return GTN_OK;
}

int gtn_map_create_kind(gtn_ctx ctx, const gtn_site_desc* desc, int n_tensors, const gtn_tensor* tensors,
                        int precision, gtn_map* out) {
  if (!ctx || !desc || !out || n_tensors < 0 || (n_tensors > 0 && !tensors))
    return set_err(ctx, GTN_ERR_INVALID, "gtn_map_create_kind: null argument");
  *out = nullptr;
  if (desc->kind == GTN_MAP_ENV) return set_err(ctx, GTN_ERR_INVALID, "environments are built by gtn_env_build");
  Spec s;
  if (build_spec(desc, &s) != GTN_OK) return set_err(ctx, GTN_ERR_INVALID, "gtn_map_create_kind: bad site description");
  std::vector<const gtn_tensor_s*> given(tensors, tensors + n_tensors);
  for (auto* t : given)
    if (!t || t->ctx != ctx) return set_err(ctx, GTN_ERR_INVALID, "gtn_map_create_kind: tensors must belong to ctx");
  std::vector<int64_t> dims;
  std::string why;
  int st = spec_dims(s, desc->kind, given, &dims, &why);
  if (st != GTN_OK) return set_err(ctx, st, "gtn_map_create_kind: " + why);
  const int nops = (int)s.labels.size();
  std::vector<int> ranks, labels, conj(nops, 0);
  for (auto& l : s.labels) {
    ranks.push_back((int)l.size());
    for (int v : l) labels.push_back(v);
  }
  if (desc->col_major) to_row_major(ranks, labels, dims);
  std::vector<const void*> ptrs(nops, nullptr);
  void* capbuf = nullptr;
  for (int i = 1, gi = 0; i < nops; ++i) {
    if (s.cap && i == nops - 1) {
      const double2 one = make_double2(1.0, 0.0);
      GTN_CUDA_TRY(ctx, cudaMalloc(&capbuf, sizeof(double2)));
      GTN_CUDA_TRY(ctx, cudaMemcpy(capbuf, &one, sizeof(double2), cudaMemcpyHostToDevice));
      ptrs[i] = capbuf;
    } else {
      ptrs[i] = given[gi++]->data;
    }
  }
  st = gtn_map_create(ctx, nops, ranks.data(), dims.data(), labels.data(), conj.data(), s.order.data(), ptrs.data(),
                      precision, out);
  if (capbuf) {
    cudaStreamSynchronize(ctx->stream);  // the statics were packed into the map on the stream
    cudaFree(capbuf);
  }
  return st;
}

int gtn_env_build(gtn_ctx ctx, const gtn_site_desc* desc, gtn_tensor A, gtn_tensor W, int n_envs, const gtn_tensor* envs,
                  void* out, int precision) {
  if (!ctx || !desc || !A || !W || !out || n_envs < 0 || (n_envs > 0 && !envs))
    return set_err(ctx, GTN_ERR_INVALID, "gtn_env_build: null argument");
  if (desc->kind != GTN_MAP_ENV) return set_err(ctx, GTN_ERR_INVALID, "gtn_env_build: desc.kind must be GTN_MAP_ENV");
  Spec s;
  if (build_spec(desc, &s) != GTN_OK) return set_err(ctx, GTN_ERR_INVALID, "gtn_env_build: bad site description");
  std::vector<const gtn_tensor_s*> given;
  given.push_back(A);
  for (int i = 0; i < n_envs; ++i) given.push_back(envs[i]);
  given.push_back(W);
  for (auto* t : given)
    if (!t || t->ctx != ctx) return set_err(ctx, GTN_ERR_INVALID, "gtn_env_build: tensors must belong to ctx");
  std::vector<int64_t> dims;
  std::string why;
  int st = spec_dims(s, GTN_MAP_ENV, given, &dims, &why);
  if (st != GTN_OK) return set_err(ctx, st, "gtn_env_build: " + why);
  const int nops = (int)s.labels.size();
  std::vector<int> ranks, labels, conj(nops, 0);
  conj[nops - 1] = 1;
  for (auto& l : s.labels) {
    ranks.push_back((int)l.size());
    for (int v : l) labels.push_back(v);
  }
  if (desc->col_major) to_row_major(ranks, labels, dims);
  std::vector<const void*> ptrs(nops, nullptr);
  void* capbuf = nullptr;
  int gi = 0;
  for (int i = 0; i < nops; ++i) {
    if (s.cap && i == nops - 3) {
      const double2 one = make_double2(1.0, 0.0);
      GTN_CUDA_TRY(ctx, cudaMalloc(&capbuf, sizeof(double2)));
      GTN_CUDA_TRY(ctx, cudaMemcpy(capbuf, &one, sizeof(double2), cudaMemcpyHostToDevice));
      ptrs[i] = capbuf;
    } else if (i == nops - 1) {
      ptrs[i] = A->data;
    } else {
      ptrs[i] = given[gi++]->data;
    }
  }
  st = gtn_contract(ctx, nops, ranks.data(), dims.data(), labels.data(), conj.data(), s.order.data(), ptrs.data(), out,
                    precision);
  if (capbuf) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(capbuf);
  }
  return st;
}

}  // extern "C"
