"""Environment cache and effective-Hamiltonian maps on the device.

Mirrors lib/GraftContractions/src/Contractions/envcache.jl (EnvCache, env!, build_env,
invalidation) and effective.jl (eff_h1 / eff_h2 / eff_h0): the label graphs are the
reference's, operand by operand and leg by leg, and the contraction order is its env-first
``preferred_slots`` order.  A map compiles once into a libgrafttn plan (statics packed on
the device) and is then applied many times by the Krylov solvers.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import check, i64_array, int_array, ptr_array
from .device import Context
from .networks import TTNO, TTNS


def _stateleg(t, u, w):
    """(envcache.jl:852-853)"""
    return t.nchildren(u) + 1 if t.parent[u] == w else t.childslot(u, w)


def _opleg(t, u, w):
    """(envcache.jl:856-857)"""
    return t.nchildren(u) + 2 if t.parent[u] == w else t.childslot(u, w)


class _Fresh:
    def __init__(self):
        self.n = 0

    def __call__(self):
        self.n += 1
        return self.n


def env_spec(t, u, v, a_rank, w_rank):
    """Sandwich at u with the legs towards v open (envcache.jl:919-999).  Operands:
    (ket, env(w->u) for neighbours w != v..., root cap?, W, conj(bra)).  Output (ket, op, bra)."""
    K = t.nchildren(u)
    fresh = _Fresh()
    aidx, bidx, widx = [0] * a_rank, [0] * a_rank, [0] * w_rank
    pin, pout = fresh(), fresh()
    aidx[K] = pin
    widx[K + 1] = pin
    widx[K] = pout
    bidx[K] = pout
    envs, envlabels = [], []
    for w in t.neighbors(u):
        la = _stateleg(t, u, w)
        if w == v:
            aidx[la], widx[_opleg(t, u, w)], bidx[la] = -1, -2, -3
        else:
            e = [fresh(), fresh(), fresh()]
            aidx[la], widx[_opleg(t, u, w)], bidx[la] = e
            envs.append(w)
            envlabels.append(e)
    cap = None
    if t.parent[u] < 0:
        ka, ko, kb = fresh(), fresh(), fresh()
        aidx[-1], widx[-1], bidx[-1] = ka, ko, kb
        cap = [kb, ko, ka]
    labels = [aidx] + envlabels + ([cap] if cap else []) + [widx, bidx]
    conj = [False] * (len(labels) - 1) + [True]
    return labels, conj, envs, cap is not None


def h1_spec(t, n, x_rank, w_rank):
    """(effective.jl:627-686) operands (x, W, env(w->n) for neighbours..., cap?), env-first order."""
    K = t.nchildren(n)
    fresh = _Fresh()
    xidx, widx = [0] * x_rank, [0] * w_rank
    labels = [xidx, widx]
    pin = fresh()
    xidx[K] = pin
    widx[K + 1] = pin
    widx[K] = -(K + 1)
    children, parents, caps, envs = [], [], [], []
    for w in t.neighbors(n):
        lx = _stateleg(t, n, w)
        kk, oo = fresh(), fresh()
        xidx[lx] = kk
        widx[_opleg(t, n, w)] = oo
        labels.append([kk, oo, -(lx + 1)])
        envs.append((w, n))
        (parents if t.parent[n] == w else children).append(len(labels) - 1)
    if t.parent[n] < 0:
        ka, ko = fresh(), fresh()
        xidx[-1] = ka
        widx[-1] = ko
        labels.append([ka, ko, -x_rank])
        caps.append(len(labels) - 1)
    return labels, [0] + children + [1] + parents + caps, envs


def h2_spec(t, n, m, x_rank, wn_rank, wm_rank, pn):
    """(effective.jl:878-976) operands (Θ, Wn, Wm, env(w->n)..., env(w->m)..., cap?)."""
    k = t.childslot(m, n)
    Kn, Km = t.nchildren(n), t.nchildren(m)
    fresh = _Fresh()
    xidx, wnidx, wmidx = [0] * x_rank, [0] * wn_rank, [0] * wm_rank
    labels = [xidx, wnidx, wmidx]

    def mpos(j):
        return pn + (j if j < k else j - 1)
    ob = fresh()
    wnidx[-1] = ob
    wmidx[k] = ob
    pin = fresh()
    xidx[Kn] = pin
    wnidx[Kn + 1] = pin
    wnidx[Kn] = -(Kn + 1)
    pin = fresh()
    xidx[mpos(Km)] = pin
    wmidx[Km + 1] = pin
    wmidx[Km] = -(mpos(Km) + 1)
    envn, envmc, envmp, caps, envs = [], [], [], [], []
    for w in t.neighbors(n):
        if w == m:
            continue
        lx = t.childslot(n, w)
        kk, oo = fresh(), fresh()
        xidx[lx] = kk
        wnidx[lx] = oo
        labels.append([kk, oo, -(lx + 1)])
        envs.append((w, n))
        envn.append(len(labels) - 1)
    for w in t.neighbors(m):
        if w == n:
            continue
        if t.parent[m] == w:
            lw, lx = wm_rank - 1, x_rank - 1
        else:
            lw = t.childslot(m, w)
            lx = mpos(lw)
        kk, oo = fresh(), fresh()
        xidx[lx] = kk
        wmidx[lw] = oo
        labels.append([kk, oo, -(lx + 1)])
        envs.append((w, m))
        (envmp if t.parent[m] == w else envmc).append(len(labels) - 1)
    if t.parent[m] < 0:
        ka, ko = fresh(), fresh()
        xidx[-1] = ka
        wmidx[-1] = ko
        labels.append([ka, ko, -x_rank])
        caps.append(len(labels) - 1)
    order = [0] + envn + [1] + envmc + [2] + envmp + caps
    return labels, order, envs


def chain_cost(shapes, labels, order):
    """(complex MACs, largest intermediate in elements) of the pairwise chain that starts
    at operand order[0] and absorbs the others in order."""
    dims = {}
    for shp, lab in zip(shapes, labels):
        for l, d in zip(lab, shp):
            dims[l] = int(d)
    cur = list(labels[order[0]])
    macs, peak = 0, math.prod(dims[l] for l in cur)
    for j in order[1:]:
        L = labels[j]
        sh = [l for l in cur if l > 0 and l in L]
        M = math.prod(dims[l] for l in cur if l not in sh)
        K = math.prod(dims[l] for l in sh)
        N = math.prod(dims[l] for l in L if l not in sh)
        macs += M * K * N
        peak = max(peak, M * N)
        cur = [l for l in L if l not in sh] + [l for l in cur if l not in sh]
    return macs, peak


def best_order(shapes, labels, first=0, out_weight=8):
    """Cheapest left-deep chain from operand ``first``: dynamic programming over the set
    of absorbed operands (the running tensor's legs depend only on that set), minimising
    sum over steps of M*K*N + out_weight * M*N (MACs plus the written intermediate)."""
    dims = {}
    for shp, lab in zip(shapes, labels):
        for l, d in zip(lab, shp):
            dims[l] = int(d)
    others = [j for j in range(len(labels)) if j != first]
    n = len(others)

    def legs(mask):
        cnt = {}
        for l in labels[first]:
            cnt[l] = cnt.get(l, 0) + 1
        for b in range(n):
            if mask >> b & 1:
                for l in labels[others[b]]:
                    cnt[l] = cnt.get(l, 0) + 1
        return [l for l, c in cnt.items() if not (l > 0 and c == 2)]
    best = {0: (0.0, [])}
    for mask in sorted(range(1 << n), key=lambda m: bin(m).count("1")):
        if mask not in best:
            continue
        cost, seq = best[mask]
        cur = legs(mask)
        for b in range(n):
            if mask >> b & 1:
                continue
            L = labels[others[b]]
            sh = [l for l in cur if l > 0 and l in L]
            M = math.prod(dims[l] for l in cur if l not in sh)
            K = math.prod(dims[l] for l in sh)
            N = math.prod(dims[l] for l in L if l not in sh)
            c = cost + M * K * N + out_weight * M * N
            nm = mask | (1 << b)
            if nm not in best or c < best[nm][0]:
                best[nm] = (c, seq + [others[b]])
    return [first] + best[(1 << n) - 1][1]


def _objective(shapes, labels, order, out_weight=8):
    macs = 0
    dims = {}
    for shp, lab in zip(shapes, labels):
        for l, d in zip(lab, shp):
            dims[l] = int(d)
    cur = list(labels[order[0]])
    for j in order[1:]:
        L = labels[j]
        sh = [l for l in cur if l > 0 and l in L]
        M = math.prod(dims[l] for l in cur if l not in sh)
        K = math.prod(dims[l] for l in sh)
        N = math.prod(dims[l] for l in L if l not in sh)
        macs += M * K * N + out_weight * M * N
        cur = [l for l in L if l not in sh] + [l for l in cur if l not in sh]
    return macs


_ORDER_MEMO = {}


def choose_order(shapes, labels, order):
    """The given (env-first) order unless the cheapest chain is clearly cheaper (by 1.5x in
    MACs plus written intermediates).  This matters at high-degree nodes, where absorbing
    every environment before the TTNO tensor multiplies the running tensor by w per leg;
    on binary trees and chains the env-first chain is kept.  The answer depends only on the
    shapes, labels and order, so it is remembered (sweeps ask again at every node visit)."""
    if len(labels) > 13:
        return list(order)
    key = (tuple(tuple(int(d) for d in s) for s in shapes), tuple(tuple(l) for l in labels), tuple(order))
    got = _ORDER_MEMO.get(key)
    if got is None:
        b = best_order(shapes, labels, order[0])
        got = b if 3 * _objective(shapes, labels, b) < 2 * _objective(shapes, labels, order) else list(order)
        if len(_ORDER_MEMO) > 100000:
            _ORDER_MEMO.clear()
        _ORDER_MEMO[key] = got
    return list(got)


class EffectiveMap:
    """Callable y = H_eff x backed by a compiled libgrafttn plan (types.jl:410-445)."""

    @classmethod
    def from_kind(cls, ctx: Context, desc, statics, precision=_lib.PREC_FP64):
        """The map of a site description (gtn_map_create_kind: the library writes the label
        graph); statics as gtn_map_create_kind lists them, as device tensors."""
        from .device import TensorHandle
        prec = _lib.PRECISIONS.get(precision, precision) if isinstance(precision, str) else precision
        hs = [TensorHandle(ctx, s) for s in statics]
        arr = (C.c_void_p * max(1, len(hs)))(*[h.h for h in hs])
        h = C.c_void_p()
        check(ctx.lib.gtn_map_create_kind(ctx.h, C.byref(desc), len(hs), arr, prec, C.byref(h)), ctx.h,
              "map_create_kind")
        self = cls.__new__(cls)
        self.ctx, self.h, self.precision = ctx, h, prec
        self._statics, self.labels, self.order = list(statics), None, None
        rank = C.c_int()
        odims = (C.c_int64 * 32)()
        check(ctx.lib.gtn_map_out_shape(self.h, C.byref(rank), odims), ctx.h, "map_out_shape")
        self.y_shape = tuple(odims[i] for i in range(rank.value))
        self.x_shape = self.y_shape
        xe, ye, fl, ns, by = C.c_int64(), C.c_int64(), C.c_double(), C.c_int(), C.c_int64()
        check(ctx.lib.gtn_map_info(self.h, C.byref(xe), C.byref(ye), C.byref(fl), C.byref(ns), C.byref(by)),
              ctx.h, "map_info")
        self.flops, self.n_steps, self.bytes = fl.value, ns.value, by.value
        return self

    def __init__(self, ctx: Context, x_shape, labels, order, statics, precision=_lib.PREC_FP64):
        self.ctx = ctx
        self.x_shape = tuple(int(s) for s in x_shape)
        self.precision = _lib.PRECISIONS.get(precision, precision) if isinstance(precision, str) else precision
        ranks = [len(self.x_shape)] + [s.dim() for s in statics]
        dims = list(self.x_shape) + [int(d) for s in statics for d in s.shape]
        labs = [int(l) for lab in labels for l in lab]
        h = C.c_void_p()
        self._statics = statics  # keep alive until the packing kernels ran (and for vjp)
        self.labels = [list(l) for l in labels]
        self.order = list(order)
        st = ctx.lib.gtn_map_create(ctx.h, len(ranks), int_array(ranks), i64_array(dims), int_array(labs),
                                    int_array([0] * len(ranks)), int_array(order),
                                    ptr_array([0] + [s.data_ptr() for s in statics]), self.precision,
                                    C.byref(h))
        check(st, ctx.h, "map_create")
        self.h = h
        rank = C.c_int()
        odims = (C.c_int64 * 32)()
        check(ctx.lib.gtn_map_out_shape(self.h, C.byref(rank), odims), ctx.h, "map_out_shape")
        self.y_shape = tuple(odims[i] for i in range(rank.value))
        xe, ye, fl, ns, by = C.c_int64(), C.c_int64(), C.c_double(), C.c_int(), C.c_int64()
        check(ctx.lib.gtn_map_info(self.h, C.byref(xe), C.byref(ye), C.byref(fl), C.byref(ns), C.byref(by)),
              ctx.h, "map_info")
        self.flops = fl.value
        self.n_steps = ns.value
        self.bytes = by.value

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gtn_map_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def apply_into(self, x, y, precision=None):
        prec = self.precision if precision is None else precision
        check(self.ctx.lib.gtn_map_apply_prec(self.h, prec, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr())),
              self.ctx.h, "map_apply")
        return y

    def __call__(self, x, precision=None):
        """Fresh output, as the reference's executor allocates the root output (executor.jl:122-127)."""
        if tuple(x.shape) != self.x_shape:
            raise _lib.SpaceMismatch(f"map input shape {tuple(x.shape)} != {self.x_shape}")
        return self.apply_into(x.contiguous(), self.ctx.empty(self.y_shape), precision)

    def apply_profiled(self, x, y, precision=None, cap=256):
        """One application with CUDA events around each launch: list of (kernel, ms, flops)."""
        prec = self.precision if precision is None else precision
        ms = (C.c_double * cap)()
        kind = (C.c_int * cap)()
        fl = (C.c_double * cap)()
        cnt = C.c_int()
        check(self.ctx.lib.gtn_map_apply_profiled(self.h, prec, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                                                  cap, ms, kind, fl, C.byref(cnt)), self.ctx.h, "map_apply_profiled")
        return [(_lib.KERNEL_NAMES.get(kind[i], str(kind[i])), ms[i], fl[i]) for i in range(min(cnt.value, cap))]

    def apply_host(self, x_host):
        """Host buffers in and out (host->device copy, apply, device->host copy in one call)."""
        xh = np.ascontiguousarray(x_host, dtype=np.complex128)
        yh = np.empty(self.y_shape, dtype=np.complex128)
        check(self.ctx.lib.gtn_map_apply_host(self.h, xh.ctypes.data_as(C.c_void_p), yh.ctypes.data_as(C.c_void_p)),
              self.ctx.h, "map_apply_host")
        return yh

    def lanczos_min(self, x0, krylovdim=20, tol=1e-12, maxiter=100, rq_fp64=False):
        """Lowest eigenpair (groundstate_eigsolve_backend, GroundState.jl:25-39); x0 untouched."""
        x = self.ctx.copy(x0)
        E = C.c_double()
        info = (C.c_int * 3)()
        res = C.c_double()
        st = self.ctx.lib.gtn_lanczos_min(self.h, C.c_void_p(x.data_ptr()), krylovdim, tol, maxiter,
                                          1 if rq_fp64 else 0, C.byref(E), info, C.byref(res))
        if st not in (_lib.GTN_OK, _lib.GTN_ERR_NOT_CONVERGED):
            check(st, self.ctx.h, "lanczos")
        return E.value, x, dict(restarts=info[0], matvecs=info[1], converged=bool(info[2]), resid=res.value)

    def set_fp64_map(self, other):
        """Serve this map's FP64 applications (Rayleigh quotients, refinement residuals) with
        `other`, an FP64 or "fp64e" map of the same shape (gtn_map_set_fp64); None resets."""
        check(self.ctx.lib.gtn_map_set_fp64(self.h, other.h if other is not None else None), self.ctx.h,
              "map_set_fp64")
        self._fp64_map = other

    def vjp(self, x, ybar, slot):
        """Adjoint of operand `slot` (0 = x, 1.. = statics) of y = H_eff x at this x: the
        tensor G with <G, d op_slot> = <ybar, dy> (gtn_contract_vjp), in FP64."""
        return self.ctx.contract_vjp([x.contiguous()] + list(self._statics), self.labels, ybar.contiguous(), slot)

    def refine(self, x0, tol=1e-8, max_outer=6, inner_dim=20):
        """FP64 iterative refinement of an approximate lowest eigenvector (gtn_lanczos_refine):
        FP64 residuals, corrections from mixed-precision Lanczos bases.  Returns (E, x, info)
        with E the FP64 Rayleigh quotient of the returned x; x0 untouched."""
        x = self.ctx.copy(x0)
        E = C.c_double()
        info = (C.c_int * 4)()
        res = C.c_double()
        st = self.ctx.lib.gtn_lanczos_refine(self.h, C.c_void_p(x.data_ptr()), inner_dim, tol, max_outer,
                                             C.byref(E), info, C.byref(res))
        if st not in (_lib.GTN_OK, _lib.GTN_ERR_NOT_CONVERGED):
            check(st, self.ctx.h, "lanczos_refine")
        return E.value, x, dict(corrections=info[0], mixed_matvecs=info[1], fp64_matvecs=info[2],
                                converged=bool(info[3]), resid=res.value)

    def exponentiate(self, dz, x0, krylovdim=30, tol=1e-12, hermitian=True):
        """exp(dz H) x0 (evolution_exponentiate_backend, Evolution.jl:54-68): Lanczos for a
        Hermitian map, Arnoldi otherwise (KrylovKit's exponentiate with ishermitian, as the
        TDVP sweeps pass it from the TTNO, tdvp.jl:204-281)."""
        x = self.ctx.copy(x0)
        info = (C.c_int * 2)()
        dz = complex(dz)
        fn = self.ctx.lib.gtn_expm_apply if hermitian else self.ctx.lib.gtn_expm_apply_arnoldi
        check(fn(self.h, dz.real, dz.imag, C.c_void_p(x.data_ptr()), krylovdim, tol, info), self.ctx.h, "expm")
        return x, dict(substeps=info[0], matvecs=info[1])


def apply_batched(maps, xs, ys=None, precision=None):
    """y_i = H_i x_i for independent maps in grouped launches (one per step and kernel kind)."""
    ctx = maps[0].ctx
    prec = maps[0].precision if precision is None else precision
    ys = ys if ys is not None else [ctx.empty(m.y_shape) for m in maps]
    n = len(maps)
    check(ctx.lib.gtn_map_apply_batched(n, ptr_array([m.h.value for m in maps]), ptr_array([x.data_ptr() for x in xs]),
                                        ptr_array([y.data_ptr() for y in ys]), prec), ctx.h, "map_apply_batched")
    return ys


class MapBatch:
    """A fixed batch of maps and buffers, optionally replayed as one CUDA graph."""

    def __init__(self, maps, xs, ys, precision=None, graph=True):
        self.ctx = maps[0].ctx
        self.maps, self.xs, self.ys = list(maps), list(xs), list(ys)
        prec = maps[0].precision if precision is None else precision
        h = C.c_void_p()
        n = len(maps)
        check(self.ctx.lib.gtn_batch_create(n, ptr_array([m.h.value for m in maps]), ptr_array([x.data_ptr() for x in xs]),
                                            ptr_array([y.data_ptr() for y in ys]), prec, 1 if graph else 0, C.byref(h)),
              self.ctx.h, "batch_create")
        self.h = h

    def run(self):
        check(self.ctx.lib.gtn_batch_run(self.h), self.ctx.h, "batch_run")
        return self.ys

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gtn_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class EnvCache:
    """Directed-edge environments on the device (envcache.jl:61-109) with the reference's
    invalidation rule: an env is dropped when its contracted side contains a touched node
    (envcache.jl:812-844).  ``max_env_bytes`` bounds the cached bytes with least-recently-
    used eviction (envcache.jl:571-594); evicted environments are recomputed on demand."""

    def __init__(self, topo, max_env_bytes=None, precision="fp64"):
        """``precision`` of the environment contractions: "fp64" (FP64 SIMT kernels) or
        "fp64e" (the FP64-grade digit products on the tensor cores, about 1e-14)."""
        from collections import OrderedDict
        self.topo = topo
        self.precision = _lib.PRECISIONS[precision] if isinstance(precision, str) else precision
        self.envs = OrderedDict()
        self.max_env_bytes = max_env_bytes
        self.bytes = 0
        self.builds = 0
        self.evictions = 0

    def copy(self):
        """A cache holding the same environments (the device tensors are shared: an
        environment is never modified in place, only dropped and rebuilt)."""
        c = EnvCache(self.topo, self.max_env_bytes, self.precision)
        c.envs.update(self.envs)
        c.bytes = self.bytes
        return c

    def _drop(self, key):
        E = self.envs.pop(key)
        self.bytes -= E.numel() * E.element_size()

    def invalidate_node(self, n):
        t = self.topo
        for key in [k for k in self.envs if t.in_subtree(n, k[0], k[1])]:
            self._drop(key)

    def invalidate_edge(self, n, m):
        self.invalidate_node(n)
        self.invalidate_node(m)

    def env(self, psi: TTNS, H: TTNO, u, v):
        """E(u->v)[ket, op, bra], built lazily after its prerequisites (envcache.jl:1440-1476)."""
        key = (u, v)
        if key in self.envs:
            self.envs.move_to_end(key)
            return self.envs[key]
        t = self.topo
        # prerequisites stay referenced here even if the byte budget evicts them meanwhile
        pre = {w: self.env(psi, H, w, u) for w in t.neighbors(u) if w != v}
        A, W = psi.tensors[u], H.tensors[u]
        labels, conj, envs, has_cap = env_spec(t, u, v, A.dim(), W.dim())
        ops = [A] + [pre[w] for w in envs]
        if has_cap:
            ops.append(psi.ctx.upload(np.ones((1, 1, 1))))
        ops += [W, A]
        order = choose_order([tuple(o.shape) for o in ops], labels, list(range(len(ops))))
        E = psi.ctx.contract(ops, labels, conj, order, self.precision)
        self.envs[key] = E
        self.bytes += E.numel() * E.element_size()
        self.builds += 1
        if self.max_env_bytes is not None:
            while self.bytes > self.max_env_bytes and len(self.envs) > 1:
                old = next(iter(self.envs))
                self._drop(old)
                self.evictions += 1
        return E


def _cap(ctx):
    return ctx.upload(np.ones((1, 1, 1)))


def eff_h1(cache: EnvCache, psi: TTNS, H: TTNO, n, precision=_lib.PREC_FP64):
    """(effective.jl:709-730)"""
    t = psi.topo
    x = psi.tensors[n]
    labels, order, envs = h1_spec(t, n, x.dim(), H.tensors[n].dim())
    statics = [H.tensors[n]] + [cache.env(psi, H, w, u) for (w, u) in envs]
    if t.parent[n] < 0:
        statics.append(_cap(psi.ctx))
    order = choose_order([tuple(x.shape)] + [tuple(s.shape) for s in statics], labels, order)
    return EffectiveMap(psi.ctx, x.shape, labels, order, statics, precision)


def two_site_shape(psi: TTNS, n, m):
    k = psi.topo.childslot(m, n)
    return tuple(psi.tensors[n].shape[:-1]) + tuple(s for j, s in enumerate(psi.tensors[m].shape) if j != k)


def eff_h2(cache: EnvCache, psi: TTNS, H: TTNO, n, m, precision=_lib.PREC_FP64):
    """(effective.jl:986-1034)"""
    t = psi.topo
    if t.parent[n] != m:
        raise ValueError("eff_h2: m must be the parent of n")
    pn = psi.tensors[n].dim() - 1
    xs = two_site_shape(psi, n, m)
    labels, order, envs = h2_spec(t, n, m, len(xs), H.tensors[n].dim(), H.tensors[m].dim(), pn)
    statics = [H.tensors[n], H.tensors[m]] + [cache.env(psi, H, w, u) for (w, u) in envs]
    if t.parent[m] < 0:
        statics.append(_cap(psi.ctx))
    order = choose_order([tuple(xs)] + [tuple(s.shape) for s in statics], labels, order)
    return EffectiveMap(psi.ctx, xs, labels, order, statics, precision)


def eff_h0(cache: EnvCache, psi: TTNS, H: TTNO, n, m, precision=_lib.PREC_FP64):
    """Link map y = E(n->m) C E(m->n) (effective.jl:739-797)."""
    if psi.topo.parent[n] != m:
        raise ValueError("eff_h0: m must be the parent of n")
    En = cache.env(psi, H, n, m)
    Em = cache.env(psi, H, m, n)
    labels = [[1, 2], [1, 3, -1], [2, 3, -2]]
    return EffectiveMap(psi.ctx, (En.shape[0], Em.shape[0]), labels, [0, 1, 2], [En, Em], precision)


def expect(psi: TTNS, H: TTNO):
    """<psi|H|psi> / <psi|psi> closed at the centre (expectation.jl:32-40)."""
    cache = EnvCache(psi.topo)
    c = psi.center
    x = psi.tensors[c]
    h1 = eff_h1(cache, psi, H, c)
    y = h1(x)
    return psi.ctx.dot(x, y) / psi.ctx.dot(x, x)
