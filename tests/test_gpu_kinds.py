"""Tensor objects and maps by kind through the C ABI: gtn_tensor create / upload / download /
wrap, and eff_h1, eff_h2, eff_h0 and environment updates built by gtn_map_create_kind /
gtn_env_build from a site description, against the maps and environments the host harness
builds from its own label graphs (same graphs, same order: equal to rounding)."""
import numpy as np
import pytest

import grafttn as G
from grafttn import _lib
from grafttn.contractions import EffectiveMap, EnvCache, eff_h0, eff_h1, eff_h2

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_tensor_create_upload_download(ctx):
    import ctypes as C
    rng = np.random.default_rng(1)
    a = rng.standard_normal((3, 4, 5)) + 1j * rng.standard_normal((3, 4, 5))
    h = C.c_void_p()
    dims = (C.c_int64 * 3)(3, 4, 5)
    assert ctx.lib.gtn_tensor_create(ctx.h, 3, dims, C.byref(h)) == _lib.GTN_OK
    assert ctx.lib.gtn_tensor_upload(h, a.ctypes.data_as(C.c_void_p), a.size) == _lib.GTN_OK
    b = np.empty_like(a)
    assert ctx.lib.gtn_tensor_download(h, b.ctypes.data_as(C.c_void_p), b.size) == _lib.GTN_OK
    assert np.array_equal(a, b)
    rank, od = C.c_int(), (C.c_int64 * 16)()
    assert ctx.lib.gtn_tensor_shape(h, C.byref(rank), od) == _lib.GTN_OK
    assert rank.value == 3 and list(od)[:3] == [3, 4, 5]
    assert ctx.lib.gtn_tensor_upload(h, a.ctypes.data_as(C.c_void_p), a.size - 1) == _lib.GTN_ERR_INVALID
    assert ctx.lib.gtn_tensor_destroy(h) == _lib.GTN_OK


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("fp16x3", 1e-6)])
def test_maps_by_kind_match_host_graphs(ctx, precision, tol):
    topo = G.binary_topology(3)
    H = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    psi = G.random_ttns(np.random.default_rng(5), topo, 2, 8, ctx=ctx)
    rng = np.random.default_rng(6)
    for n in [7, 3, 1, 0]:
        G.move_center(psi, n)
        cache = EnvCache(topo)
        K = topo.nchildren(n)
        root = topo.parent[n] < 0
        # eff_h1
        ref = eff_h1(cache, psi, H, n, precision)
        envs = [cache.env(psi, H, w, n) for w in topo.neighbors(n)]
        km = EffectiveMap.from_kind(ctx, _lib.SiteDesc(_lib.MAP_H1, K, int(root), 0, 0, 0, 0), [H.tensors[n]] + envs,
                                    precision)
        assert km.x_shape == ref.x_shape
        x = ctx.upload(rng.standard_normal(ref.x_shape) + 1j * rng.standard_normal(ref.x_shape))
        assert rel(ctx.download(km(x)), ctx.download(ref(x))) < tol, ("h1", n)
        km.close()
        ref.close()
        if root:
            continue
        m = topo.parent[n]
        Km = topo.nchildren(m)
        # eff_h2
        ref = eff_h2(cache, psi, H, n, m, precision)
        envs = [cache.env(psi, H, w, n) for w in topo.children[n]]
        envs += [cache.env(psi, H, w, m) for w in topo.neighbors(m) if w != n]
        km = EffectiveMap.from_kind(ctx, _lib.SiteDesc(_lib.MAP_H2, K, 0, Km, topo.childslot(m, n),
                                                       int(topo.parent[m] < 0)),
                                    [H.tensors[n], H.tensors[m]] + envs, precision)
        assert km.x_shape == ref.x_shape
        x = ctx.upload(rng.standard_normal(ref.x_shape) + 1j * rng.standard_normal(ref.x_shape))
        assert rel(ctx.download(km(x)), ctx.download(ref(x))) < tol, ("h2", n)
        km.close()
        ref.close()
        # eff_h0
        ref = eff_h0(cache, psi, H, n, m, precision)
        km = EffectiveMap.from_kind(ctx, _lib.SiteDesc(_lib.MAP_H0, 0, 0, 0, 0, 0),
                                    [cache.env(psi, H, n, m), cache.env(psi, H, m, n)], precision)
        x = ctx.upload(rng.standard_normal(ref.x_shape) + 1j * rng.standard_normal(ref.x_shape))
        assert rel(ctx.download(km(x)), ctx.download(ref(x))) < tol, ("h0", n)
        km.close()
        ref.close()


def test_env_build_by_kind_matches_cache(ctx):
    topo = G.binary_topology(3)
    H = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    psi = G.random_ttns(np.random.default_rng(7), topo, 2, 8, ctx=ctx)
    cache = EnvCache(topo)
    for u in range(topo.nnodes):
        K = topo.nchildren(u)
        root = topo.parent[u] < 0
        for v in topo.neighbors(u):
            slot = -1 if topo.parent[u] == v else topo.childslot(u, v)
            others = [cache.env(psi, H, w, u) for w in topo.neighbors(u) if w != v]
            E = ctx.env_build(_lib.SiteDesc(_lib.MAP_ENV, K, int(root), 0, slot, 0), psi.tensors[u].contiguous(),
                              H.tensors[u], others)
            ref = cache.env(psi, H, u, v)
            assert rel(ctx.download(E), ctx.download(ref)) < 1e-13, (u, v)


def test_col_major_tensors_match_row_major(ctx):
    # TensorKit/Julia arrays: column-major buffers with dims in the reference's leg order
    topo = G.binary_topology(3)
    H = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    psi = G.random_ttns(np.random.default_rng(8), topo, 2, 6, ctx=ctx)
    n = 3
    m = topo.parent[n]
    G.move_center(psi, n)
    cache = EnvCache(topo)
    K, Km = topo.nchildren(n), topo.nchildren(m)
    envs = [cache.env(psi, H, w, n) for w in topo.children[n]]
    envs += [cache.env(psi, H, w, m) for w in topo.neighbors(m) if w != n]
    statics = [H.tensors[n], H.tensors[m]] + envs
    desc = _lib.SiteDesc(_lib.MAP_H2, K, 0, Km, topo.childslot(m, n), int(topo.parent[m] < 0), 0)
    row = EffectiveMap.from_kind(ctx, desc, statics, "fp64")
    rng = np.random.default_rng(9)
    x = rng.standard_normal(row.x_shape) + 1j * rng.standard_normal(row.x_shape)
    y_row = ctx.download(row(ctx.upload(x)))

    def colmajor(a):  # the same array stored first-leg-fastest: a row-major buffer of a.T
        return np.ascontiguousarray(np.transpose(a))
    cm_statics = [ctx.upload(colmajor(ctx.download(s))) for s in statics]
    import ctypes as C
    from grafttn.device import TensorHandle
    hs = []
    for s_dev, s_orig in zip(cm_statics, statics):
        h = C.c_void_p()
        dims = (C.c_int64 * s_orig.dim())(*[int(v) for v in s_orig.shape])
        assert ctx.lib.gtn_tensor_wrap(ctx.h, s_orig.dim(), dims, C.c_void_p(s_dev.data_ptr()), C.byref(h)) == 0
        hs.append(h)
    desc.col_major = 1
    arr = (C.c_void_p * len(hs))(*[h.value for h in hs])
    mh = C.c_void_p()
    assert ctx.lib.gtn_map_create_kind(ctx.h, C.byref(desc), len(hs), arr, 0, C.byref(mh)) == 0
    xc = ctx.upload(colmajor(x))
    yc = ctx.empty(tuple(reversed(row.y_shape)))
    assert ctx.lib.gtn_map_apply(mh, C.c_void_p(xc.data_ptr()), C.c_void_p(yc.data_ptr())) == 0
    y_col = np.transpose(ctx.download(yc))
    assert rel(y_col, y_row) < 1e-13
    ctx.lib.gtn_map_destroy(mh)
    for h in hs:
        ctx.lib.gtn_tensor_destroy(h)
    row.close()
    del TensorHandle
