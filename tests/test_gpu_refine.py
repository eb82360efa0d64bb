"""FP64 iterative refinement of mixed-precision eigenvectors (gtn_lanczos_refine): the local
two-site problem of a 16-site Heisenberg chain at bond 64, solved by mixed Lanczos and then
refined, against the FP64 Lanczos eigenpair of the same map; and the refined energy of a
mixed two-site DMRG step at the middle of mps63 at D = 256 against FP64."""
import numpy as np
import pytest

import grafttn as G
from grafttn.contractions import EnvCache, eff_h2
from grafttn.networks import move_center, two_site_tensor

pytestmark = pytest.mark.gpu


def local_problem(ctx, L, D, seed):
    topo = G.mps_topology(L)
    W = G.TTNO.from_hamiltonian(G.heisenberg(topo), ctx)
    bond = {}
    for c in range(topo.nnodes):
        if topo.parent[c] >= 0:
            below = len(topo.subtree_nodes(c, topo.parent[c]))
            bond[c] = int(min(D, 2 ** min(below, 40), 2 ** min(L - below, 40)))
    psi = G.random_ttns(np.random.default_rng(seed), topo, 2, bond, ctx=ctx)
    n = topo.index[f"site{L // 2}"]
    m = topo.parent[n]
    cache = EnvCache(topo)
    move_center(psi, n, cache)
    return psi, W, cache, n, m


@pytest.mark.parametrize("precision", ["fp16x3", "bf16x6"])
def test_refined_eigenpair_matches_fp64(ctx, precision):
    psi, W, cache, n, m = local_problem(ctx, 16, 64, 21)
    theta = two_site_tensor(psi, n, m)
    h64 = eff_h2(cache, psi, W, n, m, "fp64")
    E64, v64, info64 = h64.lanczos_min(theta, krylovdim=20, tol=1e-12, maxiter=200)
    assert info64["converged"]
    hm = eff_h2(cache, psi, W, n, m, precision)
    Em, vm, _ = hm.lanczos_min(theta, krylovdim=20, tol=1e-12, maxiter=200, rq_fp64=True)
    tol = 1e-9 * abs(E64)
    Er, vr, info = hm.refine(vm, tol=tol, max_outer=10)
    assert info["converged"] and info["resid"] <= tol, info
    assert info["fp64_matvecs"] == info["corrections"] + 1
    assert abs(Er - E64) <= 1e-12 * abs(E64), (Er, E64, Em)
    # the same eigenvector up to a phase
    ov = abs(ctx.dot(v64, vr))
    assert abs(1 - ov) < 1e-12, ov
    # refinement helps: the mixed Lanczos vector alone has a larger FP64 residual
    _, _, info0 = hm.refine(vm, tol=0.0, max_outer=0)
    assert info0["resid"] > 10 * info["resid"]
    h64.close()
    hm.close()


def test_refine_is_idempotent_on_a_converged_vector(ctx):
    psi, W, cache, n, m = local_problem(ctx, 12, 32, 22)
    theta = two_site_tensor(psi, n, m)
    hm = eff_h2(cache, psi, W, n, m, "fp16x3")
    E64, v64, _ = hm.lanczos_min(theta, krylovdim=20, tol=1e-12, maxiter=200)
    E1, v1, i1 = hm.refine(v64, tol=1e-9 * abs(E64), max_outer=10)
    E2, v2, i2 = hm.refine(v1, tol=1e-9 * abs(E64), max_outer=10)
    assert i2["corrections"] == 0 and i2["fp64_matvecs"] == 1
    assert abs(E2 - E1) <= 1e-13 * abs(E1)
    hm.close()


def test_dmrg_step_mps63_d256_refined_vs_fp64(ctx):
    # one two-site step in the middle of mps63 at D = 256 from a random state: the refined
    # mixed energy against the FP64 Lanczos energy of the same local problem
    psi, W, cache, n, m = local_problem(ctx, 63, 256, 7)
    theta = two_site_tensor(psi, n, m)
    h64 = eff_h2(cache, psi, W, n, m, "fp64")
    E64, _, _ = h64.lanczos_min(theta, krylovdim=20, tol=1e-10, maxiter=200)
    hm = eff_h2(cache, psi, W, n, m, "fp16x3")
    Em, vm, _ = hm.lanczos_min(theta, krylovdim=20, tol=1e-10, maxiter=200)
    from grafttn.solvers import refine_local
    Er, _ = refine_local(hm, Em, vm, 1e-8)
    assert abs(Er - E64) / abs(E64) <= 1e-10, (Er, E64, Em)
    h64.close()
    hm.close()


def test_refinement_with_fp64e_twin_matches_fp64(ctx):
    # the residuals of the refinement through the FP64-grade tensor-core map (gtn_map_set_fp64)
    psi, W, cache, n, m = local_problem(ctx, 63, 256, 7)
    theta = two_site_tensor(psi, n, m)
    h64 = eff_h2(cache, psi, W, n, m, "fp64")
    E64, v64, _ = h64.lanczos_min(theta, krylovdim=20, tol=1e-10, maxiter=200)
    hm = eff_h2(cache, psi, W, n, m, "fp16x3")
    he = eff_h2(cache, psi, W, n, m, "fp64e")
    hm.set_fp64_map(he)
    Em, vm, _ = hm.lanczos_min(theta, krylovdim=20, tol=1e-10, maxiter=200)
    Er, vr, info = hm.refine(vm, tol=1e-8 * abs(Em), max_outer=8)
    assert info["converged"]
    assert abs(Er - E64) / abs(E64) <= 1e-10, (Er, E64)
    # the FP64E map agrees with the FP64 map on the refined vector
    y64, ye = ctx.download(h64(vr)), ctx.download(he(vr))
    assert np.linalg.norm(ye - y64) <= 1e-12 * np.linalg.norm(y64)
    hm.close()
    he.close()
    h64.close()
